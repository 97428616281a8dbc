import pathlib
import sys

import numpy as np
import pytest

REPO = pathlib.Path(__file__).resolve().parents[1]
PKG = REPO / "tensor-viterbi_gb300"
GOLDEN = REPO / "tests" / "golden"
for p in (str(REPO), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built decoder library")


def golden_names():
    return sorted(p.stem for p in GOLDEN.glob("*.npz"))


def load_golden(name):
    z = np.load(GOLDEN / f"{name}.npz")
    args = (int(z["n_states"]), z["trans_mat"], z["emission_probs"], z["duration_probs_linear"],
            z["start_probs"], z["duration_probs"], z["obs_seq"])
    return args, {k: z[k] for k in z.files}


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:  # pragma: no cover
        return False


@pytest.fixture(scope="session")
def tvlib():
    """The built decoder library (compiled on demand; no CPU fallback)."""
    sys.path.insert(0, str(PKG))
    import build as tvbuild  # tensor-viterbi_gb300/build.py
    tvbuild.build()
    from tensor_viterbi.viterbi import native
    native.configure("gb300", "cuda")
    return native


# Oracle results at the benchmarked shapes, on T-prefixes long enough to reach
# the fully rolled window (t > 2D): computed once per session and shared by the
# parity tests of this decoder and of the reference's CUDA kernels.
def _headline_prefix(prob):
    Tp = 2 * prob.D + 2000
    return prob.model_args() + (np.ascontiguousarray(prob.obs_seq[:Tp]),)


@pytest.fixture(scope="session")
def c1_case():
    """N=75, D=5000, M=32: the single-sequence bench model (seed 1) and its
    observations, T-prefix 2D + 2000 = 12000, with the oracle's result."""
    import tensor_viterbi.synthetic as syn
    from oracle import oracle as orc
    args = _headline_prefix(syn.config1())
    return args, orc.decode(*args, variant="omp")


@pytest.fixture(scope="session")
def c4_case():
    """N=100, D=1e4, M=64: the stress-shape bench model (seed 4), T-prefix
    2D + 2000 = 22000, with the oracle's result."""
    import tensor_viterbi.synthetic as syn
    from oracle import oracle as orc
    args = _headline_prefix(syn.config4(T=1_000_000))
    return args, orc.decode(*args, variant="omp")
