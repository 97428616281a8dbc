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
