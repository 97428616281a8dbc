"""Generate the golden decode fixtures under tests/golden/ by running the
reference project's own code (development host only: it needs the read-only
reference checkout and oracle/build_ref.sh's compiled `_native`).

Each fixture `<name>.npz` holds the exact float64 decoder inputs in the
reference binding's layouts (src/bindings.cpp:19-32) and the paths the
reference returned:
  path_cpp       _native.decode_tensor_viterbi_cpp, IEEE build (the pin)
  path_omp       _native.decode_tensor_viterbi_omp, IEEE build
  path_cpp_fast  _native.decode_tensor_viterbi_cpp, the reference's own
                 -O3 -march=native -ffast-math build
  path_py        decode_log_tensor_viterbi_cached (tensor_viterbi/viterbi/
                 tensor.py:89-166), when small enough to run
Sources: a few of the reference's data/*.json fixtures (loaded with its
HSMM.load_model + to_log_space, tensor_viterbi/hsmm.py:76-132), seeded
synthetic models of the benchmark family, and constructed exact-tie cases.

Usage: python tests/golden/make_golden.py [REFERENCE_ROOT]
"""
from __future__ import annotations

import copy
import importlib.util
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))
from oracle import oracle as orc  # noqa: E402

# the checkout: the argument, else $TV_REFERENCE_ROOT or the root recorded by
# oracle/build_ref.sh
REF = pathlib.Path(sys.argv[1]) if len(sys.argv) > 1 else orc.reference_root()
if REF is None:
    sys.exit("make_golden: no reference checkout (pass its root or set TV_REFERENCE_ROOT)")

spec = importlib.util.spec_from_file_location(
    "tv_synthetic", str(REPO / "tensor-viterbi_gb300" / "tensor_viterbi" / "synthetic.py"))
syn = importlib.util.module_from_spec(spec)
sys.modules["tv_synthetic"] = syn
spec.loader.exec_module(syn)

sys.path.insert(0, str(REF))
from tensor_viterbi.hsmm import HSMM  # noqa: E402  (the reference's loader)
from tensor_viterbi.viterbi.tensor import decode_log_tensor_viterbi_cached  # noqa: E402

REF_FIXTURES = [
    "10states_1000steps_100dur",
    "15states_1000steps_250dur",
    "25states_1000steps_100dur",
    "10states_10000steps_250dur",
    "50states_1000steps_100dur",
    "75states_1000steps_100dur",
]


def run_reference(args, py_hsmm=None):
    ieee = orc.reference_module("ieee")
    fast = orc.reference_module("shipped")
    if ieee is None or fast is None:
        raise SystemExit("build the reference first: oracle/build_ref.sh")
    out = dict(
        path_cpp=np.asarray(ieee.decode_tensor_viterbi_cpp(*args), dtype=np.int32),
        path_omp=np.asarray(ieee.decode_tensor_viterbi_omp(*args), dtype=np.int32),
        path_cpp_fast=np.asarray(fast.decode_tensor_viterbi_cpp(*args), dtype=np.int32),
    )
    if py_hsmm is not None:
        out["path_py"] = np.asarray(decode_log_tensor_viterbi_cached(py_hsmm), dtype=np.int32)
    return out


def save(name, N, trans, em, dur_lin, start, dur, obs, source, py_hsmm=None):
    args = (N, trans, em, dur_lin, start, dur, obs)
    res = run_reference(args, py_hsmm)
    np.savez_compressed(
        HERE / f"{name}.npz",
        n_states=np.int64(N), trans_mat=trans, emission_probs=em, duration_probs_linear=dur_lin,
        start_probs=start, duration_probs=dur, obs_seq=obs.astype(np.int32), source=np.str_(source), **res)
    agree = {k: bool(np.array_equal(v, res["path_cpp"])) for k, v in res.items()}
    print(f"{name:34s} N={N:3d} D={dur.shape[0]:5d} T={obs.size:6d}  agree-with-cpp {agree}")


def from_json(stem):
    h = HSMM.load_model(str(REF / "data" / f"{stem}.json"))
    h.to_log_space()
    N = len(h.states)
    obs = np.asarray(h.obs_seq).astype(np.int32)
    py = copy.copy(h)
    small = obs.size * N * N * h.duration_probs.shape[0] <= 2e9
    save(f"ref_{stem}", N, np.ascontiguousarray(h.trans_mat), np.ascontiguousarray(h.emission_probs),
         np.ascontiguousarray(h.duration_probs_linear), np.ascontiguousarray(h.start_probs),
         np.ascontiguousarray(h.duration_probs), obs, f"reference data/{stem}.json", py if small else None)


def from_problem(name, p, source):
    save(name, p.N, p.trans_mat, p.emission_probs, p.duration_probs_linear, p.start_probs, p.duration_probs,
         p.obs_seq, source)


def tie_problems():
    """Models with exact ties, so that the lowest-(d, i) rule decides."""
    rng = np.random.default_rng(123)
    out = []
    # (a) two identical states: every score is tied between them.
    N, D, M, T = 4, 12, 5, 200
    lm = syn.random_model(rng, N, D, M, 2.0, 6.0)
    lm.B[1] = lm.B[0]
    lm.P[1] = lm.P[0]
    lm.A[:, [0, 1]] = lm.A[:, [0, 1]].mean(axis=1, keepdims=True)
    lm.A[[0, 1]] = lm.A[[0, 1]].mean(axis=0)
    np.fill_diagonal(lm.A, 0.0)
    lm.A /= lm.A.sum(axis=1, keepdims=True)
    lm.pi[[0, 1]] = lm.pi[[0, 1]].mean()
    st = syn.sample_states(rng, lm, T)
    out.append(("tie_twin_states", syn.to_problem(lm, syn.sample_discrete_obs(rng, lm.B, st)),
                "constructed: two identical states"))
    # (b) everything uniform: all candidates of a segment length tie.
    N, D, M, T = 5, 8, 3, 120
    pi = np.full(N, 1.0 / N)
    A = np.full((N, N), 1.0 / (N - 1))
    np.fill_diagonal(A, 0.0)
    B = np.full((N, M), 1.0 / M)
    P = np.full((N, D), 1.0 / D)
    lm = syn.LinearModel(pi, A, B, P)
    obs = rng.integers(0, M, size=T).astype(np.int32)
    out.append(("tie_uniform", syn.to_problem(lm, obs), "constructed: uniform model"))
    # (c) dyadic probabilities: sums of logs of powers of two tie often.
    N, D, M, T = 6, 16, 4, 400
    pi = np.full(N, 1.0 / 8); pi[0] += 1 - pi.sum()
    A = np.zeros((N, N))
    for i in range(N):
        others = [k for k in range(N) if k != i]
        A[i, others] = 1.0 / 8
        A[i, others[0]] += 1 - A[i].sum()
    B = np.full((N, M), 0.25)
    B[::2, 0] = 0.5; B[::2, 1] = 0.125; B[::2, 2] = 0.125
    P = np.full((N, D), 1.0 / 16)
    lm = syn.LinearModel(pi, A, B, P)
    obs = rng.integers(0, M, size=T).astype(np.int32)
    out.append(("tie_dyadic", syn.to_problem(lm, obs), "constructed: dyadic probabilities"))
    return out


def edge_problems():
    out = []
    p = syn.discrete_problem(1, 5, 40, 3, 2.0, 4.0, seed=7)
    out.append(("edge_one_state", p, "synthetic: N=1"))
    p = syn.discrete_problem(3, 1, 30, 4, 1.0, 1.0, seed=8)
    out.append(("edge_max_dur_one", p, "synthetic: D=1"))
    p = syn.discrete_problem(4, 25, 25, 6, 3.0, 10.0, seed=9)
    out.append(("edge_T_equals_D", p, "synthetic: T=D"))
    p = syn.discrete_problem(3, 1, 1, 4, 1.0, 1.0, seed=10)
    out.append(("edge_T_one", p, "synthetic: T=1, D=1"))
    p = syn.discrete_problem(5, 40, 41, 6, 3.0, 30.0, seed=11)
    out.append(("edge_T_D_plus_one", p, "synthetic: T=D+1"))
    return out


def main():
    for stem in REF_FIXTURES:
        from_json(stem)
    from_problem("syn_config0", syn.config0(), "synthetic config 0: N10 D100 T1000 M16 seed 0")
    from_problem("syn_batch_member", syn.discrete_problem(10, 250, 3000, 16, 5.0, 50.0, seed=21),
                 "synthetic batched-mix member: N10 D250 T3000 M16")
    from_problem("syn_long_dur", syn.discrete_problem(12, 400, 2500, 32, 50.0, 300.0, seed=22),
                 "synthetic long durations: N12 D400 T2500 M32")
    from_problem("syn_gaussian", syn.gaussian_problem(8, 60, 1500, 5.0, 40.0, seed=23),
                 "synthetic Gaussian emissions as a (T, N) table: N8 D60 T1500")
    for name, p, src in tie_problems():
        from_problem(name, p, src)
    for name, p, src in edge_problems():
        from_problem(name, p, src)


if __name__ == "__main__":
    main()
