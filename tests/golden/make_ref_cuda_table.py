"""The agreement table of the reference's CUDA backend with its C++ decoder.

For every golden fixture and for the single-sequence bench model on a
T-prefix, decodes with the CPU restatement of the reference CUDA kernels
(oracle/tv_oracle_cuda.c, all four differences on) and with the C++ decoder
(the oracle), and records per case:
  cuda_path_equals_cpp   the two paths agree
  cuda_loglik_minus_cpp  difference of the final scores
  cuda_path_sha256       digest of the CUDA-semantics path (the GPU test checks
                         the reference kernels' own path against it)
  causes                 each difference that alone turns the C++ path into
                         the CUDA path, or, if none does alone, the ones whose
                         removal restores the C++ path
The reference kernels' own results on the GPU are checked against these
records by tests/test_ref_cuda_gpu.py.  CPU only; the reference checkout is not
needed (the fixtures hold the reference's inputs).

Usage: python tests/golden/make_ref_cuda_table.py
"""
from __future__ import annotations

import hashlib
import json
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "tensor-viterbi_gb300"))
from oracle import oracle as orc  # noqa: E402

C1_PREFIX = 12000  # 2D + 2000 at D = 5000


def tie_cases():
    """Exact-tie models whose tail block is at least one warp (min(T-1, D) >
    16), so the reference kernels run on them with defined results: a uniform
    model, dyadic probabilities and two identical states."""
    import tensor_viterbi.synthetic as syn
    rng = np.random.default_rng(321)
    out = []
    N, D, M, T = 5, 40, 3, 400
    A = np.full((N, N), 1.0 / (N - 1))
    np.fill_diagonal(A, 0.0)
    lm = syn.LinearModel(np.full(N, 1.0 / N), A, np.full((N, M), 1.0 / M), np.full((N, D), 1.0 / D))
    out.append(("cutie_uniform_D40", syn.to_problem(lm, rng.integers(0, M, size=T).astype(np.int32))))
    N, D, M, T = 6, 32, 4, 600
    pi = np.full(N, 1.0 / 8)
    pi[0] += 1 - pi.sum()
    A = np.zeros((N, N))
    for i in range(N):
        others = [k for k in range(N) if k != i]
        A[i, others] = 1.0 / 8
        A[i, others[0]] += 1 - A[i].sum()
    B = np.full((N, M), 0.25)
    B[::2, 0] = 0.5
    B[::2, 1] = 0.125
    B[::2, 2] = 0.125
    lm = syn.LinearModel(pi, A, B, np.full((N, D), 1.0 / 32))
    out.append(("cutie_dyadic_D32", syn.to_problem(lm, rng.integers(0, M, size=T).astype(np.int32))))
    N, D, M, T = 4, 48, 5, 500
    lm = syn.random_model(rng, N, D, M, 4.0, 20.0)
    lm.B[1] = lm.B[0]
    lm.P[1] = lm.P[0]
    lm.A[:, [0, 1]] = lm.A[:, [0, 1]].mean(axis=1, keepdims=True)
    lm.A[[0, 1]] = lm.A[[0, 1]].mean(axis=0)
    np.fill_diagonal(lm.A, 0.0)
    lm.A /= lm.A.sum(axis=1, keepdims=True)
    lm.pi[[0, 1]] = lm.pi[[0, 1]].mean()
    st = syn.sample_states(rng, lm, T)
    out.append(("cutie_twin_states_D48", syn.to_problem(lm, syn.sample_discrete_obs(rng, lm.B, st))))
    return [(name, p.args()) for name, p in out]


def cases():
    for p in sorted(HERE.glob("*.npz")):
        z = np.load(p)
        yield p.stem, (int(z["n_states"]), z["trans_mat"], z["emission_probs"], z["duration_probs_linear"],
                       z["start_probs"], z["duration_probs"], z["obs_seq"])
    yield from tie_cases()
    import tensor_viterbi.synthetic as syn
    prob = syn.config1()
    yield f"bench_N75_D5000_prefix{C1_PREFIX}", prob.model_args() + (np.ascontiguousarray(prob.obs_seq[:C1_PREFIX]),)


def sha(path):
    return hashlib.sha256(np.ascontiguousarray(path, dtype=np.int32).tobytes()).hexdigest()


def row(args):
    cpp = orc.decode(*args, variant="omp")
    cu = orc.decode_cuda_semantics(*args, flags=orc.CU_ALL)
    same = bool(np.array_equal(cu["path"], cpp["path"]))
    r = {"N": int(args[0]), "D": int(np.asarray(args[5]).shape[0]), "T": int(np.asarray(args[6]).size),
         "cuda_path_equals_cpp": same, "cuda_loglik_minus_cpp": cu["loglik"] - cpp["loglik"],
         "cuda_path_sha256": sha(cu["path"]), "causes": []}
    if not same:
        alone = [k for k in orc.CU_NAMES
                 if np.array_equal(orc.decode_cuda_semantics(*args, flags=k)["path"], cu["path"])]
        if alone:
            r["causes"] = [orc.CU_NAMES[k] for k in alone]
        else:
            needed = [k for k in orc.CU_NAMES
                      if np.array_equal(orc.decode_cuda_semantics(*args, flags=orc.CU_ALL & ~k)["path"], cpp["path"])]
            r["causes"] = ["combination of: " + ", ".join(orc.CU_NAMES[k] for k in needed or orc.CU_NAMES)]
    return r


def main():
    table = {}
    for name, args in cases():
        table[name] = row(args)
        print(name, table[name]["cuda_path_equals_cpp"], table[name]["causes"], flush=True)
    out = {"what": "reference CUDA backend (src/kernels.cu) vs its C++ decoder (src/hsmm.cu:233-373), "
                   "from the CPU restatement oracle/tv_oracle_cuda.c; made by tests/golden/make_ref_cuda_table.py",
           "cases": table}
    (HERE / "ref_cuda_agreement.json").write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main()
