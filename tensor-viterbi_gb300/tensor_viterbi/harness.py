"""Benchmark harness writing the reference's per-iteration CSV
(viterbi_app.py:66-76 there): one file per decoder function with the header
`function,n_states,timesteps,max_duration,iteration,elapsed_s` and one row
per timed iteration (elapsed wall time of the whole call, six decimals), so
the reference's plotting scripts read the numbers unchanged.

    python -m tensor_viterbi.harness MODEL.json [--iterations 5] [--out STEM]

decodes the JSON model (tensor_viterbi.hsmm.HSMM.load_model + to_log_space,
as the reference app does before each call) with decode_tensor_viterbi_cuda
and writes STEM_decode_tensor_viterbi_cuda.csv.
"""
from __future__ import annotations

import argparse
import copy
import csv
import time

CSV_HEADER = ["function", "n_states", "timesteps", "max_duration", "iteration", "elapsed_s"]


def bench_csv(fname: str, run_fn, model, n_states: int, timesteps: int, max_duration: int, iterations: int,
              path: str):
    """Time `run_fn(copy of model)` `iterations` times; write the CSV; return
    (times, last result).  Each iteration gets a shallow copy, as the
    reference's harness does, so in-place log conversion starts afresh."""
    times, last = [], None
    with open(path, "w", newline="") as f:
        w = csv.writer(f)
        w.writerow(CSV_HEADER)
        for i in range(iterations):
            m = copy.copy(model)
            t0 = time.perf_counter()
            res = run_fn(m)
            dt = time.perf_counter() - t0
            times.append(dt)
            w.writerow([fname, n_states, timesteps, max_duration, i, f"{dt:.6f}"])
            f.flush()
            last = res
    return times, last


def main(argv=None) -> int:
    from .hsmm import HSMM
    from .viterbi import native

    ap = argparse.ArgumentParser(description="decode a JSON HSMM and write the reference's timing CSV")
    ap.add_argument("model")
    ap.add_argument("--iterations", type=int, default=5)
    ap.add_argument("--out", default="")
    a = ap.parse_args(argv)
    native.configure("gb300", "cuda")
    h = HSMM.load_model(a.model)
    N, D, T = len(h.states), h.duration_probs.shape[0], len(h.obs_seq)
    stem = a.out or a.model.rsplit(".", 1)[0]

    def run(m):
        m.to_log_space()
        return native.decode_tensor_viterbi_cuda(*m.decoder_args())

    fname = native.decode_tensor_viterbi_cuda.__name__
    times, _ = bench_csv(fname, run, h, N, T, D, a.iterations, f"{stem}_{fname}.csv")
    print(f"{fname}: N={N} D={D} T={T} avg {sum(times) / len(times):.4f} s over {len(times)} iterations")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
