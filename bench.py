#!/usr/bin/env python3
"""HSMM Viterbi decode benchmark on GB300: T*N*D cells per second.

Default workload: one long sequence, N=75 states, max duration D=5000,
T=1,000,000 observations over M=32 symbols, duration means ~U[50, 2500]
(seeded synthetic model of the benchmark family; the reference publishes no
dataset for this shape).  A "step" is one full decode of that sequence.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value   device time of K decodes with the inputs resident in HBM, L2 flushed
        (256 MiB write) between decodes, CUDA events on the decode stream;
        max over ranks; whole-job cells/s.
e2e     the reference-facing call decode_tensor_viterbi_cuda(...) with host
        numpy buffers: model preparation and upload, observation H2D, decode,
        path D2H, all inside the timed region.
roofline the grid decode kernel's algorithmic bytes (24 B per T*N*D cell:
        window score, emission window sum and duration log-pmf, FP64) over its
        event-timed duration, against the measured HBM copy bandwidth.
cpu_baseline / --impl reference: the CPU restatement of the reference's
        OpenMP decoder (oracle/, -O3 -ffast-math) on the host's cores, on a
        bounded T-prefix of the same workload.
Under torchrun (N > 1) every rank decodes its own replica: a single sequence
does not shard (each step needs the whole previous score vector).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import pathlib
import statistics
import subprocess
import sys
import tempfile
import time

REPO = pathlib.Path(__file__).resolve().parent
PKG = REPO / "tensor-viterbi_gb300"
for _p in (str(REPO), str(PKG)):
    if _p not in sys.path:
        sys.path.insert(0, _p)

ALGO_BYTES_PER_CELL = 24
METRIC = "T*N*D cells/s (HSMM Viterbi decode, FP64 log space, exact paths)"

WORKLOADS = {
    "single_N75_D5000_T1e6": dict(N=75, D=5000, T=1_000_000, M=32, lo=50.0, hi=2500.0, seed=1),
    "single_N10_D100_T1e3": dict(N=10, D=100, T=1000, M=16, lo=5.0, hi=50.0, seed=0),
    "single_N100_D10000_T1e6": dict(N=100, D=10_000, T=1_000_000, M=64, lo=5.0, hi=50.0, seed=4),
    "single_N100_D10000_T1e7": dict(N=100, D=10_000, T=10_000_000, M=64, lo=5.0, hi=50.0, seed=4),
    # 4096 sequences sharing one model, lengths log-uniform in [1e3, 1e5]
    "batch_4096_N10_D250": dict(kind="batch", n_seq=4096, N=10, D=250, M=16, lo=1e3, hi=1e5, seed=2),
    # the training step: one forward-backward E step of hsmmlearn's EM fit
    # (FBImpl.cpp) on one sequence, J states, M durations, T observations
    "fb_J10_M100_T1e5": dict(kind="fb", J=10, M=100, T=100_000, K=16, seed=5),
    # served: Poisson arrivals of requests with their own models; N from
    # {10,15,25,50}, D from {100,250,500,1000}, T log-uniform in [1e3, 1e6],
    # half discrete (M = 32), half Gaussian; arrival rates at fractions of the
    # measured capacity
    "served_N10-50_D100-1000_T1e3-1e6": dict(kind="served", n_req=5000, Ns=[10, 15, 25, 50], Ds=[100, 250, 500, 1000],
                                             Tlo=1e3, Thi=1e6, M=32, lo=5.0, hi=50.0, loads=[0.25, 0.5, 0.8],
                                             seed=3),
}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def make_problem(w):
    import tensor_viterbi.synthetic as syn
    return syn.discrete_problem(w["N"], w["D"], w["T"], w["M"], w["lo"], w["hi"], seed=w["seed"])


def measured_peaks():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def committed_traffic(kernel: str, workload: str):
    """DRAM bytes per launch from a committed ncu summary, if there is one."""
    p = REPO / "profiles" / "traffic.json"
    if not p.exists():
        return None
    try:
        d = json.loads(p.read_text())
        return d.get(kernel, {}).get(workload)
    except Exception:
        return None


def committed_onchip(kernel: str, workload: str, kernel_ms: float):
    """L2 and shared-memory bytes per launch from a committed ncu summary
    (profiles/traffic.json, scaled to the workload), as GB/s over the
    measured kernel time."""
    p = REPO / "profiles" / "traffic.json"
    out = {"l2_gbs": None, "smem_gbs": None}
    if not p.exists():
        return out
    try:
        d = json.loads(p.read_text()).get(kernel + "_onchip", {}).get(workload)
    except Exception:
        return out
    if d and kernel_ms and kernel_ms > 0:
        out["l2_gbs"] = d["l2_bytes"] / (kernel_ms / 1e3) / 1e9
        out["smem_gbs"] = d["smem_bytes"] / (kernel_ms / 1e3) / 1e9
        out["onchip_source"] = d.get("source")
    return out


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append(dict(sm=float(parts[1]), smax=float(parts[2]), reasons=parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        active = sorted({names[k] for r in rows for k in range(4) if r["reasons"][k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(r["sm"] for r in rows), "sm_max_mhz": max(r["smax"] for r in rows),
                "reasons": active, "samples": len(rows)}


def window_cells(Ts, N, D):
    """Window cells the recursion evaluates over a T-prefix: N * min(t, D) at
    every step t >= 1.  Over a whole sequence this is T*N*D less the ramp
    (N*D^2/2), so a CPU rate taken with it is the steady-state rate of the
    metric's cells."""
    n = Ts - 1
    ramp = min(n, D)
    return N * (ramp * (ramp + 1) // 2 + max(0, n - D) * D)


def prefix_for(w, cells_cap, longest):
    """The longest T-prefix up to `longest` steps whose window cells stay
    within cells_cap (at least D + 1000 steps, at most the workload's T)."""
    N, D = w["N"], w["D"]
    Ts = min(w["T"], longest)
    while Ts > D + 1000 and window_cells(Ts, N, D) > cells_cap:
        Ts -= max(1, (window_cells(Ts, N, D) - int(cells_cap)) // (N * D) + 1)
    return max(min(w["T"], D + 1000), Ts)


# CPU-baseline sample: the T-prefix 2D + 20000 (long enough for the window to
# be fully rolled for 20000 steps), capped at ~1.1e10 window cells (about a
# minute of a 16-core host); the reference arm's per-step sample is ~1.2e9
# window cells (about 7 s), so that 25 of them take about three minutes.
CPU_BASELINE_CELLS = 1.1e10
REFERENCE_STEP_CELLS = 1.2e9
# Parity check of the timed workload: the IEEE oracle on the T-prefix 2D + 2000.
PARITY_CELLS = 6.0e9


def cpu_sample(prob, w, threads: int, cells_cap: float):
    """The oracle's OpenMP decoder (-O3 -ffast-math build, the reference's CPU
    flags) on a T-prefix of the workload.  Returns (cells/s, seconds,
    T_sample, cells) with cells counted by window_cells."""
    from oracle import oracle as orc
    Ts = prefix_for(w, cells_cap, 2 * w["D"] + 20000)
    args = prob.model_args() + (prob.obs_seq[:Ts],)
    t0 = time.perf_counter()
    orc.decode(*args, variant="omp", nthreads=threads, fast=True)
    dt = time.perf_counter() - t0
    cells = window_cells(Ts, w["N"], w["D"])
    return cells / dt, dt, Ts, cells


def run_reference(args, w, wname):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import oracle as orc
    orc.build()
    threads = orc.cpu_count()
    prob = make_problem(w)
    for _ in range(args.warmup):
        cpu_sample(prob, w, threads, REFERENCE_STEP_CELLS)
    secs = []
    for _ in range(args.steps):
        v, dt, Ts, cells = cpu_sample(prob, w, threads, REFERENCE_STEP_CELLS)
        secs.append(dt)
    value = cells * len(secs) / sum(secs)
    sample = (f"T-prefix {Ts} of the workload per step ({cells:.3e} window cells, N*min(t,D) per step), "
              f"OpenMP restatement of src/hsmm.cu:376-600 built -O3 -ffast-math, {threads} threads")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(secs) / len(secs),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_of(w, wname, ws),
        "cpu_baseline": {"value": value, "unit": "cells/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def fb_problem(w):
    """A seeded HSMM (Dirichlet transition, duration and emission rows, zero
    self-transitions) and a sequence sampled from it; returns (d, p, pi, pdf)
    in hsmmlearn's _fb_impl layouts, pdf the emission likelihoods."""
    import numpy as np
    import tensor_viterbi.synthetic as syn
    rng = np.random.default_rng(w["seed"])
    J, M, T, K = w["J"], w["M"], w["T"], w["K"]
    lm = syn.random_model(rng, J, M, K, 5.0, M / 2.0)
    states = syn.sample_states(rng, lm, T)
    obs = syn.sample_discrete_obs(rng, lm.B, states)
    pdf = np.ascontiguousarray(lm.B[:, obs])
    pdf[pdf < 1e-12] = 1e-12
    return np.ascontiguousarray(lm.P), np.ascontiguousarray(lm.A), lm.pi, pdf


FB_FLOPS_PER_CELL = 8  # forward: a multiply and a fused multiply-add; backward: a multiply and two


def run_fb(args, w, wname):
    """The forward-backward E step (tv_fb) through its host-buffer call, as
    hsmmlearn's fit makes it; cells = T*J*M per pass.  `value`: the kernel's
    own device time (CUDA events around its launch, inputs in HBM); `e2e`:
    the whole call, inputs copied in and outputs copied out.  L2 is flushed
    (256 MiB write) before every pass, outside the timed region.  Roofline:
    the FP64 issue of the one SM that runs the sequence (tv_fp64_peak,
    measured in the same process).  CPU baseline: the oracle's restatement of
    FBImpl.cpp (serial, bit-exact to the reference's build)."""
    import numpy as np
    import torch
    from tensor_viterbi.viterbi import native
    ws, rank, _ = dist_env()
    torch.cuda.set_device(0)
    native.configure("gb300", "cuda")
    d, p, pi, pdf = fb_problem(w)
    J, M, T = w["J"], w["M"], w["T"]
    cells = T * J * M
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(args.warmup):
        native.forward_backward(1, d, p, pi, pdf)
    peak = native.fp64_peak()
    torch.cuda.synchronize()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    secs, kms = [], []
    for _ in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = native.forward_backward(1, d, p, pi, pdf)
        secs.append(time.perf_counter() - t0)
        kms.append(native.fb_last_kernel_ms())
    clk = clocks.stop()
    e2e_value = cells * len(secs) / sum(secs)
    # kernels per pass: the E step, then (J <= 32, M <= 128) eta's window terms in chunks and eta's sum
    fb_launches = 3 if (J <= 32 and M <= 128) else 1
    kernel_ms = sum(kms) / len(kms)
    value = cells / (kernel_ms / 1e3)
    achieved = FB_FLOPS_PER_CELL * cells / (kernel_ms / 1e3) / 1e9
    roofline = {"bound": "fp64 (the one SM that runs the sequence)", "achieved": achieved,
                "peak": peak["flops"] / 1e9, "unit": "GFLOP/s", "frac": achieved / (peak["flops"] / 1e9),
                "traffic": committed_traffic("fb_small_kernel", wname),
                "flops_per_cell": FB_FLOPS_PER_CELL, "kernel_ms": kernel_ms,
                "peak_source": "measured in this run: tv_fp64_peak (one SM, 8 warps x 8 independent FP64 "
                               "fused multiply-add chains)",
                "fp64_warp_insts_per_clock": peak["warp_insts_per_clock"],
                "fp64_dependent_clocks": peak["dependent_clocks"],
                "note": "a step is a serial chain on one SM; DRAM traffic is O(J*T): the window stays on chip"}
    cpu = parity = None
    if not args.no_cpu_baseline or not args.no_parity:
        from oracle import oracle as orc
        t0 = time.perf_counter()
        ref = orc.forward_backward(1, d, p, pi, pdf)
        dt = time.perf_counter() - t0
        cpu = {"value": cells / dt, "unit": "cells/s", "cores": 1, "kind": "port",
               "sample": f"the whole workload ({dt:.1f} s): the serial C restatement of hsmmlearn's FBImpl.cpp, "
                         f"bit-exact to the reference's own build"}
        big = {k: float(np.abs(ref[k]).max()) for k in orc.FB_KEYS}
        parity = {"err_equal": r["err"] == ref["err"],
                  "max_err_over_max_entry": max(float(np.abs(r[k] - ref[k]).max()) / big[k] for k in orc.FB_KEYS),
                  "oracle": "C restatement of hsmmlearn FBImpl.cpp"}
    io = (J * M + J * J + J + J * T) * 8 + 2 * J * T * 8
    line = {"metric": "T*J*M cells/s (HSMM forward-backward E step, FP64)", "value": value, "unit": "cells/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": kernel_ms,
            "e2e_ms_per_step": 1e3 * sum(secs) / len(secs),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": wname, "states": J, "durations": M, "T": T, "symbols": w["K"], "censoring": 1,
                       "form": "one sequence, host buffers (hsmmlearn's _fb_impl call)",
                       "l2": "flushed between steps (256 MiB write)"},
            "roofline": roofline, "cpu_baseline": cpu, "parity": parity,
            "e2e": {"value": e2e_value, "unit": "cells/s", "h2d_bytes_per_step": io,
                    "d2h_bytes_per_step": (5 * J * T + T + J * M) * 8},
            "gpu_launches": args.steps * fb_launches, "clocks": clk}
    print(json.dumps(line), flush=True)
    return 0


def run_reference_batch(args, w, wname):
    """The reference's way to decode many sequences: one CPU decode per
    sequence (src/hsmm.cu:376-600, the OpenMP port), over every 256th sequence
    of the same mix per step (16 sequences, about 1/256 of its cells), on all
    host cores."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    import tensor_viterbi.synthetic as syn
    from oracle import oracle as orc
    orc.build()
    threads = orc.cpu_count()
    prob, seqs = syn.batch_problem(w["n_seq"], w["N"], w["D"], w["M"], w["lo"], w["hi"], seed=w["seed"])
    sample = seqs[::256]
    N, D = w["N"], w["D"]
    cells = sum(window_cells(s.size, N, D) for s in sample)

    def step():
        t0 = time.perf_counter()
        for s in sample:
            orc.decode(*prob.model_args(), s, variant="omp", nthreads=threads, fast=True)
        return time.perf_counter() - t0

    for _ in range(args.warmup):
        step()
    secs = [step() for _ in range(args.steps)]
    value = cells * len(secs) / sum(secs)
    sample_txt = (f"every 256th sequence of the mix per step ({len(sample)} sequences, {cells:.3e} window cells), "
                  f"decoded one at a time by the OpenMP restatement of src/hsmm.cu:376-600 built -O3 -ffast-math, "
                  f"{threads} threads")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(secs) / len(secs),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": wname, "n_seq": w["n_seq"], "n_states": N, "max_dur": D, "symbols": w["M"],
                   "lengths": f"log-uniform [{w['lo']:g},{w['hi']:g}]", "form": "one decode per sequence"},
        "cpu_baseline": {"value": value, "unit": "cells/s", "cores": threads, "kind": "port", "sample": sample_txt},
        "e2e": {"value": value, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def config_of(w, wname, ws):
    return {"workload": wname, "n_states": w["N"], "max_dur": w["D"], "T": w["T"], "symbols": w["M"],
            "duration_means": f"U[{w['lo']:g},{w['hi']:g}]", "seed": w["seed"],
            "l2": "flushed between steps (256 MiB write)", "parallelism": f"replicas x{ws}",
            "form": "single sequence"}


def run_ours(args, w, wname):
    import numpy as np
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.device("cuda", torch.cuda.current_device())

    from tensor_viterbi.viterbi import native
    native.configure("gb300", "cuda")
    prob = make_problem(w)
    N, D, T = w["N"], w["D"], w["T"]
    cells = T * N * D

    model = native.Model(*prob.model_args())
    model.set_timing(True)
    obs = torch.from_numpy(prob.obs_seq).to(dev)
    path = torch.empty_like(obs)
    ll = torch.zeros(1, dtype=torch.float64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()

    def one_decode():
        flush.fill_(1)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        model.decode_device(obs.data_ptr(), T, path.data_ptr(), ll.data_ptr(), stream.cuda_stream)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1), model.kernel_ms(), model.last_launches()

    for _ in range(args.warmup):
        one_decode()
    barrier(ws)
    torch.cuda.synchronize()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    t_wall = time.perf_counter()
    step_ms, kern_ms, launches = [], [], 0
    for _ in range(args.steps):
        a, k, n = one_decode()
        step_ms.append(a)
        kern_ms.append(k)
        launches += n
    torch.cuda.synchronize()
    barrier(ws)
    wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    total_ms = max_over_ranks(sum(step_ms), ws)
    value = cells * args.steps * ws / (total_ms / 1e3)

    # Roofline of the grid decode kernel (events on its own stream).
    peak, peak_kind = measured_peaks()
    kmean = statistics.mean(kern_ms) if kern_ms and min(kern_ms) > 0 else float("nan")
    achieved = ALGO_BYTES_PER_CELL * cells / (kmean / 1e3) / 1e9
    traffic = committed_traffic("grid_decode_kernel", wname)
    # The recurrence is serial: the step period against the measured floor of
    # the head's critical chain (matvec, exact score, barrier alone on one SM).
    floor = None
    if model.last_path() == "grid" and N <= 128:
        floor = native.step_floor(N, D, 20000)

    # e2e: the drop-in call with host buffers, copies inside the timed region.
    h2d = (N * N + prob.O * N + N + 2 * D * N) * 8 + T * 4
    d2h = T * 4 + 8 + 16
    if args.no_e2e:
        e2e_value, e2e_total, same = None, float("nan"), None
        ll_host = float(ll.item())
    else:
        args_host = prob.args()
        for _ in range(max(1, min(args.warmup, 2))):
            native.decode_tensor_viterbi_cuda(*args_host)
        barrier(ws)
        e2e_s = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            p_host, ll_host = native.decode_tensor_viterbi_cuda_loglik(*args_host)
            e2e_s.append(time.perf_counter() - t0)
        e2e_total = max_over_ranks(sum(e2e_s), ws)
        e2e_value = cells * args.steps * ws / e2e_total
        # The timed device-resident decode and the drop-in call must agree.
        same = bool(np.array_equal(path.cpu().numpy(), p_host)) and float(ll.item()) == ll_host

    line = None
    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            from oracle import oracle as orc
            orc.build()
            threads = orc.cpu_count()
            v, dt, Ts, cc = cpu_sample(prob, w, threads, CPU_BASELINE_CELLS)
            cpu = {"value": v, "unit": "cells/s", "cores": threads, "kind": "port",
                   "sample": f"T-prefix {Ts} ({cc:.3e} window cells, N*min(t,D) per step, {dt:.1f} s), "
                             f"OpenMP restatement of src/hsmm.cu:376-600 built -O3 -ffast-math, {threads} threads"}
        parity = None
        if not args.no_parity:
            # The timed workload's own model and observations, decoded on a
            # T-prefix by the same model and kernel, against the IEEE oracle.
            from oracle import oracle as orc
            Tp = prefix_for(w, PARITY_CELLS, 2 * D + 2000)
            obs_p = np.ascontiguousarray(prob.obs_seq[:Tp])
            gp, gl = model.decode(obs_p, return_loglik=True)
            t0 = time.perf_counter()
            ref = orc.decode(*prob.model_args(), obs_p, variant="omp")
            parity = {"T_prefix": Tp, "kernel_path": model.last_path(),
                      "path_equal": bool(np.array_equal(gp, ref["path"])), "loglik_equal": gl == ref["loglik"],
                      "oracle": "IEEE OpenMP restatement of src/hsmm.cu:376-600",
                      "oracle_s": round(time.perf_counter() - t0, 1)}
        line = {
            "metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_of(w, wname, ws),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "grid_decode_kernel", "kernel_ms": kmean,
                         "algo_bytes_per_launch": ALGO_BYTES_PER_CELL * cells, "peak_source": peak_kind,
                         "step_us": 1e3 * kmean / T,
                         "floor_us": floor["chain_us_per_step"] if floor else None,
                         "step_over_floor": (1e3 * kmean / T) / floor["chain_us_per_step"] if floor else None,
                         "xsm_roundtrip_us": floor["roundtrip_us"] if floor else None,
                         **committed_onchip("grid_decode_kernel", wname, kmean)},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "cells/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": 1e3 * e2e_total / args.steps},
            "gpu_launches": launches,
            "clocks": clk,
            "kernel_path": model.last_path(),
            "wall_s": wall,
            "consistent": same,
            "parity": parity,
            "loglik": ll_host,
        }
        print(json.dumps(line), flush=True)
    model.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def served_request(w, k):
    """Request k of the served workload: (kind, problem, T), with its own
    seeded model (seed (w.seed, k), so every arrival rate replays the same
    requests) and observations sampled from it.  N from w.Ns, D from w.Ds, T
    log-uniform in [Tlo, Thi]; odd requests Gaussian, even ones discrete."""
    import bisect
    import math
    import numpy as np
    import tensor_viterbi.synthetic as syn
    rng = np.random.default_rng([w["seed"], k])
    N = int(rng.choice(w["Ns"]))
    D = int(rng.choice(w["Ds"]))
    T = max(int(math.exp(rng.uniform(math.log(w["Tlo"]), math.log(w["Thi"])))), D)
    gauss = k % 2 == 1
    lm = syn.random_model(rng, N, D, 2 if gauss else w["M"], w["lo"], w["hi"])
    # segment-wise state path (bisect on cumulative rows: fast per segment)
    cP = [list(np.cumsum(r) / r.sum()) for r in lm.P]
    cA = [list(np.cumsum(r) / r.sum()) for r in lm.A]
    cpi = list(np.cumsum(lm.pi) / lm.pi.sum())
    u = rng.random(2 * T + 2).tolist()
    states = np.empty(T, dtype=np.int32)
    t, ui = 0, 0
    s_ = min(bisect.bisect_right(cpi, u[ui]), N - 1)
    ui += 1
    while t < T:
        dlen = min(bisect.bisect_right(cP[s_], u[ui]), D - 1) + 1
        states[t:t + dlen] = s_
        t += dlen
        s_ = min(bisect.bisect_right(cA[s_], u[ui + 1]), N - 1)
        ui += 2
    if gauss:
        mu = rng.normal(0.0, 2.0, size=N)
        sd = rng.uniform(0.5, 2.0, size=N)
        x = rng.normal(mu[states], sd[states])
        p = syn.to_problem(lm, np.zeros(0, dtype=np.int32), emission_log=np.zeros((1, N)),
                           meta=dict(x=x, mu=mu, sd=sd))
        return "gauss", p, T
    obs = syn.sample_discrete_obs(rng, lm.B, states)
    return "disc", syn.to_problem(lm, obs), T


def run_served(args, w, wname):
    """Served decode.  First the saturated capacity: a burst of requests all
    submitted at once, completed requests per second over the makespan.  Then
    Poisson arrivals at fixed fractions of that capacity (--loads), the same
    requests at every rate, generated just ahead of their arrival times.  Per
    rate: p50/p99 of the whole latency (submission to completion), of the
    service time (admission to completion) and of the queue time (submission
    to admission), all on the server's clock; throughput over the makespan.
    Beside it, the plain per-request loop on a sample of the same requests."""
    import functools
    import multiprocessing as mp
    import queue as queue_mod
    import random
    import threading
    import numpy as np
    # Requests are generated by a pool of host processes (spawned, before any
    # CUDA work) so that generation keeps ahead of the highest arrival rate.
    pool = mp.get_context("spawn").Pool(processes=max(1, min(8, (os.cpu_count() or 2) - 2)))
    make = functools.partial(served_request, w)
    from tensor_viterbi.viterbi import native
    native.configure("gb300", "cuda")
    n_req = args.requests or w["n_req"]

    def submit(srv, kind, p):
        if kind == "disc":
            return srv.submit(*p.args())
        return srv.submit_gaussian(p.n_states, p.trans_mat, p.duration_probs_linear, p.start_probs,
                                   p.duration_probs, p.meta["x"], p.meta["mu"], p.meta["sd"])

    def plain(k, p):
        if k == "disc":
            with native.Model(*p.model_args()) as m:
                m.decode(p.obs_seq)
        else:
            with native.GaussianModel(p.n_states, p.trans_mat, p.duration_probs_linear, p.start_probs,
                                      p.duration_probs, p.meta["x"], p.meta["mu"], p.meta["sd"]) as m:
                m.decode()

    # plain loop: a sample of the same requests decoded one at a time
    plain(*served_request(w, 0)[:2])  # warm-up (context, kernel loading)
    sample = pool.map(make, range(8, 32))
    t0 = time.perf_counter()
    for k, p, _ in sample:
        plain(k, p)
    loop_rate = sum(T * p.n_states * p.D for _, p, T in sample) / (time.perf_counter() - t0)
    del sample
    with native.Server() as srv:  # warm-up: kernel loading, pool growth
        for t in [submit(srv, k, p) for k, p, _ in pool.map(make, range(8))]:
            srv.wait(t)

    def run_rate(n, rate):
        """n requests; Poisson arrivals at `rate` per second, or all at once
        when rate is None.  The process pool generates requests ahead of
        their arrival (at most 64 waiting), a feeder thread submits them on
        time, and this thread collects the results in submission order."""
        rnd = random.Random(int((rate or 0) * 1000) * 7919 + w["seed"])
        arrivals, acc = [], 0.0
        for _ in range(n):
            if rate:
                acc += rnd.expovariate(rate)
            arrivals.append(acc)
        made = queue_mod.Queue(maxsize=64)
        tickets = [None] * n
        cells = [0] * n
        lat, svc, que, errors = [], [], [], []

        def producer():
            for item in pool.imap(make, range(n), chunksize=2):
                made.put(item)

        with native.Server(max_inflight=args.max_inflight) as srv:
            prod = threading.Thread(target=producer, daemon=True)
            prod.start()
            ready = [made.get() for _ in range(n)] if rate is None else []  # a burst: all made first
            t0 = time.perf_counter()

            def feeder():
                for i in range(n):
                    k, p, T = ready[i] if i < len(ready) else made.get()
                    dt = arrivals[i] - (time.perf_counter() - t0)
                    if dt > 0:
                        time.sleep(dt)
                    cells[i] = T * p.n_states * p.D
                    tickets[i] = submit(srv, k, p)

            th = threading.Thread(target=feeder)
            th.start()
            for i in range(n):
                while tickets[i] is None:
                    time.sleep(0.0005)
                try:
                    _, _, l_ms, q_ms = srv.wait(tickets[i])
                except RuntimeError as e:
                    errors.append(f"request {i}: {e} stats={srv.stats()}")
                    continue
                lat.append(l_ms)
                que.append(q_ms)
                svc.append(l_ms - q_ms)
            th.join()
            makespan = time.perf_counter() - t0
            st = srv.stats()
        pct = lambda a, q: float(np.percentile(a, q)) if a else None
        return {"requests": n, "completed": st["completed"], "failed": st["failed"],
                "latency_p50_ms": pct(lat, 50), "latency_p99_ms": pct(lat, 99),
                "service_p50_ms": pct(svc, 50), "service_p99_ms": pct(svc, 99),
                "queue_p50_ms": pct(que, 50), "queue_p99_ms": pct(que, 99),
                "throughput_cells_per_s": sum(cells) / makespan, "requests_per_s": len(lat) / makespan,
                "makespan_s": makespan, "mean_cells_per_request": sum(cells) / n,
                "peak_bytes": st["peak_bytes"], "budget_bytes": st["budget"], "errors": errors[:3]}

    import torch
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    n_cap = min(n_req, args.capacity_requests)
    cap = run_rate(n_cap, None)
    capacity = cap["requests_per_s"]
    out = []
    loads = ([] if args.loads == "none" else [float(x) for x in args.loads.split(",")]) if args.loads else w["loads"]
    for f in loads:
        r = run_rate(n_req, f * capacity)
        r.update({"offered_load": f, "rate_per_s": f * capacity})
        out.append(r)
    clk = clocks.stop()
    pool.close()
    line = {"metric": "served decode: p50/p99 latency (service and queue) and cells/s at fractions of capacity",
            "value": cap["throughput_cells_per_s"], "unit": "cells/s", "n_gpus": 1, "higher_is_better": True,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": wname, "requests_per_rate": n_req, "capacity_burst": n_cap, "N": w["Ns"],
                       "D": w["Ds"], "T": f"log-uniform [{w['Tlo']:g}, {w['Thi']:g}]",
                       "emissions": "half discrete (M=32), half Gaussian", "form": "served (continuous batching)"},
            "capacity": cap, "rates": out, "plain_loop_cells_per_s": loop_rate,
            "vs_plain_loop": cap["throughput_cells_per_s"] / loop_rate, "clocks": clk}
    print(json.dumps(line), flush=True)
    return 0


def run_batch(args, w, wname):
    """Batched form: all sequences in one persistent launch, against the plain
    single-sequence decode looped over a sample of the same sequences."""
    import numpy as np
    import torch
    import tensor_viterbi.synthetic as syn
    from tensor_viterbi.viterbi import native
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.device("cuda", torch.cuda.current_device())
    native.configure("gb300", "cuda")
    prob, seqs = syn.batch_problem(w["n_seq"], w["N"], w["D"], w["M"], w["lo"], w["hi"], seed=w["seed"])
    # ranks take a longest-processing-time share of the sequences (no collective)
    from tensor_viterbi.sharding import my_shard
    mine = my_shard([s.size for s in seqs], ws, rank)
    my = [seqs[k] for k in mine]
    N, D = w["N"], w["D"]
    lens = np.array([s.size for s in my], dtype=np.int64)
    cells = int(lens.sum()) * N * D
    off = np.zeros(len(my) + 1, dtype=np.int64)
    off[1:] = np.cumsum(lens)
    model = native.Model(*prob.model_args())
    model.set_timing(True)
    obs = torch.from_numpy(np.concatenate(my)).to(dev)
    path = torch.empty_like(obs)
    ll = torch.zeros(len(my), dtype=torch.float64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()

    def one():
        flush.fill_(1)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        model.decode_batch_device(off, obs.data_ptr(), path.data_ptr(), ll.data_ptr(), stream.cuda_stream)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1), model.kernel_ms(), model.last_launches()

    for _ in range(args.warmup):
        one()
    barrier(ws)
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    step_ms, kern_ms, launches = [], [], 0
    for _ in range(args.steps):
        a, k, n = one()
        step_ms.append(a)
        kern_ms.append(k)
        launches += n
    barrier(ws)
    clk = clocks.stop()
    total_ms = max_over_ranks(sum(step_ms), ws)
    value = sum_over_ranks(cells, ws) * args.steps / (total_ms / 1e3)
    peak, peak_kind = measured_peaks()
    kmean = statistics.mean(kern_ms)
    achieved = ALGO_BYTES_PER_CELL * cells / (kmean / 1e3) / 1e9

    # plain single-sequence decode looped over a sample of the same sequences
    samp = np.linspace(0, len(my) - 1, num=min(24, len(my))).astype(int)
    pt, pc = 0.0, 0
    for k in samp:
        o = torch.from_numpy(my[k]).to(dev)
        p = torch.empty_like(o)
        model.decode_device(o.data_ptr(), o.numel(), p.data_ptr(), 0, stream.cuda_stream)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        model.decode_device(o.data_ptr(), o.numel(), p.data_ptr(), 0, stream.cuda_stream)
        torch.cuda.synchronize()
        pt += time.perf_counter() - t0
        pc += int(o.numel()) * N * D
    plain = pc / pt

    # end to end with host buffers
    e2e_s = []
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        paths, lls = model.decode_batch(my, return_loglik=True)
        e2e_s.append(time.perf_counter() - t0)
    e2e_value = sum_over_ranks(cells, ws) * len(e2e_s) / max_over_ranks(sum(e2e_s), ws)
    same = all(np.array_equal(a, b) for a, b in zip(paths, np.split(path.cpu().numpy(), off[1:-1])))
    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            from oracle import oracle as orc
            orc.build()
            threads = orc.cpu_count()
            t0 = time.perf_counter()
            cc = 0
            for s in my[: len(my)]:
                orc.decode(*prob.model_args(), s, variant="omp", nthreads=threads, fast=True)
                cc += s.size * N * D
                if time.perf_counter() - t0 > 15.0:
                    break
            dt = time.perf_counter() - t0
            cpu = {"value": cc / dt, "unit": "cells/s", "cores": threads, "kind": "port",
                   "sample": f"{cc / (N * D):.0f} steps of the mix decoded one sequence at a time ({dt:.1f} s), "
                             f"OpenMP restatement of src/hsmm.cu:376-600, {threads} threads"}
        parity = None
        if not args.no_parity:
            # Sequences of the timed mix, as the batched launch decoded them,
            # against the IEEE oracle: every 512th sequence of up to 2e4 steps.
            from oracle import oracle as orc
            pick = [k for k in range(0, len(my), 512) if my[k].size <= 20000][:8]
            t0 = time.perf_counter()
            ok_p = ok_l = True
            for k in pick:
                ref = orc.decode(*prob.model_args(), my[k], variant="omp")
                ok_p = ok_p and bool(np.array_equal(paths[k], ref["path"]))
                ok_l = ok_l and float(lls[k]) == ref["loglik"]
            parity = {"sequences": len(pick), "path_equal": ok_p, "loglik_equal": ok_l,
                      "oracle": "IEEE OpenMP restatement of src/hsmm.cu:376-600",
                      "oracle_s": round(time.perf_counter() - t0, 1)}
        line = {
            "metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": wname, "n_seq": w["n_seq"], "n_states": N, "max_dur": D, "symbols": w["M"],
                       "lengths": f"log-uniform [{w['lo']:g},{w['hi']:g}]", "total_steps": int(lens.sum()),
                       "l2": "flushed between steps (256 MiB write)", "parallelism": f"sequence shards x{ws}",
                       "form": "batched, one persistent launch", "cta_threads": model.batch_threads(),
                       "cta_grid": model.batch_grid()},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None, "kernel": "cta_decode_kernel", "kernel_ms": kmean,
                         "algo_bytes_per_launch": ALGO_BYTES_PER_CELL * cells, "peak_source": peak_kind},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "cells/s", "h2d_bytes_per_step": int(lens.sum()) * 4 + 8 * (len(my) + 1),
                    "d2h_bytes_per_step": int(lens.sum()) * 4 + 8 * len(my) + 4 * len(my),
                    "ms_per_step": 1e3 * sum(e2e_s) / len(e2e_s)},
            "plain_loop": {"value": plain, "unit": "cells/s", "sample_sequences": int(len(samp)),
                           "speedup_batched_vs_plain": value / plain},
            "gpu_launches": launches, "clocks": clk, "consistent": same, "parity": parity,
        }
        print(json.dumps(line), flush=True)
    model.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def sum_over_ranks(x: float, ws: int) -> float:
    if ws == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="single_N75_D5000_T1e6")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the oracle check of the workload's T-prefix")
    ap.add_argument("--no-e2e", action="store_true",
                    help="skip the host-buffer (drop-in call) measurement: long stress workloads")
    ap.add_argument("--T", type=int, default=0, help="override the sequence length (profiling runs)")
    ap.add_argument("--n-seq", type=int, default=0, help="batched workload: override the number of sequences "
                                                         "(profiling runs)")
    ap.add_argument("--loads", default="", help="served workload: comma-separated fractions of the capacity "
                                                "('none': capacity only)")
    ap.add_argument("--max-inflight", type=int, default=64, help="served workload: requests in flight at most")
    ap.add_argument("--requests", type=int, default=0, help="served workload: number of requests per rate")
    ap.add_argument("--capacity-requests", type=int, default=1000,
                    help="served workload: requests in the burst that measures the capacity")
    args = ap.parse_args()
    w = dict(WORKLOADS[args.workload])
    if args.T:
        w["T"] = args.T
    if args.n_seq:
        w["n_seq"] = args.n_seq
    if args.requests:
        w["n_req"] = args.requests
    if w.get("kind") == "served":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no served form; its arm is measured on the single-sequence workload"}))
            return 0
        return run_served(args, w, args.workload)
    if w.get("kind") == "fb":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference arm is measured on the "
                              "single-sequence decode workload"}))
            return 0
        return run_fb(args, w, args.workload)
    if w.get("kind") == "batch":
        if args.impl == "reference":
            return run_reference_batch(args, w, args.workload)
        return run_batch(args, w, args.workload)
    if args.impl == "reference":
        return run_reference(args, w, args.workload)
    return run_ours(args, w, args.workload)


if __name__ == "__main__":
    sys.exit(main())
