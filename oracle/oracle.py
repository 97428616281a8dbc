"""ctypes wrapper of the CPU oracle (tv_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker.  The product never imports it.

Also gives access to the reference's own compiled CPU module when
oracle/build_ref.sh has built it (development host only; the GPU host has no
reference checkout).
"""
from __future__ import annotations

import ctypes as C
import importlib.util
import os
import pathlib
import subprocess
import sys
import threading

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
_lock = threading.Lock()
_libs: dict[str, C.CDLL] = {}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_bp = C.POINTER(C.c_uint8)

STATUS = {0: "ok", -1: "invalid argument", -2: "T < D", -3: "observation out of range", -4: "out of memory"}


def build(quiet: bool = True) -> None:
    """Compile liboracle.so / liboracle_fast.so (make, gcc)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)


def _load(name: str) -> C.CDLL:
    with _lock:
        if name in _libs:
            return _libs[name]
        path = HERE / name
        if not path.exists():
            build()
        h = C.CDLL(str(path))
        h.tvo_decode.restype = C.c_int
        h.tvo_decode.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _ip, C.c_int, C.c_int,
                                 _ip, _dp, _dp, _dp, _ip, _ip, _bp]
        h.tvo_score_segments.restype = C.c_double
        h.tvo_score_segments.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _ip, _ip, _bp]
        h.tvo_survival.restype = None
        h.tvo_survival.argtypes = [C.c_int, C.c_int, _dp, _dp]
        _libs[name] = h
        return h


def _f64(x):
    return np.ascontiguousarray(np.asarray(x, dtype=np.float64))


def decode(n_states, trans_mat, emission_probs, duration_probs_linear, start_probs, duration_probs, obs_seq,
           variant: str = "serial", nthreads: int = 0, tables: bool = False, fast: bool = False):
    """Run the oracle.  Returns dict(path, loglik[, delta, tail, psi_state,
    psi_dur, seg_start]).  variant: 'serial' (src/hsmm.cu:233-373) or 'omp'
    (src/hsmm.cu:376-600).  fast=True uses the -O3 -ffast-math build."""
    h = _load("liboracle_fast.so" if fast else "liboracle.so")
    N = int(n_states)
    tm, ep, sp, dp = _f64(trans_mat), _f64(emission_probs), _f64(start_probs).reshape(-1), _f64(duration_probs)
    obs = np.ascontiguousarray(np.asarray(obs_seq).astype(np.int32).reshape(-1))
    O, D, T = ep.shape[0], dp.shape[0], obs.size
    path = np.empty(T, dtype=np.int32)
    ll = np.zeros(1, dtype=np.float64)
    out = dict(path=path)
    if tables:
        delta = np.empty((T, N), dtype=np.float64)
        tail = np.empty(N, dtype=np.float64)
        ps = np.empty((T, N), dtype=np.int32)
        pdu = np.empty((T, N), dtype=np.int32)
        seg = np.empty(T, dtype=np.uint8)
        ptrs = (delta.ctypes.data_as(_dp), tail.ctypes.data_as(_dp), ps.ctypes.data_as(_ip),
                pdu.ctypes.data_as(_ip), seg.ctypes.data_as(_bp))
        out.update(delta=delta, tail=tail, psi_state=ps, psi_dur=pdu, seg_start=seg)
    else:
        ptrs = (None, None, None, None, None)
    rc = h.tvo_decode(N, O, D, T, tm.ctypes.data_as(_dp), ep.ctypes.data_as(_dp), sp.ctypes.data_as(_dp),
                      dp.ctypes.data_as(_dp), obs.ctypes.data_as(_ip), 1 if variant == "omp" else 0,
                      int(nthreads), path.ctypes.data_as(_ip), ll.ctypes.data_as(_dp), *ptrs)
    if rc != 0:
        raise ValueError(f"oracle: {STATUS.get(rc, rc)}")
    out["loglik"] = float(ll[0])
    return out


def score_segments(n_states, trans_mat, emission_probs, start_probs, duration_probs, obs_seq, path,
                   seg_start) -> float:
    """Long-double score of a decoded segmentation (independent of the
    recursion's association), for the log-likelihood check."""
    h = _load("liboracle.so")
    tm, ep, sp, dp = _f64(trans_mat), _f64(emission_probs), _f64(start_probs).reshape(-1), _f64(duration_probs)
    obs = np.ascontiguousarray(np.asarray(obs_seq).astype(np.int32))
    pth = np.ascontiguousarray(np.asarray(path, dtype=np.int32))
    seg = np.ascontiguousarray(np.asarray(seg_start, dtype=np.uint8))
    return float(h.tvo_score_segments(int(n_states), ep.shape[0], dp.shape[0], obs.size,
                                      tm.ctypes.data_as(_dp), ep.ctypes.data_as(_dp), sp.ctypes.data_as(_dp),
                                      dp.ctypes.data_as(_dp), obs.ctypes.data_as(_ip), pth.ctypes.data_as(_ip),
                                      seg.ctypes.data_as(_bp)))


def reference_module(kind: str = "ieee"):
    """The reference's own compiled `_native` (oracle/build_ref.sh), or None
    when it has not been built here."""
    d = HERE / "_ref" / kind
    so = sorted(d.glob("_native*.so")) if d.exists() else []
    if not so:
        return None
    name = f"_native_ref_{kind}"
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location("_native", str(so[0]))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    sys.modules[name] = mod
    return mod


def reference_root() -> pathlib.Path | None:
    """The reference checkout: $TV_REFERENCE_ROOT, else the root that
    oracle/build_ref.sh recorded when it compiled the reference here; None
    when neither names an existing directory (the GPU host has no checkout)."""
    env = os.environ.get("TV_REFERENCE_ROOT")
    cands = [pathlib.Path(env)] if env else []
    rec = HERE / "_ref" / "ROOT"
    if rec.exists():
        cands.append(pathlib.Path(rec.read_text().strip()))
    for c in cands:
        if (c / "src" / "hsmm.cu").exists():
            return c
    return None


def cpu_count() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:  # pragma: no cover
        return os.cpu_count() or 1
