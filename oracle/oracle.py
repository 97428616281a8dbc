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
        if hasattr(h, "tvo_fb"):
            h.tvo_fb.restype = C.c_int
            h.tvo_fb.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int] + [_dp] * 11
        if hasattr(h, "tvo_decode_cuda"):
            h.tvo_decode_cuda.restype = C.c_int
            h.tvo_decode_cuda.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, _ip, C.c_int,
                                          _dp, C.c_int, _ip, _dp, _dp]
            h.tvo_lin_suffix.restype = None
            h.tvo_lin_suffix.argtypes = [C.c_int, C.c_int, _dp, _dp]
            h.tvo_block_scan.restype = None
            h.tvo_block_scan.argtypes = [_dp, C.c_int, _dp]
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


# Flag bits of decode_cuda_semantics: the reference CUDA backend's four
# differences from its C++ decoder (tv_oracle_cuda.c).
CU_INIT_SCAN, CU_WINDOW, CU_TAIL, CU_ITREE = 1, 2, 4, 8
CU_ALL = 15
CU_NAMES = {CU_INIT_SCAN: "init scan", CU_WINDOW: "window roll", CU_TAIL: "linear-survival tail",
            CU_ITREE: "i-tree argmax"}


def lin_suffix(n_states, duration_probs_linear):
    """Linear duration suffix sums in kernel_initialization's block-scan
    association, (N, D) [j][d]."""
    h = _load("liboracle.so")
    lin = _f64(duration_probs_linear)
    D = lin.shape[0]
    out = np.empty((int(n_states), D), dtype=np.float64)
    h.tvo_lin_suffix(int(n_states), D, lin.ctypes.data_as(_dp), out.ctypes.data_as(_dp))
    return out


def block_scan(x):
    """Inclusive prefix sums of x in kernel_initialization's association."""
    h = _load("liboracle.so")
    x = _f64(x).reshape(-1)
    out = np.empty_like(x)
    h.tvo_block_scan(x.ctypes.data_as(_dp), x.size, out.ctypes.data_as(_dp))
    return out


def decode_cuda_semantics(n_states, trans_mat, emission_probs, duration_probs_linear, start_probs,
                          duration_probs, obs_seq, flags: int = CU_ALL, log_suffix=None, nthreads: int = 0):
    """The reference CUDA backend's values with the differences in `flags`
    (CU_* bits) and the C++ decoder's rules elsewhere (flags = 0 is the C++
    decoder).  log_suffix (N, D) replaces the C library's log of lin_suffix()
    in the tail (the device's log).  Returns dict(path, loglik, final)."""
    h = _load("liboracle.so")
    N = int(n_states)
    tm, ep, lin = _f64(trans_mat), _f64(emission_probs), _f64(duration_probs_linear)
    sp, dp = _f64(start_probs).reshape(-1), _f64(duration_probs)
    obs = np.ascontiguousarray(np.asarray(obs_seq).astype(np.int32).reshape(-1))
    O, D, T = ep.shape[0], dp.shape[0], obs.size
    ls = None if log_suffix is None else _f64(log_suffix)
    path = np.empty(T, dtype=np.int32)
    ll = np.zeros(1, dtype=np.float64)
    final = np.empty(N, dtype=np.float64)
    rc = h.tvo_decode_cuda(N, O, D, T, tm.ctypes.data_as(_dp), ep.ctypes.data_as(_dp), lin.ctypes.data_as(_dp),
                           sp.ctypes.data_as(_dp), dp.ctypes.data_as(_dp), obs.ctypes.data_as(_ip), int(flags),
                           None if ls is None else ls.ctypes.data_as(_dp), int(nthreads),
                           path.ctypes.data_as(_ip), ll.ctypes.data_as(_dp), final.ctypes.data_as(_dp))
    if rc != 0:
        raise ValueError(f"oracle: {STATUS.get(rc, rc)}")
    return dict(path=path, loglik=float(ll[0]), final=final)


def ref_cuda_files():
    """(cubin, names) of the reference's CUDA kernels built by
    oracle/build_ref.sh, or None when they are absent."""
    d = HERE / "_ref" / "cuda"
    cubin, names = d / "kernels_sm103a.cubin", d / "kernels.names"
    return (cubin, names) if cubin.exists() and names.exists() else None


_ref_cuda_lib = None


def _ref_cuda():
    global _ref_cuda_lib
    with _lock:
        if _ref_cuda_lib is None:
            path = HERE / "libref_cuda.so"
            if not path.exists():
                build()
            h = C.CDLL(str(path))
            h.tvr_decode.restype = C.c_int
            h.tvr_decode.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp,
                                     _dp, _ip, _ip, _dp, _dp, _dp]
            h.tvr_last_error.restype = C.c_char_p
            _ref_cuda_lib = h
    return _ref_cuda_lib


def ref_cuda_decode(n_states, trans_mat, emission_probs, duration_probs_linear, start_probs, duration_probs,
                    obs_seq):
    """The reference's own CUDA kernels on this GPU (oracle/ref_cuda.c drives
    them as src/hsmm.cu:604-791 does).  Returns dict(path, loglik, final,
    ms_call, ms_kernels)."""
    files = ref_cuda_files()
    if files is None:
        raise RuntimeError("the reference CUDA kernels are not built (oracle/build_ref.sh on a host with the checkout)")
    h = _ref_cuda()
    N = int(n_states)
    tm, ep, lin = _f64(trans_mat), _f64(emission_probs), _f64(duration_probs_linear)
    sp, dp = _f64(start_probs).reshape(-1), _f64(duration_probs)
    obs = np.ascontiguousarray(np.asarray(obs_seq).astype(np.int32).reshape(-1))
    O, D, T = ep.shape[0], dp.shape[0], obs.size
    path = np.empty(T, dtype=np.int32)
    ll = np.zeros(1, dtype=np.float64)
    final = np.empty(N, dtype=np.float64)
    ms = np.zeros(2, dtype=np.float64)
    rc = h.tvr_decode(str(files[0]).encode(), str(files[1]).encode(), N, O, D, T, tm.ctypes.data_as(_dp),
                      ep.ctypes.data_as(_dp), lin.ctypes.data_as(_dp), sp.ctypes.data_as(_dp),
                      dp.ctypes.data_as(_dp), obs.ctypes.data_as(_ip), path.ctypes.data_as(_ip),
                      ll.ctypes.data_as(_dp), final.ctypes.data_as(_dp), ms.ctypes.data_as(_dp))
    if rc != 0:
        raise RuntimeError(f"reference CUDA decode failed ({rc}): {h.tvr_last_error().decode()}")
    return dict(path=path, loglik=float(ll[0]), final=final, ms_call=float(ms[0]), ms_kernels=float(ms[1]))


FB_KEYS = ("F", "L", "G", "L1", "N", "Norm", "eta")


def forward_backward(censoring, d, p, pi, pdf):
    """hsmmlearn's forward-backward (FBImpl.cpp) restated in C: d (J, M)
    duration pmf, p (J, J) [from][to], pi (J), pdf (J, tau) likelihoods.
    Returns dict(err, F, L, G, L1, N, Norm, eta) with hsmmlearn's layouts."""
    h = _load("liboracle.so")
    d, p, pi, pdf = _f64(d), _f64(p), _f64(pi).reshape(-1), _f64(pdf)
    J, M = d.shape
    tau = pdf.shape[1]
    out = {k: np.zeros((J, tau)) for k in ("F", "L", "G", "L1", "Norm")}
    out["N"] = np.zeros(tau)
    out["eta"] = np.zeros((J, M))
    rc = h.tvo_fb(int(censoring), tau, J, M, d.ctypes.data_as(_dp), p.ctypes.data_as(_dp), pi.ctypes.data_as(_dp),
                  pdf.ctypes.data_as(_dp), *(out[k].ctypes.data_as(_dp) for k in FB_KEYS))
    if rc < 0:
        raise ValueError(f"oracle forward-backward: bad argument ({rc})")
    out["err"] = int(rc)
    return out


def reference_hsmmlearn():
    """The reference's hsmmlearn package (its Python modules from the
    checkout, its compiled core from oracle/build_ref.sh), or None where
    either is absent (the GPU host has no checkout)."""
    root = reference_root()
    d = HERE / "_ref" / "hsmmlearn"
    so = sorted(d.glob("base*.so")) if d.exists() else []
    if root is None or not so:
        return None
    if "hsmmlearn.hsmm" in sys.modules:
        return sys.modules["hsmmlearn.hsmm"]
    pkg_dir = root / "hsmmlearn"
    if str(pkg_dir) not in sys.path:
        sys.path.insert(0, str(pkg_dir))
    spec = importlib.util.spec_from_file_location("hsmmlearn.base", str(so[0]))
    base = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(base)
    import hsmmlearn  # noqa: F401  (the package, from the checkout)
    sys.modules["hsmmlearn.base"] = base
    import hsmmlearn.hsmm as hh
    return hh


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
