"""Drop-in replacement for the reference's `tensor_viterbi/viterbi/native.py`
CUDA backend (native.py:67-81 there), backed by the GB300 decoder.

`decode_tensor_viterbi_cuda(n_states, trans_mat, emission_probs,
duration_probs_linear, start_probs, duration_probs, obs_seq)` keeps the
reference signature, argument meaning and layouts (src/bindings.cpp:19-32):
log-space (N,N) transitions indexed [to j][from i], (O,N) emissions, (D,N)
linear and log duration pmfs, (N,) start, 0-based observations (any numeric
dtype, cast like the binding's forcecast).  It returns a fresh int32 (T,)
path that equals the reference C++ backend's path.

`configure(system, toolchain)` is kept for callers such as the reference
benchmark app: the arguments are accepted and ignored, and it loads the GB300
library.  As in the reference, decoding before `configure` raises
RuntimeError.  The C++ and OpenMP CPU backends are not part of this build;
their entry points raise RuntimeError like an absent backend does in the
reference (native.py:77-79).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

_native = None
_sys_name: str = ""


def configure(system: str = "", toolchain: str = "") -> None:
    """Load the GB300 decoder library.  `system`/`toolchain` are accepted for
    compatibility with the reference's per-system builds and ignored."""
    global _native, _sys_name
    _sys_name = f"{system}/{toolchain}"
    try:
        _native = _lib.lib()
    except OSError as e:  # pragma: no cover - loader failure
        raise RuntimeError(f"[native] Could not load the GB300 decoder library: {e}") from e


def _ensure_configured() -> None:
    if _native is None:
        raise RuntimeError(
            "[native] Native extension not loaded.\n"
            "Call tensor_viterbi.viterbi.native.configure(system, toolchain) first."
        )


def _f64(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=np.float64))


def _obs_i32(x) -> np.ndarray:
    a = np.asarray(x)
    if a.dtype != np.int32:
        a = a.astype(np.int32)
    return np.ascontiguousarray(a.reshape(-1))


def _model_arrays(n_states, trans_mat, emission_probs, duration_probs_linear, start_probs, duration_probs):
    N = int(n_states)
    tm = _f64(trans_mat)
    ep = _f64(emission_probs)
    dl = _f64(duration_probs_linear)
    sp = _f64(start_probs).reshape(-1)
    dp = _f64(duration_probs)
    if ep.ndim != 2 or dp.ndim != 2:
        raise ValueError("[native] emission_probs and duration_probs must be 2-D")
    O, D = ep.shape[0], dp.shape[0]
    if tm.shape != (N, N):
        raise ValueError(f"[native] trans_mat has shape {tm.shape}, expected ({N}, {N})")
    if ep.shape != (O, N):
        raise ValueError(f"[native] emission_probs has shape {ep.shape}, expected (O, {N})")
    if dp.shape != (D, N):
        raise ValueError(f"[native] duration_probs has shape {dp.shape}, expected (D, {N})")
    if dl.shape != (D, N):
        raise ValueError(f"[native] duration_probs_linear has shape {dl.shape}, expected ({D}, {N})")
    if sp.shape != (N,):
        raise ValueError(f"[native] start_probs has shape {sp.shape}, expected ({N},)")
    return N, O, D, tm, ep, dl, sp, dp


class Model:
    """A device-resident HSMM (the tables the reference uploads on every call,
    src/hsmm.cu:173-201, uploaded once).  Reuse it to decode many sequences."""

    def __init__(self, n_states, trans_mat, emission_probs, duration_probs_linear, start_probs, duration_probs):
        L = _lib.lib()
        N, O, D, tm, ep, dl, sp, dp = _model_arrays(
            n_states, trans_mat, emission_probs, duration_probs_linear, start_probs, duration_probs)
        self.N, self.O, self.D = N, O, D
        h = C.c_void_p()
        _lib.check(L.tv_model_create(N, O, D, _lib.dptr(tm), _lib.dptr(ep), _lib.dptr(dl),
                                     _lib.dptr(sp), _lib.dptr(dp), C.byref(h)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.lib().tv_model_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def decode(self, obs_seq, return_loglik: bool = False):
        """Decode one sequence (host arrays in and out, synchronous)."""
        obs = _obs_i32(obs_seq)
        T = obs.size
        path = np.empty(T, dtype=np.int32)
        ll = np.zeros(1, dtype=np.float64)
        _lib.check(_lib.lib().tv_decode(self._h, _lib.iptr(obs), T, _lib.iptr(path), _lib.dptr(ll)))
        return (path, float(ll[0])) if return_loglik else path

    def decode_batch(self, sequences, return_loglik: bool = False):
        """Decode many sequences of any lengths in one persistent launch."""
        seqs = [_obs_i32(s) for s in sequences]
        off = np.zeros(len(seqs) + 1, dtype=np.int64)
        off[1:] = np.cumsum([s.size for s in seqs])
        cat = np.ascontiguousarray(np.concatenate(seqs)) if seqs else np.zeros(0, np.int32)
        out = np.empty(int(off[-1]), dtype=np.int32)
        ll = np.zeros(len(seqs), dtype=np.float64)
        _lib.check(_lib.lib().tv_decode_batch(self._h, len(seqs), _lib.lptr(off), _lib.iptr(cat),
                                              _lib.iptr(out), _lib.dptr(ll)))
        paths = [out[off[k]:off[k + 1]] for k in range(len(seqs))]
        return (paths, ll) if return_loglik else paths

    def decode_device(self, obs_dev_ptr: int, T: int, path_dev_ptr: int, loglik_dev_ptr: int = 0,
                      stream: int = 0) -> None:
        """Asynchronous decode of device-resident observations (raw device
        pointers, e.g. torch `data_ptr()`), on `stream` (a cudaStream_t)."""
        _lib.check(_lib.lib().tv_decode_device(self._h, C.c_void_p(obs_dev_ptr), int(T),
                                               C.c_void_p(path_dev_ptr), C.c_void_p(loglik_dev_ptr or None),
                                               C.c_void_p(stream or None)))

    def decode_batch_device(self, offsets: np.ndarray, obs_dev_ptr: int, path_dev_ptr: int,
                            loglik_dev_ptr: int = 0, stream: int = 0) -> None:
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        _lib.check(_lib.lib().tv_decode_batch_device(self._h, off.size - 1, _lib.lptr(off),
                                                     C.c_void_p(obs_dev_ptr), C.c_void_p(path_dev_ptr),
                                                     C.c_void_p(loglik_dev_ptr or None),
                                                     C.c_void_p(stream or None)))

    def decode_device_static(self, obs_dev_ptr: int, T: int, path_dev_ptr: int, loglik_dev_ptr: int = 0,
                             status_dev_ptr: int = 0, stream: int = 0) -> None:
        """Like decode_device, but allocates no device memory: for callers
        that must not call cudaMalloc while decoding (inside a CUDA graph
        capture, in a stream callback, in a latency-critical loop, or under a
        memory pool reserved up front).  Scratch comes from a fixed array in
        the library (TV_STATIC_SCRATCH_BYTES, held by every GPU that uses the
        library); problems that do not fit raise ValueError.  The first call
        on a device does a one-time set-up and should come before any stream
        capture.  All calls share the array: calls that overlap on the GPU
        race, so serialise them.  status_dev_ptr (optional, device int)
        receives 0 or a TV_* code."""
        _lib.check(_lib.lib().tv_decode_device_static(
            self._h, C.c_void_p(obs_dev_ptr), int(T), C.c_void_p(path_dev_ptr), C.c_void_p(loglik_dev_ptr or None),
            C.c_void_p(status_dev_ptr or None), C.c_void_p(stream or None)))

    def drop_partial(self, step: int, segment: int = 0) -> None:
        """Test-only failure injection: the next grid decode loses the worker
        partial message of `step` for worker segment `segment`, and returns
        TV_ETIMEOUT (RuntimeError) once the bounded wait for it runs out."""
        _lib.check(_lib.lib().tv_model_drop_partial(self._h, int(step), int(segment)))

    def last_launches(self) -> int:
        return int(_lib.lib().tv_model_last_launches(self._h))

    def set_path(self, path: str = "auto", grid_ctas: int = 0) -> None:
        """Kernel choice for single-sequence decodes: 'auto', 'cta' (one CTA,
        window in its shared memory), 'grid' (whole-GPU persistent grid) or
        'grid-l2' (the grid with its window in global memory, as used when the
        window does not fit the workers' shared memory); grid_ctas > 0 caps
        the grid size.  Results are identical."""
        code = {"auto": _lib.TV_PATH_AUTO, "cta": _lib.TV_PATH_CTA, "grid": _lib.TV_PATH_GRID,
                "grid-l2": _lib.TV_PATH_GRID_L2}[path]
        _lib.check(_lib.lib().tv_model_set_path(self._h, code, int(grid_ctas)))

    def set_timing(self, enable: bool = True) -> None:
        """Bracket the main decode kernel with CUDA events on its stream."""
        _lib.check(_lib.lib().tv_model_set_timing(self._h, 1 if enable else 0))

    def kernel_ms(self) -> float:
        """Main-kernel time of the most recent decode (waits for it); < 0 if
        timing was off."""
        return float(_lib.lib().tv_model_kernel_ms(self._h))

    def last_path(self) -> str:
        return {_lib.TV_PATH_CTA: "cta", _lib.TV_PATH_GRID: "grid"}.get(
            int(_lib.lib().tv_model_last_path(self._h)), "none")

    def batch_threads(self) -> int:
        """Threads per CTA of the most recent batched decode (the autotuned
        shape), 0 before any."""
        return int(_lib.lib().tv_model_batch_threads(self._h))

    def batch_grid(self) -> int:
        """CTAs of the most recent batched decode, 0 before any."""
        return int(_lib.lib().tv_model_batch_grid(self._h))


class GaussianModel(Model):
    """A model whose emissions are Gaussian per state: the (T x N)
    log-likelihood table of the float64 observations x is built on the device
    (no reference counterpart; the reference decodes a discrete table, and the
    same decode runs here on the per-timestep table with obs = 0..T-1)."""

    def __init__(self, n_states, trans_mat, duration_probs_linear, start_probs, duration_probs, x, mean, sd):
        L = _lib.lib()
        N = int(n_states)
        tm, dl, sp, dp = _f64(trans_mat), _f64(duration_probs_linear), _f64(start_probs).reshape(-1), _f64(duration_probs)
        xs, mu, sdv = _f64(x).reshape(-1), _f64(mean).reshape(-1), _f64(sd).reshape(-1)
        if tm.shape != (N, N) or dp.ndim != 2 or dp.shape[1] != N or dl.shape != dp.shape or sp.shape != (N,):
            raise ValueError("[native] model table shapes do not match n_states")
        if mu.shape != (N,) or sdv.shape != (N,):
            raise ValueError("[native] mean and sd must have n_states entries")
        self.N, self.O, self.D, self.T = N, xs.size, dp.shape[0], xs.size
        h = C.c_void_p()
        _lib.check(L.tv_model_create_gaussian(N, self.D, xs.size, _lib.dptr(tm), _lib.dptr(dl), _lib.dptr(sp),
                                              _lib.dptr(dp), _lib.dptr(xs), _lib.dptr(mu), _lib.dptr(sdv),
                                              C.byref(h)))
        self._h = h

    def decode(self, obs_seq=None, return_loglik: bool = False):
        """Decode the model's own observations (emission row t = x_t)."""
        return super().decode(np.arange(self.T, dtype=np.int32) if obs_seq is None else obs_seq, return_loglik)


def gaussian_loglik_device(x_dev_ptr: int, T: int, mean, sd, table_dev_ptr: int, stream: int = 0) -> None:
    """Device front-end: table (T x N, device) = log N(x_t; mean_j, sd_j) for
    the T float64 observations at x_dev_ptr; asynchronous on `stream`."""
    mu, sdv = _f64(mean).reshape(-1), _f64(sd).reshape(-1)
    _lib.check(_lib.lib().tv_gaussian_loglik(C.c_void_p(x_dev_ptr), int(T), mu.size, _lib.dptr(mu), _lib.dptr(sdv),
                                             C.c_void_p(table_dev_ptr), C.c_void_p(stream or None)))


class Server:
    """Decode server: continuous batching of independent requests, each with
    its own model (no reference counterpart).  A native scheduler thread
    admits requests in arrival order while the device-memory budget allows and
    runs each on its own stream, so they overlap on the GPU; a result is the
    one the request gives decoded alone.  submit()/submit_gaussian() copy the
    inputs and return a ticket; poll() returns None while pending, else
    (path, loglik, latency_ms, queue_ms); wait() blocks."""

    def __init__(self, budget_bytes: int = 0, max_inflight: int = 64):
        L = _lib.lib()
        h = L.tv_server_create(int(budget_bytes), int(max_inflight))
        if not h:
            raise RuntimeError("[native] " + L.tv_last_error().decode(errors="replace"))
        self._h = C.c_void_p(h)
        self._T = {}

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.lib().tv_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, n_states, trans_mat, emission_probs, duration_probs_linear, start_probs, duration_probs,
               obs_seq) -> int:
        N, O, D, tm, ep, dl, sp, dp = _model_arrays(
            n_states, trans_mat, emission_probs, duration_probs_linear, start_probs, duration_probs)
        obs = _obs_i32(obs_seq)
        t = _lib.lib().tv_server_submit(self._h, N, O, D, obs.size, _lib.dptr(tm), _lib.dptr(ep), _lib.dptr(dl),
                                        _lib.dptr(sp), _lib.dptr(dp), _lib.iptr(obs))
        if t < 0:
            _lib.check(int(t))
        self._T[t] = obs.size
        return int(t)

    def submit_gaussian(self, n_states, trans_mat, duration_probs_linear, start_probs, duration_probs, x, mean,
                        sd) -> int:
        N = int(n_states)
        tm, dl, sp, dp = _f64(trans_mat), _f64(duration_probs_linear), _f64(start_probs).reshape(-1), _f64(duration_probs)
        xs, mu, sdv = _f64(x).reshape(-1), _f64(mean).reshape(-1), _f64(sd).reshape(-1)
        if tm.shape != (N, N) or dp.ndim != 2 or dp.shape[1] != N or mu.shape != (N,) or sdv.shape != (N,):
            raise ValueError("[native] Gaussian request shapes do not match n_states")
        t = _lib.lib().tv_server_submit_gaussian(self._h, N, dp.shape[0], xs.size, _lib.dptr(tm), _lib.dptr(dl),
                                                 _lib.dptr(sp), _lib.dptr(dp), _lib.dptr(xs), _lib.dptr(mu),
                                                 _lib.dptr(sdv))
        if t < 0:
            _lib.check(int(t))
        self._T[t] = xs.size
        return int(t)

    def _take(self, ticket: int, block: bool):
        T = self._T[ticket]
        path = np.empty(T, dtype=np.int32)
        ll = np.zeros(1, dtype=np.float64)
        lat = np.zeros(2, dtype=np.float64)
        fn = _lib.lib().tv_server_wait if block else _lib.lib().tv_server_poll
        rc = fn(self._h, int(ticket), _lib.iptr(path), _lib.dptr(ll), _lib.dptr(lat))
        if rc == 0:
            return None
        del self._T[ticket]
        if rc < 0:
            _lib.check(rc)
        return path, float(ll[0]), float(lat[0]), float(lat[1])

    def poll(self, ticket: int):
        return self._take(ticket, False)

    def wait(self, ticket: int):
        return self._take(ticket, True)

    def stats(self) -> dict:
        out = np.zeros(8, dtype=np.int64)
        _lib.check(_lib.lib().tv_server_stats(self._h, _lib.lptr(out)))
        keys = ["admitted", "completed", "failed", "running", "pending", "bytes_in_use", "peak_bytes", "budget"]
        return dict(zip(keys, map(int, out)))


def decode_tensor_viterbi_cuda_loglik(n_states, trans_mat, emission_probs, duration_probs_linear,
                                      start_probs, duration_probs, obs_seq):
    """Like decode_tensor_viterbi_cuda, also returning the path log-likelihood."""
    _ensure_configured()
    N, O, D, tm, ep, dl, sp, dp = _model_arrays(
        n_states, trans_mat, emission_probs, duration_probs_linear, start_probs, duration_probs)
    obs = _obs_i32(obs_seq)
    path = np.empty(obs.size, dtype=np.int32)
    ll = np.zeros(1, dtype=np.float64)
    _lib.check(_native.tv_decode_tensor_viterbi_cuda(
        N, O, D, obs.size, _lib.dptr(tm), _lib.dptr(ep), _lib.dptr(dl), _lib.dptr(sp), _lib.dptr(dp),
        _lib.iptr(obs), _lib.iptr(path), _lib.dptr(ll)))
    return path, float(ll[0])


def decode_tensor_viterbi_cuda(
        n_states,
        trans_mat,
        emission_probs,
        duration_probs_linear,
        start_probs,
        duration_probs,
        obs_seq,
) -> np.ndarray:
    return decode_tensor_viterbi_cuda_loglik(n_states, trans_mat, emission_probs, duration_probs_linear,
                                             start_probs, duration_probs, obs_seq)[0]


def decode_tensor_viterbi_cpp(n_states, trans_mat, emission_probs, duration_probs_linear, start_probs,
                              duration_probs, obs_seq) -> np.ndarray:
    _ensure_configured()
    raise RuntimeError("C++ backend not available in this build.")


def decode_tensor_viterbi_omp(n_states, trans_mat, emission_probs, duration_probs_linear, start_probs,
                              duration_probs, obs_seq) -> np.ndarray:
    _ensure_configured()
    raise RuntimeError("OMP backend not available in this build.")


def step_floor(n_states: int, max_dur: int, steps: int = 20000) -> dict:
    """Per-step latency floor of the grid decoder for a shape (diagnostics):
    the head's critical chain alone on one SM, and one cross-SM tagged round
    trip.  Returns clocks and microseconds per step and per round trip."""
    out = np.zeros(7, dtype=np.float64)
    _lib.check(_lib.lib().tv_step_floor(int(n_states), int(max_dur), int(steps), _lib.dptr(out)))
    return {"chain_clocks_per_step": float(out[0]), "chain_us_per_step": float(out[1]),
            "roundtrip_clocks": float(out[2]), "roundtrip_us": float(out[3]), "matvec_split": bool(out[4]),
            "roundtrip_sms": [int(out[5]), int(out[6])]}


def fp64_peak() -> dict:
    """One SM's FP64 unit (diagnostics): issue rate with eight warps of
    independent fused multiply-add chains, that SM's FLOP/s, the SM clock over
    the run, and the dependent latency of one FP64 instruction."""
    out = np.zeros(4, dtype=np.float64)
    _lib.check(_lib.lib().tv_fp64_peak(_lib.dptr(out)))
    return {"warp_insts_per_clock": float(out[0]), "flops": float(out[1]), "sm_mhz": float(out[2]),
            "dependent_clocks": float(out[3])}


def fb_last_kernel_ms() -> float:
    """Device time of this thread's last forward_backward kernel (ms)."""
    return float(_lib.lib().tv_fb_last_kernel_ms())


def forward_backward(censoring, d, p, pi, pdf) -> dict:
    """The forward-backward E step of HSMM training on the GPU (tv_fb), with
    hsmmlearn's _fb_impl arguments and layouts (hsmmlearn/hsmmlearn/base.pyx):
    censoring 0 or 1, d (J, M) duration pmf, p (J, J) [from][to], pi (J),
    pdf (J, tau) likelihoods.  Returns dict(err, F, L, G, L1, N, Norm, eta):
    err = 1 where the reference reports a non-positive normaliser or forward
    variable, as its _fb_impl does; other failures raise."""
    d = np.ascontiguousarray(d, dtype=np.float64)
    p = np.ascontiguousarray(p, dtype=np.float64)
    pi = np.ascontiguousarray(pi, dtype=np.float64).reshape(-1)
    pdf = np.ascontiguousarray(pdf, dtype=np.float64)
    J, M = d.shape
    tau = pdf.shape[1]
    if p.shape != (J, J) or pi.shape != (J,) or pdf.shape[0] != J:
        raise ValueError("forward_backward: shapes must be d (J, M), p (J, J), pi (J), pdf (J, tau)")
    out = {k: np.zeros((J, tau)) for k in ("F", "L", "G", "L1", "Norm")}
    out["N"] = np.zeros(tau)
    out["eta"] = np.zeros((J, M))
    rc = _lib.lib().tv_fb(int(censoring), tau, J, M, _lib.dptr(d), _lib.dptr(p), _lib.dptr(pi), _lib.dptr(pdf),
                          *(_lib.dptr(out[k]) for k in ("F", "L", "G", "L1", "N", "Norm", "eta")))
    if rc == _lib.TV_ENONPOS:
        out["err"] = 1
        return out
    _lib.check(rc)
    out["err"] = 0
    return out
