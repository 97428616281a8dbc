"""The C-ABI library: it builds for sm_103a, loads, and exports every entry
point include/tv_gb300.h declares.  No compute calls (CPU only)."""
import ctypes
import re

import numpy as np
import pytest

from conftest import REPO


def declared_functions():
    text = (REPO / "include" / "tv_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tv_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ("tv_decode_tensor_viterbi_cuda", "tv_model_create", "tv_decode", "tv_decode_device",
                     "tv_decode_batch", "tv_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol(tvlib):
    from tensor_viterbi.viterbi import _lib
    h = ctypes.CDLL(str(_lib.LIB_PATH))
    for name in declared_functions():
        assert hasattr(h, name), name
        assert name in _lib.EXPORTS, f"{name} declared in the header but not bound in _lib.EXPORTS"


def test_python_validation_before_device(tvlib):
    from tensor_viterbi.viterbi import native
    N = 3
    tm = np.log(np.full((N, N), 0.5))
    em = np.log(np.full((4, N), 0.25))
    dl = np.full((5, N), 0.2)
    dp = np.log(dl)
    sp = np.log(np.full(N, 1 / 3))
    with pytest.raises(ValueError, match="trans_mat"):
        native.Model(N, tm[:2], em, dl, sp, dp)
    with pytest.raises(ValueError, match="duration_probs_linear"):
        native.Model(N, tm, em, dl[:4], sp, dp)
    bad = em.copy()
    bad[0, 0] = np.nan
    with pytest.raises(ValueError, match="finite"):
        native.Model(N, tm, bad, dl, sp, dp)


def test_cpu_backends_are_absent(tvlib):
    from tensor_viterbi.viterbi import native
    with pytest.raises(RuntimeError, match="not available"):
        native.decode_tensor_viterbi_cpp(1, [[0.0]], [[0.0]], [[1.0]], [0.0], [[0.0]], [0])
    with pytest.raises(RuntimeError, match="not available"):
        native.decode_tensor_viterbi_omp(1, [[0.0]], [[0.0]], [[1.0]], [0.0], [[0.0]], [0])


def test_unconfigured_call_raises_like_reference():
    from tensor_viterbi.viterbi import native
    saved = native._native
    try:
        native._native = None
        with pytest.raises(RuntimeError, match="not loaded"):
            native.decode_tensor_viterbi_cuda(1, [[0.0]], [[0.0]], [[1.0]], [0.0], [[0.0]], [0])
    finally:
        native._native = saved
