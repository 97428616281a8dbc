"""The CPU restatement of the reference's CUDA backend (oracle/tv_oracle_cuda.c)
and the committed agreement table of that backend with the reference's C++
decoder (tests/golden/ref_cuda_agreement.json).  CPU only; the reference
kernels themselves are checked against both on the GPU in
test_ref_cuda_gpu.py."""
import json

import numpy as np
import pytest

from conftest import GOLDEN, golden_names, load_golden
from oracle import oracle as orc


@pytest.mark.parametrize("name", golden_names())
def test_no_cuda_difference_selected_is_the_cpp_decoder(name):
    args, z = load_golden(name)
    ref = orc.decode(*args)
    r = orc.decode_cuda_semantics(*args, flags=0)
    np.testing.assert_array_equal(r["path"], z["path_cpp"])
    assert r["loglik"] == ref["loglik"]


@pytest.mark.parametrize("n", [1, 2, 5, 31, 32, 33, 100, 1023, 1024, 1025, 2049, 5000])
def test_block_scan_sums_exactly_on_integers(n):
    x = np.random.default_rng(n).integers(-1000, 1000, size=n).astype(np.float64)
    np.testing.assert_array_equal(orc.block_scan(x), np.cumsum(x))


def test_block_scan_association_on_a_small_block():
    """n = 3: one block of 4 lanes.  Stride 1 gives v1 = x1 + x0 and
    v2 = x2 + x1; stride 2 gives v2 = (x2 + x1) + x0 -- not the oldest-first
    (x0 + x1) + x2, which rounds differently here."""
    x = np.array([1e16, 1.0, 1.0])
    out = orc.block_scan(x)
    assert out[0] == x[0] and out[1] == x[1] + x[0]
    assert out[2] == (x[2] + x[1]) + x[0]
    assert out[2] != (x[0] + x[1]) + x[2]


def test_block_scan_chunks_carry_the_running_offset():
    """n = 1025: a full 1024-lane block and a second chunk of one element,
    which is x[1024] + the first chunk's total (the last warp total)."""
    x = np.random.default_rng(3).random(1025)
    out = orc.block_scan(x)
    assert out[1024] == x[1024] + out[1023]


def test_linear_suffix_is_the_reversed_scan():
    rng = np.random.default_rng(4)
    lin = rng.dirichlet(np.ones(37), size=3).T  # (D, N)
    s = orc.lin_suffix(3, lin)
    for j in range(3):
        np.testing.assert_array_equal(s[j], orc.block_scan(lin[::-1, j])[::-1])
    np.testing.assert_allclose(s[:, 0], 1.0, rtol=1e-12)


def _table():
    return json.loads((GOLDEN / "ref_cuda_agreement.json").read_text())["cases"]


def _small_cases():
    import sys
    from conftest import REPO
    sys.path.insert(0, str(REPO / "tests" / "golden"))
    import make_ref_cuda_table as mk
    return [(n, load_golden(n)[0]) for n in golden_names()] + mk.tie_cases()


@pytest.mark.parametrize("name,args", _small_cases(), ids=[c[0] for c in _small_cases()])
def test_agreement_table_rows_recomputed(name, args):
    """Every row but the long bench-model case, recomputed: the CUDA-semantics
    path digest, its agreement with the C++ decoder and the named causes."""
    import make_ref_cuda_table as mk
    assert mk.row(args) == _table()[name]
