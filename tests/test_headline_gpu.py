"""Oracle parity at the benchmarked shapes.

The bench's own seeded models, decoded on a T-prefix long enough to reach the
fully rolled window (t > 2D) and compared with the oracle's OpenMP
restatement of the reference decoder (src/hsmm.cu:376-600), bit for bit:
  * N=75, D=5000, M=32 (the single-sequence headline): the grid kernel with
    its window in the workers' shared memory (row-aligned, two workers per
    state) and with the window forced into global memory (L2);
  * N=100, D=1e4, M=64 (the stress shape): the grid kernel with its window in
    L2, in equal-cost chunks that span two states, at one CTA per SM and at
    a smaller grid (other chunk boundaries).
These are the shapes where the certified margin's D^2 term is largest and
where the equal-cost chunking is exercised.  Each oracle run is made once per
session (fixtures in conftest.py) and shared by the plans.
"""
import numpy as np
import pytest


pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["auto", "grid-l2"])
def test_headline_N75_D5000_prefix_equals_oracle(tvlib, c1_case, kind):
    args, ref = c1_case
    with tvlib.Model(*args[:6]) as m:
        m.set_path(kind, 0)
        path, ll = m.decode(args[6], return_loglik=True)
        assert m.last_path() == "grid"
    np.testing.assert_array_equal(path, ref["path"])
    assert ll == ref["loglik"]


@pytest.mark.parametrize("grid_ctas", [0, 120])
def test_stress_N100_D10000_prefix_equals_oracle(tvlib, c4_case, grid_ctas):
    args, ref = c4_case
    with tvlib.Model(*args[:6]) as m:
        m.set_path("auto", grid_ctas)
        path, ll = m.decode(args[6], return_loglik=True)
        assert m.last_path() == "grid"
    np.testing.assert_array_equal(path, ref["path"])
    assert ll == ref["loglik"]
