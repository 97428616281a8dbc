"""HSMM training step on the GPU: the forward-backward kernel (tv_fb) against
the reference's own outputs (tests/golden/fb/) and the oracle, and the EM fit
with the GPU E step against the reference's HSMMModel.fit.  Tolerance: the
kernel associates some products and sums differently from the reference
(rings of likelihood-ratio products, lane-parallel sums over durations), so
every array agrees within 1e-11 of its largest entry, and each entry above
1e-6 of the largest within 1e-7 relative (the smoothed probabilities
L = L1 + L[t+1] - G*S cancel, which magnifies the rounding of small entries,
in the reference and here alike); the fitted parameters agree to 1e-8
relative or 1e-12 absolute."""
import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle as orc
from test_fb import FB, _model, check_fit, em_cases, fb_cases

pytestmark = pytest.mark.gpu

NORM_TOL = 1e-11
ENTRY_RTOL = 1e-7


def _close(got, want, name):
    big = float(np.abs(want).max()) if want.size else 0.0
    diff = np.abs(got - want)
    assert float(diff.max(initial=0.0)) <= NORM_TOL * big + 1e-300, (name, float(diff.max()) / big)
    scale = np.maximum(np.abs(want), big * 1e-6 + 1e-300)
    assert float((diff / scale).max(initial=0.0)) <= ENTRY_RTOL, (name, float((diff / scale).max()))


@pytest.mark.parametrize("name", fb_cases())
def test_gpu_forward_backward_matches_the_reference(tvlib, name):
    z = np.load(FB / f"{name}.npz")
    r = tvlib.forward_backward(int(z["censoring"]), z["d"], z["p"], z["pi"], z["pdf"])
    assert r["err"] == int(z["err"])
    for k in orc.FB_KEYS:
        _close(r[k], z[k], k)


# J <= 32 and M <= 128: the window in registers (M = 5, 100, 128: one, four
# partial and four full blocks of 32 durations, J = 32 a full CTA); M > 128:
# the shared-memory rings (M = 129, 200, 333) or, past shared memory, global
# ones (J = 32, M = 300); J > 32: the general kernel.
@pytest.mark.parametrize("J,M,tau,cens", [(20, 200, 3000, 1), (7, 333, 1200, 0), (40, 64, 2000, 1), (3, 5, 4000, 1),
                                          (12, 128, 1500, 1), (32, 100, 700, 0), (32, 129, 800, 1),
                                          (32, 300, 900, 1)])
def test_gpu_forward_backward_matches_the_oracle_on_random_models(tvlib, J, M, tau, cens):
    rng = np.random.default_rng(J * 1000 + M)
    p = rng.dirichlet(np.ones(J), size=J)
    d = rng.dirichlet(np.ones(M) * 1.5, size=J)
    pi = rng.dirichlet(np.ones(J))
    pdf = rng.uniform(0.01, 1.0, size=(J, tau))
    want = orc.forward_backward(cens, d, p, pi, pdf)
    got = tvlib.forward_backward(cens, d, p, pi, pdf)
    assert got["err"] == want["err"] == 0
    for k in orc.FB_KEYS:
        _close(got[k], want[k], k)


@pytest.mark.parametrize("J,M", [(6, 40), (24, 150)])
def test_gpu_forward_backward_over_a_wide_likelihood_range(tvlib, J, M):
    """Likelihoods from 1e-250 to 1: window sums whose terms span hundreds of
    binary orders (the integer-aligned reductions drop the smallest)."""
    rng = np.random.default_rng(J + 7 * M)
    tau = 900
    p = rng.dirichlet(np.ones(J), size=J)
    d = rng.dirichlet(np.ones(M), size=J)
    pi = rng.dirichlet(np.ones(J))
    pdf = 10.0 ** rng.uniform(-250.0, 0.0, size=(J, tau))
    want = orc.forward_backward(1, d, p, pi, pdf)
    got = tvlib.forward_backward(1, d, p, pi, pdf)
    assert got["err"] == want["err"] == 0
    for k in orc.FB_KEYS:
        _close(got[k], want[k], k)


def test_fp64_probe_and_kernel_timing(tvlib):
    """The FP64 probe that sets the forward-backward roofline returns a
    plausible unit (a warp instruction per few to a hundred clocks, a
    dependent latency of a few to a thousand clocks), and the kernel's own
    event time is recorded."""
    pk = tvlib.fp64_peak()
    assert 0.005 < pk["warp_insts_per_clock"] <= 4.0
    assert 4.0 <= pk["dependent_clocks"] <= 1000.0
    assert pk["flops"] > 1e8 and 500.0 < pk["sm_mhz"] < 5000.0
    z = np.load(FB / "fb_J8_M60_T800_c1.npz")
    tvlib.forward_backward(1, z["d"], z["p"], z["pi"], z["pdf"])
    assert tvlib.fb_last_kernel_ms() > 0.0


def test_gpu_forward_backward_reports_a_zero_normaliser(tvlib):
    z = np.load(FB / "fb_J3_M20_T300_c1.npz")
    pdf = z["pdf"].copy()
    pdf[:, 7] = 0.0
    assert tvlib.forward_backward(1, z["d"], z["p"], z["pi"], pdf)["err"] == 1
    # and the next call is unaffected
    r = tvlib.forward_backward(1, z["d"], z["p"], z["pi"], z["pdf"])
    assert r["err"] == 0
    _close(r["N"], z["N"], "N")


def test_gpu_forward_backward_refuses_left_censoring(tvlib):
    z = np.load(FB / "fb_J3_M20_T300_c1.npz")
    with pytest.raises(ValueError, match="censoring"):
        tvlib.forward_backward(2, z["d"], z["p"], z["pi"], z["pdf"])


@pytest.mark.parametrize("name", em_cases())
def test_gpu_em_fit_matches_the_reference_fit(tvlib, name):
    z = np.load(FB / f"{name}.npz")
    model = _model(z)
    conv, llh = model.fit(z["obs"], max_iter=int(z["max_iter"]), censoring=bool(z["censoring"]))
    check_fit(model, z, conv, llh, rtol=1e-8, atol=1e-12)
