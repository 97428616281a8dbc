"""HSMM training step on the CPU: the oracle's restatement of hsmmlearn's
forward-backward (oracle/tv_fb_oracle.c) against the reference's own outputs
(tests/golden/fb/, made by tests/golden/make_fb_golden.py), and the EM of
tensor_viterbi.hsmm_em, run with the oracle as its E step, against the
reference's HSMMModel.fit (hsmmlearn/hsmmlearn/hsmm.py:181-305)."""
import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle as orc

FB = GOLDEN / "fb"


def fb_cases():
    return sorted(p.stem for p in FB.glob("fb_*.npz"))


def em_cases():
    return sorted(p.stem for p in FB.glob("em_*.npz"))


@pytest.mark.parametrize("name", fb_cases())
def test_oracle_forward_backward_equals_the_reference_bit_for_bit(name):
    z = np.load(FB / f"{name}.npz")
    r = orc.forward_backward(int(z["censoring"]), z["d"], z["p"], z["pi"], z["pdf"])
    assert r["err"] == int(z["err"])
    for k in orc.FB_KEYS:
        np.testing.assert_array_equal(r[k], z[k], err_msg=k)


def test_oracle_forward_backward_reports_a_zero_normaliser():
    z = np.load(FB / "fb_J3_M20_T300_c1.npz")
    pdf = z["pdf"].copy()
    pdf[:, 7] = 0.0
    assert orc.forward_backward(1, z["d"], z["p"], z["pi"], pdf)["err"] == 1


def _model(z):
    from tensor_viterbi import hsmm_em
    if str(z["kind"]) == "multinomial":
        return hsmm_em.MultinomialHSMM(z["emissions"], z["durations0"], z["tmat0"], startprob=z["startprob0"])
    return hsmm_em.GaussianHSMM(z["means"], z["scales"], z["durations0"], z["tmat0"], startprob=z["startprob0"])


def check_fit(model, z, conv, llh, rtol, atol):
    """Fitted parameters against the reference's: relative rtol, and atol for
    the probabilities near zero (start and duration probabilities floored at
    1e-14 or vanishing), whose relative error is large at any precision."""
    assert conv == bool(z["converged"])
    np.testing.assert_allclose(llh, float(z["llh"]), rtol=rtol)
    np.testing.assert_allclose(model.tmat, z["fit_tmat"], rtol=rtol, atol=atol)
    np.testing.assert_allclose(model.durations, z["fit_durations"], rtol=rtol, atol=atol)
    np.testing.assert_allclose(model.startprob, z["fit_startprob"], rtol=rtol, atol=atol)
    if str(z["kind"]) == "multinomial":
        np.testing.assert_allclose(model.probabilities, z["fit_emissions"], rtol=rtol, atol=atol)
    else:
        np.testing.assert_allclose(model.means, z["fit_means"], rtol=rtol)
        np.testing.assert_allclose(model.scales, z["fit_scales"], rtol=rtol)


@pytest.mark.parametrize("name", em_cases())
def test_em_with_the_oracle_e_step_equals_the_reference_fit(name):
    z = np.load(FB / f"{name}.npz")
    model = _model(z)
    conv, llh = model.fit(z["obs"], max_iter=int(z["max_iter"]), censoring=bool(z["censoring"]),
                          forward_backward=orc.forward_backward)
    # the fixtures were made on x86; scipy's densities and numpy's sums differ
    # in the last bits on other hosts
    check_fit(model, z, conv, llh, rtol=1e-10, atol=1e-14)


def test_em_restores_the_parameters_when_the_e_step_fails():
    from tensor_viterbi import hsmm_em
    z = np.load(FB / "em_multinomial_J3_M20.npz")
    model = _model(z)
    before = (model.tmat.copy(), model.durations.copy(), model.probabilities.copy())

    def failing(*args):
        r = orc.forward_backward(*args)
        r["err"] = 1
        return r

    with pytest.raises(hsmm_em.NoConvergenceError):
        model.fit(z["obs"], max_iter=3, forward_backward=failing)
    np.testing.assert_array_equal(model.tmat, before[0])
    np.testing.assert_array_equal(model.durations, before[1])
    np.testing.assert_array_equal(model.probabilities, before[2])


def test_fixtures_match_a_fresh_reference_run_where_the_checkout_is_present():
    hh = orc.reference_hsmmlearn()
    if hh is None:
        pytest.skip("reference checkout or its hsmmlearn build absent")
    import sys
    base = sys.modules["hsmmlearn.base"]
    z = np.load(FB / "fb_J3_M20_T300_c1.npz")
    J, tau = z["pdf"].shape
    M = z["d"].shape[1]
    out = {k: np.zeros((J, tau)) for k in ("F", "L", "G", "L1", "Norm")}
    out["N"] = np.zeros(tau)
    out["eta"] = np.zeros((J, M))
    err = base._fb_impl(1, tau, J, M, z["d"].ravel().copy(), z["p"].ravel().copy(), z["pi"].copy(),
                        z["pdf"].ravel().copy(), *(out[k].reshape(-1) for k in orc.FB_KEYS),
                        np.zeros(J * M))
    assert err == 0
    for k in orc.FB_KEYS:
        np.testing.assert_array_equal(out[k], z[k])
