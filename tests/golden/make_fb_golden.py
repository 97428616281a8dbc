"""Generate the forward-backward / EM fixtures under tests/golden/fb/ by running
the reference's own hsmmlearn (development host only: it needs the read-only
checkout and oracle/build_ref.sh's build of hsmmlearn's compiled core).

fb_<name>.npz   one E step: the inputs of hsmmlearn's _fb_impl (censoring, d,
                p, pi, pdf) and its outputs (F, L, G, L1, N, Norm, eta, err),
                from FBImpl.cpp through the reference's Cython wrapper
em_<name>.npz   HSMMModel.fit (hsmmlearn/hsmmlearn/hsmm.py:181-305) on a
                seeded sequence: the initial and the fitted parameters, the
                converged flag and the final log-likelihood, for
                MultinomialHSMM and GaussianHSMM

Usage: python tests/golden/make_fb_golden.py [REFERENCE_ROOT]
"""
from __future__ import annotations

import os
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
REPO = HERE.parents[1]
OUT = HERE / "fb"
sys.path.insert(0, str(REPO))
if len(sys.argv) > 1:
    os.environ["TV_REFERENCE_ROOT"] = sys.argv[1]
from oracle import oracle as orc  # noqa: E402

hh = orc.reference_hsmmlearn()
if hh is None:
    sys.exit("make_fb_golden: no reference checkout or hsmmlearn build (oracle/build_ref.sh)")
base = sys.modules["hsmmlearn.base"]


def random_model(rng, J, M, zero_diag=True):
    tmat = rng.dirichlet(np.ones(J), size=J)
    if J > 1 and zero_diag:
        np.fill_diagonal(tmat, 0.0)
        tmat /= tmat.sum(1, keepdims=True)
    dur = rng.dirichlet(np.ones(M) * 2.0, size=J)
    pi = rng.dirichlet(np.ones(J))
    return tmat, dur, pi


def fb_case(name, rng, J, M, tau, censoring, lik=None):
    tmat, dur, pi = random_model(rng, J, M)
    if lik is None:
        lik = rng.uniform(0.02, 1.0, size=(J, tau))
    out = {k: np.zeros((J, tau)) for k in ("F", "L", "G", "L1", "Norm")}
    out["N"] = np.zeros(tau)
    out["eta"] = np.zeros((J, M))
    xi = np.zeros((J, M))
    err = base._fb_impl(censoring, tau, J, M, dur.ravel().copy(), tmat.ravel().copy(), pi.copy(),
                        np.ascontiguousarray(lik).ravel().copy(),
                        *(out[k].reshape(-1) for k in ("F", "L", "G", "L1", "N", "Norm", "eta")), xi.reshape(-1))
    np.savez_compressed(OUT / f"fb_{name}.npz", censoring=censoring, d=dur, p=tmat, pi=pi, pdf=lik, err=err, **out)
    print("fb", name, "err", err)


def em_case(name, rng, kind, J, M, n_obs, max_iter, censoring=True):
    tmat, dur, pi = random_model(rng, J, M)
    if kind == "multinomial":
        K = 6
        em = rng.dirichlet(np.ones(K), size=J)
        gen = hh.MultinomialHSMM(em, dur, tmat, startprob=pi)
    else:
        means = rng.normal(0.0, 3.0, size=J)
        scales = rng.uniform(0.5, 1.5, size=J)
        gen = hh.GaussianHSMM(means, scales, dur, tmat, startprob=pi)
    np.random.seed(int(rng.integers(1 << 30)))  # hsmmlearn samples with numpy's global generator
    obs, _ = gen.sample(n_obs)
    # a perturbed starting point
    t0 = tmat + rng.uniform(0.0, 0.2, size=tmat.shape)
    if J > 1:
        np.fill_diagonal(t0, 0.0)
    t0 /= t0.sum(1, keepdims=True)
    d0 = dur + rng.uniform(0.0, 0.05, size=dur.shape)
    d0 /= d0.sum(1, keepdims=True)
    p0 = np.full(J, 1.0 / J)
    if kind == "multinomial":
        e0 = em + rng.uniform(0.0, 0.1, size=em.shape)
        e0 /= e0.sum(1, keepdims=True)
        model = hh.MultinomialHSMM(e0.copy(), d0.copy(), t0.copy(), startprob=p0.copy())
        init = dict(emissions=e0)
    else:
        m0 = means + rng.normal(0.0, 0.3, size=J)
        s0 = scales * rng.uniform(0.9, 1.2, size=J)
        model = hh.GaussianHSMM(m0.copy(), s0.copy(), d0.copy(), t0.copy(), startprob=p0.copy())
        init = dict(means=m0, scales=s0)
    conv, llh = model.fit(obs, max_iter=max_iter, censoring=censoring)
    if kind == "multinomial":
        fitted = dict(fit_emissions=model.emissions._probabilities)
    else:
        fitted = dict(fit_means=model.means, fit_scales=model.scales)
    np.savez_compressed(OUT / f"em_{name}.npz", kind=kind, obs=obs, max_iter=max_iter, censoring=int(censoring),
             tmat0=t0, durations0=d0, startprob0=p0, fit_tmat=model.tmat, fit_durations=model.durations,
             fit_startprob=model._startprob, converged=conv, llh=llh, **init, **fitted)
    print("em", name, "converged", conv, "llh", llh)


def main():
    OUT.mkdir(exist_ok=True)
    rng = np.random.default_rng(2024)
    fb_case("J3_M20_T300_c0", rng, 3, 20, 300, 0)
    fb_case("J3_M20_T300_c1", rng, 3, 20, 300, 1)
    fb_case("J8_M60_T800_c1", rng, 8, 60, 800, 1)
    fb_case("J12_M100_T500_c0", rng, 12, 100, 500, 0)
    fb_case("J5_M50_T40_c1", rng, 5, 50, 40, 1)   # M > tau: durations beyond the sequence
    fb_case("J1_M10_T60_c1", rng, 1, 10, 60, 1)   # one state
    fb_case("J2_M1_T50_c1", rng, 2, 1, 50, 1)     # durations of one step only
    fb_case("J4_M30_T1_c1", rng, 4, 30, 1, 1)     # a single observation
    em_case("multinomial_J3_M20", rng, "multinomial", 3, 20, 1500, 6)
    em_case("gaussian_J4_M30", rng, "gaussian", 4, 30, 2000, 6)
    em_case("multinomial_J6_M40_nocens", rng, "multinomial", 6, 40, 2500, 5, censoring=False)


if __name__ == "__main__":
    main()
