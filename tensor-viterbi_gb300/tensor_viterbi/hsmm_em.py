"""EM training of an explicit-duration HSMM with the E step on the GPU.

The reference's training step is hsmmlearn's HSMMModel.fit
(hsmmlearn/hsmmlearn/hsmm.py:181-305), with MultinomialHSMM and GaussianHSMM
(hsmm.py:308-346) and their emission models (hsmmlearn/hsmmlearn/emissions.py).
These classes keep its interface and its M step:
  * fit(obs, max_iter=20, atol=1e-5, censoring=True) -> (has_converged, llh),
    updating the parameters in place and restoring them and raising
    NoConvergenceError when the forward-backward reports an error;
  * likelihoods clipped below at 1e-12, log-likelihood sum(log N);
  * start probabilities from the smoothed probabilities at t = 0 (floored at
    1e-14, renormalised -- in place, so the emission update sees them, as in
    the reference), transitions from sum_t G[k][t+1] F[i][t], durations from
    eta over sum_t L1 (plus L at the end with censoring), emissions from the
    smoothed probabilities L.
The E step is tv_fb (the forward-backward kernel) through
tensor_viterbi.viterbi.native.forward_backward; `forward_backward=` takes
another implementation with the same signature (the tests pass the CPU
oracle to check the M step on its own).
"""
from __future__ import annotations

import numpy as np


class NoConvergenceError(Exception):
    pass


def _default_fb():
    from .viterbi import native
    return native.forward_backward


class _HSMM:
    def __init__(self, durations, tmat, startprob=None):
        self.tmat = np.array(tmat, dtype=np.float64)
        self.durations = np.array(durations, dtype=np.float64)
        J = self.tmat.shape[0]
        if self.tmat.shape != (J, J) or self.durations.ndim != 2 or self.durations.shape[0] != J:
            raise ValueError("tmat must be (J, J) and durations (J, M)")
        self.startprob = (np.full(J, 1.0 / J) if startprob is None
                          else np.array(startprob, dtype=np.float64))

    @property
    def n_states(self):
        return self.tmat.shape[0]

    @property
    def n_durations(self):
        return self.durations.shape[1]

    # emission model hooks
    def _likelihood(self, obs):
        raise NotImplementedError

    def _reestimate(self, gamma, obs):
        raise NotImplementedError

    def _emission_state(self):
        raise NotImplementedError

    def _restore_emissions(self, state):
        raise NotImplementedError

    def fit(self, obs, max_iter=20, atol=1e-5, censoring=True, forward_backward=None):
        fb = forward_backward or _default_fb()
        obs = np.atleast_1d(obs)
        censoring = int(censoring)
        J = self.n_states
        log_likelihoods = []
        llh = -np.inf
        has_converged = False
        old = (self.tmat.copy(), self.durations.copy(), self._emission_state(), self.startprob.copy())
        err = 0
        step = 0
        for step in range(1, max_iter + 1):
            likelihoods = self._likelihood(obs)
            likelihoods[likelihoods < 1e-12] = 1e-12
            r = fb(censoring, self.durations, self.tmat, self.startprob, likelihoods)
            err = r["err"]
            if err != 0:
                break
            f, l, g, l1, n, eta = r["F"], r["L"], r["G"], r["L1"], r["N"], r["eta"]
            new_llh = np.log(n).sum()
            log_likelihoods.append(new_llh)
            if np.abs(new_llh - llh) < atol:
                has_converged = True
                break
            llh = new_llh
            # start probabilities: a view of l's first column, changed in place
            new_pi = l[:, 0]
            new_pi[new_pi < 1e-14] = 1e-14
            new_pi /= new_pi.sum()
            new_tmat = np.empty_like(self.tmat)
            for i in range(J):
                r_i = l1[i, :-1].sum()
                for k in range(J):
                    z = self.tmat[i, k] * (g[k, 1:] * f[i, :-1]).sum()
                    new_tmat[i, k] = z / r_i
            denominator = l1[:, :-1].sum(axis=1)
            if censoring:
                denominator += l[:, -1]
            new_durations = eta / denominator[:, np.newaxis]
            self._reestimate(l, obs)
            self.tmat = new_tmat
            self.durations = new_durations
            self.startprob = new_pi
        if err != 0:
            self.tmat, self.durations, em_state, self.startprob = old
            self._restore_emissions(em_state)
            raise NoConvergenceError(
                f"the forward-backward algorithm reported an error after {step} steps; "
                f"log-likelihoods so far: {log_likelihoods}")
        return has_converged, llh


class MultinomialHSMM(_HSMM):
    """Discrete emissions over 0..K-1: probabilities (J, K), rows renormalised
    as hsmmlearn's NonParametricDistribution does (hsmmlearn/utils.py)."""

    def __init__(self, probabilities, durations, tmat, startprob=None):
        super().__init__(durations, tmat, startprob)
        self._set(np.array(probabilities, dtype=np.float64))

    def _set(self, probs):
        probs[probs < 0] = 0
        for row in probs:
            row /= row.sum()
        self.probabilities = probs

    def _likelihood(self, obs):
        return self.probabilities[:, np.asarray(obs)].copy()

    def _reestimate(self, gamma, obs):
        new = np.empty_like(self.probabilities)
        for em in range(self.probabilities.shape[1]):
            mask = obs == em
            new[:, em] = gamma[:, mask].sum(axis=1) / gamma.sum(axis=1)
        self._set(new)

    def _emission_state(self):
        return self.probabilities.copy()

    def _restore_emissions(self, state):
        self.probabilities = state


class GaussianHSMM(_HSMM):
    """Gaussian emissions: per-state means and scales; densities from
    scipy.stats.norm as hsmmlearn's GaussianEmissions computes them."""

    def __init__(self, means, scales, durations, tmat, startprob=None):
        super().__init__(durations, tmat, startprob)
        self.means = np.array(means, dtype=np.float64)
        self.scales = np.array(scales, dtype=np.float64)

    def _likelihood(self, obs):
        from scipy.stats import norm
        obs = np.squeeze(obs)
        return norm.pdf(obs, loc=self.means[:, np.newaxis], scale=self.scales[:, np.newaxis])

    def _reestimate(self, gamma, obs):
        p = np.sum(gamma * obs[np.newaxis, :], axis=1)
        q = np.sum(gamma, axis=1)
        new_means = p / q
        A = obs[np.newaxis, :] - new_means[:, np.newaxis]
        p = np.sum(gamma * A ** 2, axis=1)
        variances = p / q
        self.means = new_means
        self.scales = np.sqrt(variances)

    def _emission_state(self):
        return self.means.copy(), self.scales.copy()

    def _restore_emissions(self, state):
        self.means, self.scales = state
