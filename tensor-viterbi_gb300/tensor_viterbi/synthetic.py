"""Seeded synthetic HSMMs and observation sequences.

The model family of the benchmark workloads: initial distribution ~
Dirichlet(1); transition matrix with a zero diagonal and off-diagonal rows ~
Dirichlet(1); discrete emission rows ~ Dirichlet(1) over M symbols; per-state
duration pmf a Poisson with mean ~ U[lo, hi] truncated to 1..D and
renormalised; observations sampled from the model itself.  The arrays are put
through the reference's input conventions (tensor_viterbi/hsmm.py there):
transition and duration matrices transposed to [to][from] and (D, N),
`log(x + 1e-30)` for the log-space tables, the linear duration pmf kept.

Gaussian emissions (per-state mean ~ N(0, 4), sd ~ U[0.5, 2]) are supported
through a per-timestep log-likelihood table (T, N) used with
obs = arange(T): the same decode, with O = T emission rows.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

SMOOTH = 1e-30


@dataclass
class Problem:
    """Decoder inputs in the reference binding's layouts."""

    n_states: int
    trans_mat: np.ndarray              # (N, N) log, [to j][from i]
    emission_probs: np.ndarray         # (O, N) log
    duration_probs_linear: np.ndarray  # (D, N) linear
    start_probs: np.ndarray            # (N,) log
    duration_probs: np.ndarray         # (D, N) log
    obs_seq: np.ndarray                # (T,) int32
    meta: dict = field(default_factory=dict)

    @property
    def N(self) -> int:
        return self.n_states

    @property
    def D(self) -> int:
        return self.duration_probs.shape[0]

    @property
    def T(self) -> int:
        return int(self.obs_seq.size)

    @property
    def O(self) -> int:
        return self.emission_probs.shape[0]

    def model_args(self):
        return (self.n_states, self.trans_mat, self.emission_probs, self.duration_probs_linear,
                self.start_probs, self.duration_probs)

    def args(self):
        return self.model_args() + (self.obs_seq,)


def poisson_pmf_truncated(mean: float, D: int) -> np.ndarray:
    """Poisson(mean) pmf on durations 1..D, renormalised (index d = length d+1)."""
    k = np.arange(1, D + 1, dtype=np.float64)
    logp = k * math.log(mean) - mean - np.array([math.lgamma(x + 1.0) for x in k])
    logp -= logp.max()
    p = np.exp(logp)
    return p / p.sum()


@dataclass
class LinearModel:
    pi: np.ndarray        # (N,)
    A: np.ndarray         # (N, N) [from][to]
    B: np.ndarray         # (N, M) emission rows
    P: np.ndarray         # (N, D) duration pmf rows


def random_model(rng: np.random.Generator, N: int, D: int, M: int, mean_lo: float, mean_hi: float) -> LinearModel:
    pi = rng.dirichlet(np.ones(N))
    A = np.zeros((N, N))
    if N > 1:
        for i in range(N):
            row = rng.dirichlet(np.ones(N - 1))
            A[i, np.arange(N) != i] = row
    else:
        A[0, 0] = 1.0
    B = rng.dirichlet(np.ones(M), size=N)
    means = rng.uniform(mean_lo, mean_hi, size=N)
    P = np.stack([poisson_pmf_truncated(mu, D) for mu in means])
    return LinearModel(pi, A, B, P)


def sample_states(rng: np.random.Generator, lm: LinearModel, T: int) -> np.ndarray:
    """Segment-wise HSMM simulation of the hidden state path."""
    N, D = lm.P.shape
    cdfP = np.cumsum(lm.P, axis=1)
    cdfA = np.cumsum(lm.A, axis=1)
    states = np.empty(T, dtype=np.int32)
    t = 0
    s = int(rng.choice(N, p=lm.pi))
    while t < T:
        u = rng.random()
        k = int(min(np.searchsorted(cdfP[s], u * cdfP[s, -1], side="right"), D - 1)) + 1
        states[t:t + k] = s
        t += k
        u = rng.random()
        s = int(min(np.searchsorted(cdfA[s], u * cdfA[s, -1], side="right"), N - 1))
    return states


def sample_discrete_obs(rng: np.random.Generator, B: np.ndarray, states: np.ndarray, chunk: int = 1 << 20) -> np.ndarray:
    cdf = np.cumsum(B, axis=1)
    cdf[:, -1] = 1.0
    out = np.empty(states.size, dtype=np.int32)
    for a in range(0, states.size, chunk):
        st = states[a:a + chunk]
        u = rng.random(st.size)
        c = cdf[st]
        out[a:a + chunk] = (u[:, None] >= c).sum(axis=1).astype(np.int32)
    return np.minimum(out, B.shape[1] - 1)


def to_problem(lm: LinearModel, obs: np.ndarray, emission_log: np.ndarray | None = None, meta=None) -> Problem:
    N, D = lm.P.shape
    trans = np.log(lm.A.T + SMOOTH)                 # [to][from]
    em = np.log(lm.B.T + SMOOTH) if emission_log is None else emission_log
    dur_lin = np.ascontiguousarray(lm.P.T)          # (D, N)
    return Problem(
        n_states=N,
        trans_mat=np.ascontiguousarray(trans),
        emission_probs=np.ascontiguousarray(em),
        duration_probs_linear=dur_lin,
        start_probs=np.log(lm.pi + SMOOTH),
        duration_probs=np.log(dur_lin + SMOOTH),
        obs_seq=np.ascontiguousarray(obs.astype(np.int32)),
        meta=dict(meta or {}),
    )


def discrete_problem(N: int, D: int, T: int, M: int, mean_lo: float = 5.0, mean_hi: float = 50.0,
                     seed: int = 0) -> Problem:
    """A model of the benchmark family and T observations sampled from it."""
    rng = np.random.default_rng(seed)
    lm = random_model(rng, N, D, M, mean_lo, mean_hi)
    states = sample_states(rng, lm, T)
    obs = sample_discrete_obs(rng, lm.B, states)
    return to_problem(lm, obs, meta=dict(N=N, D=D, T=T, M=M, mean_lo=mean_lo, mean_hi=mean_hi, seed=seed,
                                         states=states))


def gaussian_loglik_table(x: np.ndarray, mu: np.ndarray, sd: np.ndarray) -> np.ndarray:
    """(T, N) log N(x_t; mu_j, sd_j) in float64: ((-0.5 z) z - log sd_j) -
    log(2 pi)/2 with z = (x_t - mu_j) / sd_j, each operation rounded once and
    the logs from the C library (math.log), as the device front-end computes
    it, so the two tables agree bit for bit."""
    x, mu, sd = (np.asarray(a, dtype=np.float64) for a in (x, mu, sd))
    logsd = np.array([math.log(float(v)) for v in sd], dtype=np.float64)
    c = 0.5 * math.log(2.0 * 3.141592653589793)
    z = (x[:, None] - mu[None, :]) / sd[None, :]
    return ((-0.5 * z) * z - logsd[None, :]) - c


def gaussian_problem(N: int, D: int, T: int, mean_lo: float = 5.0, mean_hi: float = 50.0,
                     seed: int = 0) -> Problem:
    """Gaussian emissions as a per-timestep table (O = T rows, obs = arange(T))."""
    rng = np.random.default_rng(seed)
    lm = random_model(rng, N, D, 2, mean_lo, mean_hi)
    mu = rng.normal(0.0, 2.0, size=N)
    sd = rng.uniform(0.5, 2.0, size=N)
    states = sample_states(rng, lm, T)
    x = rng.normal(mu[states], sd[states])
    table = gaussian_loglik_table(x, mu, sd)
    obs = np.arange(T, dtype=np.int32)
    return to_problem(lm, obs, emission_log=np.ascontiguousarray(table),
                      meta=dict(N=N, D=D, T=T, gaussian=True, seed=seed, x=x, mu=mu, sd=sd, states=states))


# Benchmark workloads (shapes of the reference sweep and its extensions).
def config0(seed: int = 0) -> Problem:
    """N=10, D=100, T=1000, M=16, duration means ~U[5,50], seed 0."""
    return discrete_problem(10, 100, 1000, 16, 5.0, 50.0, seed)


def config1(T: int = 1_000_000, seed: int = 1) -> Problem:
    """N=75, D=5000, T=1e6, M=32, duration means ~U[50,2500]."""
    return discrete_problem(75, 5000, T, 32, 50.0, 2500.0, seed)


def config4(T: int = 10_000_000, seed: int = 4) -> Problem:
    """N=100, D=1e4, T=1e7, M=64, duration means ~U[5,50]."""
    return discrete_problem(100, 10_000, T, 64, 5.0, 50.0, seed)


def batch_lengths(n_seq: int = 4096, lo: float = 1e3, hi: float = 1e5, seed: int = 2) -> np.ndarray:
    """Log-uniform sequence lengths in [lo, hi]."""
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(math.log(lo), math.log(hi), size=n_seq)).astype(np.int64)


def sample_states_batch(rng: np.random.Generator, lm: LinearModel, lengths) -> list:
    """Hidden state paths for many sequences at once: every iteration draws the
    next segment (duration, then successor state) of all unfinished sequences
    together.  Same model family as sample_states."""
    N, D = lm.P.shape
    lengths = np.asarray(lengths, dtype=np.int64)
    K = lengths.size
    cdfP = np.cumsum(lm.P, axis=1)
    cdfP /= cdfP[:, -1:]
    cdfA = np.cumsum(lm.A, axis=1)
    cdfA /= cdfA[:, -1:]
    cdfpi = np.cumsum(lm.pi)
    cdfpi /= cdfpi[-1]
    state = np.minimum(np.searchsorted(cdfpi, rng.random(K), side="right"), N - 1)
    pos = np.zeros(K, dtype=np.int64)
    seg_starts = [[] for _ in range(K)]
    seg_states = [[] for _ in range(K)]
    active = np.arange(K)
    while active.size:
        st = state[active]
        u = rng.random(active.size)
        dur = np.minimum((u[:, None] >= cdfP[st]).sum(axis=1), D - 1) + 1
        for k, a in enumerate(active):
            seg_starts[a].append(pos[a])
            seg_states[a].append(st[k])
        pos[active] += dur
        u = rng.random(active.size)
        state[active] = np.minimum((u[:, None] >= cdfA[st]).sum(axis=1), N - 1)
        active = active[pos[active] < lengths[active]]
    out = []
    for a in range(K):
        starts = np.asarray(seg_starts[a] + [lengths[a]], dtype=np.int64)
        reps = np.minimum(np.diff(starts), lengths[a] - starts[:-1])
        out.append(np.repeat(np.asarray(seg_states[a], dtype=np.int32), np.maximum(reps, 0))[: lengths[a]])
    return out


def batch_problem(n_seq: int = 4096, N: int = 10, D: int = 250, M: int = 16, lo: float = 1e3, hi: float = 1e5,
                  seed: int = 2):
    """One shared model, n_seq sequences with log-uniform lengths.  Returns
    (Problem with an empty obs, [obs])."""
    rng = np.random.default_rng(seed)
    lm = random_model(rng, N, D, M, 5.0, 50.0)
    lengths = batch_lengths(n_seq, lo, hi, seed)
    states = sample_states_batch(rng, lm, lengths)
    flat = np.concatenate(states)
    obs_flat = sample_discrete_obs(rng, lm.B, flat)
    seqs = np.split(obs_flat, np.cumsum(lengths)[:-1])
    prob = to_problem(lm, np.zeros(0, dtype=np.int32), meta=dict(N=N, D=D, M=M, n_seq=n_seq, seed=seed))
    return prob, [np.ascontiguousarray(s) for s in seqs]
