"""HSMM model container and JSON loader, compatible with the reference's
`tensor_viterbi.hsmm.HSMM` (tensor_viterbi/hsmm.py:11-132 there), so that
code written against it (its benchmark app, `viterbi_app.py:143-234`) runs
unchanged on the reference's `data/*.json` files with this package first on
the path.

Conventions kept from the reference (they decide the decoder's inputs):
  * JSON fields (README.md:377-394 there): `n_steps`, `M` (max duration),
    `n_bins` (emission symbols), `seed`, `pi`, `trans_mat` ([from][to]),
    `obs_seq` (1-based symbols), `states` (name, `emission_probs` over the
    bins, `duration_probs` over 1..M);
  * the loader transposes the transition matrix to [to][from], lays the
    emission table out as (bins, N) and the duration tables as (M, N), and
    makes the observations 0-based (floats, as the reference does);
  * `to_log_space` replaces the transition, emission, start and duration
    tables by log(x + 1e-30) and leaves the linear duration table as it is
    (hsmm.py:76-82 there);
  * the loader seeds numpy's and Python's global generators with `seed`, as
    the reference's does.
"""
from __future__ import annotations

import json
import random

import numpy as np

SMOOTHNESS = 1e-30


class HSMM:
    """An explicit-duration HMM as the reference's decoders take it."""

    def __init__(self, states, emissions, trans_mat, emission_prob, duration_probs_linear, start_probs,
                 duration_probs):
        self.states = states
        self.emissions = emissions
        self.trans_mat = trans_mat
        self.emission_probs = emission_prob
        self.duration_probs_linear = duration_probs_linear
        self.start_probs = start_probs
        self.duration_probs = duration_probs
        self.obs_seq = None

    def set_obs_sequence(self, obs_seq) -> None:
        self.obs_seq = obs_seq

    def to_log_space(self) -> None:
        """Log tables in place: log(x + 1e-30) of the transition, emission,
        start and duration tables; the linear durations stay linear."""
        self.trans_mat = np.log(self.trans_mat + SMOOTHNESS)
        self.emission_probs = np.log(self.emission_probs + SMOOTHNESS)
        self.start_probs = np.log(self.start_probs + SMOOTHNESS)
        self.duration_probs = np.log(self.duration_probs + SMOOTHNESS)

    def decoder_args(self):
        """The seven positional arguments of decode_tensor_viterbi_cuda."""
        return (len(self.states), self.trans_mat, self.emission_probs, self.duration_probs_linear,
                self.start_probs, self.duration_probs, self.obs_seq)

    @staticmethod
    def load_model(json_path: str = "hsmm_config.json") -> "HSMM":
        with open(json_path, "r") as f:
            cfg = json.load(f)
        seed = int(cfg["seed"])
        np.random.seed(seed)
        random.seed(seed)
        n_bins = int(cfg["n_bins"])
        states = cfg["states"]
        names = [s["name"] for s in states]
        emission_rows = np.array([s["emission_probs"] for s in states], dtype=float)   # (N, bins)
        duration_rows = np.array([s["duration_probs"] for s in states], dtype=float)   # (N, M)
        trans = np.array(cfg["trans_mat"], dtype=float)                                # [from][to]
        h = HSMM(names, np.arange(n_bins), trans.T, emission_rows.T, duration_rows.T,
                 np.array(cfg["pi"], dtype=float), duration_rows.T)
        h.set_obs_sequence(np.array(cfg["obs_seq"], dtype=float) - 1)
        return h


def save_model_json(path, trans_from_to, emission_rows, duration_rows, pi, obs_zero_based, seed: int = 0,
                    names=None) -> None:
    """Write a model and observation sequence in the format load_model reads
    (linear probabilities; emission_rows (N, bins) and duration_rows (N, M)
    per state; observations 0-based here, stored 1-based)."""
    emission_rows = np.asarray(emission_rows, dtype=float)
    duration_rows = np.asarray(duration_rows, dtype=float)
    N, bins = emission_rows.shape
    obs = np.asarray(obs_zero_based).astype(np.int64) + 1
    cfg = {
        "n_steps": int(obs.size), "M": int(duration_rows.shape[1]), "n_bins": int(bins), "seed": int(seed),
        "pi": [float(v) for v in np.asarray(pi, dtype=float)],
        "trans_mat": np.asarray(trans_from_to, dtype=float).tolist(),
        "obs_seq": [int(v) for v in obs],
        "states": [{"name": (names[j] if names else f"S{j}"), "emission_probs": emission_rows[j].tolist(),
                    "duration_probs": duration_rows[j].tolist()} for j in range(N)],
    }
    with open(path, "w") as f:
        json.dump(cfg, f)
