"""Model ingest and the benchmark CSV (CPU): the JSON loader against the
reference's conventions and fixtures, and the CSV schema of the reference's
harness.  The GPU decode of a loaded model is in test_ingest_gpu.py."""
import csv
import pathlib

import numpy as np
import pytest

from conftest import load_golden
from oracle import oracle as orc

_ROOT = orc.reference_root()
REF_DATA = _ROOT / "data" if _ROOT else pathlib.Path("reference-checkout-absent")


def _hsmm():
    import sys
    from conftest import PKG
    sys.path.insert(0, str(PKG))
    from tensor_viterbi import hsmm
    return hsmm


def test_loader_round_trip_applies_the_reference_conventions(tmp_path):
    hsmm = _hsmm()
    rng = np.random.default_rng(0)
    N, bins, M, T = 4, 7, 12, 60
    trans = rng.dirichlet(np.ones(N), size=N)          # [from][to]
    em = rng.dirichlet(np.ones(bins), size=N)          # (N, bins)
    dur = rng.dirichlet(np.ones(M), size=N)            # (N, M)
    pi = rng.dirichlet(np.ones(N))
    obs = rng.integers(0, bins, T)
    path = tmp_path / "m.json"
    hsmm.save_model_json(path, trans, em, dur, pi, obs, seed=5)
    h = hsmm.HSMM.load_model(str(path))
    np.testing.assert_array_equal(h.trans_mat, trans.T)
    np.testing.assert_array_equal(h.emission_probs, em.T)
    np.testing.assert_array_equal(h.duration_probs_linear, dur.T)
    np.testing.assert_array_equal(h.obs_seq, obs.astype(float))
    assert h.obs_seq.dtype == np.float64 and list(h.emissions) == list(range(bins))
    h.to_log_space()
    np.testing.assert_array_equal(h.trans_mat, np.log(trans.T + 1e-30))
    np.testing.assert_array_equal(h.duration_probs, np.log(dur.T + 1e-30))
    np.testing.assert_array_equal(h.duration_probs_linear, dur.T)   # stays linear
    N_, tm, ep, dl, sp, dp, ob = h.decoder_args()
    assert N_ == N and ep.shape == (bins, N) and dp.shape == (M, N)


@pytest.mark.skipif(not (REF_DATA / "10states_1000steps_100dur.json").exists(),
                    reason="the reference's data files are not in this environment")
@pytest.mark.parametrize("stem", ["10states_1000steps_100dur", "15states_1000steps_250dur"])
def test_loader_matches_the_reference_loader_on_its_data(stem):
    """The golden fixtures were made with the reference's own HSMM.load_model +
    to_log_space (tests/golden/make_golden.py): the same arrays, bit for bit."""
    hsmm = _hsmm()
    args, _ = load_golden(f"ref_{stem}")
    h = hsmm.HSMM.load_model(str(REF_DATA / f"{stem}.json"))
    h.to_log_space()
    got = h.decoder_args()
    assert got[0] == args[0]
    for a, b in zip(got[1:6], args[1:6]):
        np.testing.assert_array_equal(np.asarray(a), np.asarray(b))
    np.testing.assert_array_equal(np.asarray(got[6]).astype(np.int32), args[6])


def test_harness_writes_the_reference_csv_schema(tmp_path):
    import sys
    from conftest import PKG
    sys.path.insert(0, str(PKG))
    from tensor_viterbi import harness

    class M:
        calls = 0

    def run(m):
        M.calls += 1
        return np.zeros(3, dtype=np.int32)

    out = tmp_path / "x_decode.csv"
    times, last = harness.bench_csv("decode_tensor_viterbi_cuda", run, M(), 10, 1000, 100, 3, str(out))
    rows = list(csv.reader(open(out)))
    assert rows[0] == ["function", "n_states", "timesteps", "max_duration", "iteration", "elapsed_s"]
    assert [r[:5] for r in rows[1:]] == [["decode_tensor_viterbi_cuda", "10", "1000", "100", str(i)] for i in range(3)]
    assert all(len(r[5].split(".")[1]) == 6 for r in rows[1:])
    assert len(times) == 3 and M.calls == 3 and last.shape == (3,)
