"""GPU: a JSON model loaded through tensor_viterbi.hsmm decodes, through the
drop-in call and the CSV harness, to the oracle's path."""
import csv

import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def test_json_model_through_the_harness(tvlib, tmp_path):
    from tensor_viterbi import harness, hsmm
    import tensor_viterbi.synthetic as syn
    rng = np.random.default_rng(11)
    lm = syn.random_model(rng, 6, 40, 9, 5.0, 25.0)
    states = syn.sample_states(rng, lm, 800)
    obs = syn.sample_discrete_obs(rng, lm.B, states)
    path_json = tmp_path / "model.json"
    hsmm.save_model_json(path_json, lm.A, lm.B, lm.P, lm.pi, obs, seed=1)
    assert harness.main([str(path_json), "--iterations", "2", "--out", str(tmp_path / "run")]) == 0
    rows = list(csv.reader(open(tmp_path / "run_decode_tensor_viterbi_cuda.csv")))
    assert len(rows) == 3 and rows[1][:4] == ["decode_tensor_viterbi_cuda", "6", "800", "40"]
    h = hsmm.HSMM.load_model(str(path_json))
    h.to_log_space()
    path = tvlib.decode_tensor_viterbi_cuda(*h.decoder_args())
    ref = orc.decode(*h.decoder_args())
    np.testing.assert_array_equal(path, ref["path"])
