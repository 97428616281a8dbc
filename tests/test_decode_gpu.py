"""GPU parity: the CUDA decoder, called through the C ABI, against the
reference's golden paths and the CPU oracle.

Bar: paths bit-exact; the log-likelihood bit-exact against the oracle's
(both follow the reference association) and within 1e-9 relative of the
independent long-double segment scorer.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

LL_RTOL = 1e-9


@pytest.mark.parametrize("name", golden_names())
def test_golden_paths(tvlib, name):
    args, z = load_golden(name)
    path, ll = tvlib.decode_tensor_viterbi_cuda_loglik(*args)
    np.testing.assert_array_equal(path, z["path_cpp"])
    ref = orc.decode(*args, tables=True)
    assert ll == ref["loglik"], (ll, ref["loglik"])
    if np.isfinite(ll):
        N, tm, em, _, sp, dp, obs = args
        sc = orc.score_segments(N, tm, em, sp, dp, obs, ref["path"], ref["seg_start"])
        assert abs(ll - sc) <= LL_RTOL * abs(sc)


def test_dropin_signature_returns_int32_path(tvlib):
    args, z = load_golden("syn_config0")
    out = tvlib.decode_tensor_viterbi_cuda(*args)
    assert out.dtype == np.int32 and out.shape == z["path_cpp"].shape
    np.testing.assert_array_equal(out, z["path_cpp"])


@pytest.mark.parametrize("seed", range(12))
def test_random_models_vs_oracle(tvlib, seed):
    import tensor_viterbi.synthetic as syn
    rng = np.random.default_rng(1000 + seed)
    N = int(rng.integers(1, 40))
    D = int(rng.integers(1, 120))
    T = int(rng.integers(D, D + 1500))
    M = int(rng.integers(2, 20))
    lo = float(rng.uniform(1, max(2, D / 2)))
    hi = float(rng.uniform(lo, max(lo + 1, D)))
    p = syn.discrete_problem(N, D, T, M, lo, hi, seed=seed)
    ref = orc.decode(*p.args())
    path, ll = tvlib.decode_tensor_viterbi_cuda_loglik(*p.args())
    np.testing.assert_array_equal(path, ref["path"])
    assert ll == ref["loglik"]


def test_model_reuse_and_batch_equal_single(tvlib):
    import tensor_viterbi.synthetic as syn
    prob, seqs = syn.batch_problem(n_seq=24, N=10, D=60, M=16, lo=60, hi=3000, seed=5)
    with tvlib.Model(*prob.model_args()) as m:
        singles = [m.decode(s, return_loglik=True) for s in seqs]
        paths, lls = m.decode_batch(seqs, return_loglik=True)
    for (p1, l1), p2, l2, s in zip(singles, paths, lls, seqs):
        np.testing.assert_array_equal(p1, p2)
        assert l1 == l2
        ref = orc.decode(*prob.model_args(), s)
        np.testing.assert_array_equal(p1, ref["path"])
        assert l1 == ref["loglik"]


def test_batch_autotuned_cta_shape(tvlib):
    """A batch of two waves of CTAs or more tunes the CTA shape once per
    (N, D) and decodes with it; every path equals the one-at-a-time decode,
    and the oracle on a sample.  TV_AUTOTUNE=0 keeps the default shape."""
    import os
    import tensor_viterbi.synthetic as syn
    prob, seqs = syn.batch_problem(n_seq=320, N=10, D=60, M=16, lo=60, hi=400, seed=21)
    with tvlib.Model(*prob.model_args()) as m:
        paths, lls = m.decode_batch(seqs, return_loglik=True)
        shape = m.batch_threads()
        assert shape in (128, 256, 384, 512)
        paths2, lls2 = m.decode_batch(seqs, return_loglik=True)
        assert m.batch_threads() == shape  # kept for the process
        for k in range(0, len(seqs), 37):
            p1, l1 = m.decode(seqs[k], return_loglik=True)
            np.testing.assert_array_equal(paths[k], p1)
            np.testing.assert_array_equal(paths2[k], p1)
            assert lls[k] == l1 == lls2[k]
            ref = orc.decode(*prob.model_args(), seqs[k])
            np.testing.assert_array_equal(p1, ref["path"])
            assert l1 == ref["loglik"]
    prob2, seqs2 = syn.batch_problem(n_seq=320, N=10, D=70, M=16, lo=70, hi=300, seed=22)
    os.environ["TV_AUTOTUNE"] = "0"
    try:
        with tvlib.Model(*prob2.model_args()) as m:
            paths, lls = m.decode_batch(seqs2, return_loglik=True)
            assert m.batch_threads() == 256
            p1, l1 = m.decode(seqs2[5], return_loglik=True)
            np.testing.assert_array_equal(paths[5], p1)
            assert lls[5] == l1
    finally:
        del os.environ["TV_AUTOTUNE"]


def test_batch_with_the_duration_table_in_global_memory(tvlib, monkeypatch):
    """A batch with more sequences than the full work area's grid holds (N=10,
    D=250: two CTAs of 86 KB per SM) leaves the duration table in global
    memory so that a third CTA shares each SM; every path equals the
    one-at-a-time decode (a lone CTA keeps the full work area) and the oracle
    on a sample."""
    import torch
    import tensor_viterbi.synthetic as syn
    monkeypatch.setenv("TV_AUTOTUNE", "0")  # 256 threads: three CTAs fit an SM without the table
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    prob, seqs = syn.batch_problem(n_seq=3 * sms + 24, N=10, D=250, M=16, lo=260, hi=700, seed=31)
    with tvlib.Model(*prob.model_args()) as m:
        paths, lls = m.decode_batch(seqs, return_loglik=True)
        assert m.batch_threads() == 256
        assert m.batch_grid() == 3 * sms
        for k in range(0, len(seqs), 41):
            p1, l1 = m.decode(seqs[k], return_loglik=True)
            np.testing.assert_array_equal(paths[k], p1)
            assert lls[k] == l1
            if k % 123 == 0:
                ref = orc.decode(*prob.model_args(), seqs[k])
                np.testing.assert_array_equal(p1, ref["path"])
                assert l1 == ref["loglik"]


def test_errors_are_returned_not_fatal(tvlib):
    args, _ = load_golden("syn_config0")
    N, tm, em, dl, sp, dp, obs = args
    with pytest.raises(ValueError, match="T="):
        tvlib.decode_tensor_viterbi_cuda(N, tm, em, dl, sp, dp, obs[:10])
    bad = obs.copy()
    bad[3] = 99
    with pytest.raises(ValueError, match="outside"):
        tvlib.decode_tensor_viterbi_cuda(N, tm, em, dl, sp, dp, bad)
    # in a batch the kernel's own range check reports the sequence
    with tvlib.Model(N, tm, em, dl, sp, dp) as m:
        with pytest.raises(ValueError, match="sequence 1 has an observation outside"):
            m.decode_batch([obs, bad, obs])
        np.testing.assert_array_equal(m.decode_batch([obs, obs])[1], orc.decode(*args)["path"])
    # the library stays usable after an error
    np.testing.assert_array_equal(tvlib.decode_tensor_viterbi_cuda(*args), orc.decode(*args)["path"])


@pytest.mark.parametrize("N,D,T", [(150, 400, 1000), (200, 64, 700)])
def test_large_n_falls_back_to_one_cta_with_its_window_in_global_memory(tvlib, N, D, T):
    """N above the grid kernel's 128 states, with a window far larger than one
    CTA's shared memory (34*N*D + 8*N*N bytes: 2.2 MB and 0.75 MB): the
    automatic choice is the one-CTA kernel with its window in global scratch,
    which the reference's N (any N its reduction block takes) needs.  Exact
    against the oracle; a forced grid is refused with a clear error."""
    import tensor_viterbi.synthetic as syn
    p = syn.discrete_problem(N, D, T, 24, 5.0, max(6.0, D / 2), seed=N + D)
    ref = orc.decode(*p.args(), variant="omp")
    with tvlib.Model(*p.model_args()) as m:
        path, ll = m.decode(p.obs_seq, return_loglik=True)
        assert m.last_path() == "cta"
        m.set_path("grid")
        with pytest.raises(ValueError, match="grid kernel cannot take this shape"):
            m.decode(p.obs_seq)
    np.testing.assert_array_equal(path, ref["path"])
    assert ll == ref["loglik"]
