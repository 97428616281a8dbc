"""GPU parity of the whole-GPU grid kernel (head CTA + worker CTAs): the same
results as the oracle and as the one-CTA kernel, bit for bit, on the golden
fixtures, on random shapes and at grid sizes from a handful of CTAs to one
per SM."""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _grid_ok(N, D):
    return D > 8 and N <= 128


@pytest.mark.parametrize("grid_ctas", [0, 5])
@pytest.mark.parametrize("name", golden_names())
def test_grid_golden(tvlib, name, grid_ctas):
    args, z = load_golden(name)
    N, D = args[0], args[5].shape[0]
    if not _grid_ok(N, D):
        pytest.skip("shape outside the grid kernel (D <= 8)")
    ref = orc.decode(*args)
    with tvlib.Model(*args[:6]) as m:
        m.set_path("grid", grid_ctas)
        path, ll = m.decode(args[6], return_loglik=True)
        assert m.last_path() == "grid"
    np.testing.assert_array_equal(path, z["path_cpp"])
    assert ll == ref["loglik"]


@pytest.mark.parametrize("seed", range(8))
def test_grid_random_vs_oracle_and_cta(tvlib, seed):
    import tensor_viterbi.synthetic as syn
    rng = np.random.default_rng(500 + seed)
    N = int(rng.integers(1, 60))
    D = int(rng.integers(5, 400))
    T = int(rng.integers(D, D + 2 * D + 300))
    M = int(rng.integers(2, 32))
    lo = float(rng.uniform(1, max(2, D / 3)))
    hi = float(rng.uniform(lo, max(lo + 1, D)))
    p = syn.discrete_problem(N, D, T, M, lo, hi, seed=seed)
    ref = orc.decode(*p.args(), variant="omp")
    with tvlib.Model(*p.model_args()) as m:
        m.set_path("grid", int(rng.integers(N // 2 + 2, 160)))
        pg, lg = m.decode(p.obs_seq, return_loglik=True)
        m.set_path("cta")
        pc, lc = m.decode(p.obs_seq, return_loglik=True)
    np.testing.assert_array_equal(pg, ref["path"])
    np.testing.assert_array_equal(pc, ref["path"])
    assert lg == ref["loglik"] == lc


def test_grid_long_window_early_phase(tvlib):
    """D in the thousands: the checkpointed newest-first sums (t <= D), the
    switch to running folds at t = D+1 and a window spread over many CTAs."""
    import tensor_viterbi.synthetic as syn
    p = syn.discrete_problem(12, 2500, 5600, 24, 50.0, 1200.0, seed=77)
    ref = orc.decode(*p.args(), variant="omp")
    with tvlib.Model(*p.model_args()) as m:
        path, ll = m.decode(p.obs_seq, return_loglik=True)
        assert m.last_path() == "grid"
    np.testing.assert_array_equal(path, ref["path"])
    assert ll == ref["loglik"]


def test_grid_gaussian_table(tvlib):
    import tensor_viterbi.synthetic as syn
    p = syn.gaussian_problem(20, 300, 2000, 10.0, 150.0, seed=5)
    ref = orc.decode(*p.args(), variant="omp")
    with tvlib.Model(*p.model_args()) as m:
        m.set_path("grid", 0)
        path, ll = m.decode(p.obs_seq, return_loglik=True)
    np.testing.assert_array_equal(path, ref["path"])
    assert ll == ref["loglik"]


def test_grid_device_obs_validation(tvlib):
    import torch
    import tensor_viterbi.synthetic as syn
    p = syn.discrete_problem(8, 50, 400, 6, 5.0, 30.0, seed=3)
    ref = orc.decode(*p.args())
    with tvlib.Model(*p.model_args()) as m:
        m.set_path("grid", 6)
        bad = torch.from_numpy(p.obs_seq.copy()).cuda()
        bad[123] = 6
        out = torch.empty_like(bad)
        m.decode_device(bad.data_ptr(), bad.numel(), out.data_ptr(), 0, torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        # the host-buffer call afterwards still works and is exact
        path, ll = m.decode(p.obs_seq, return_loglik=True)
    np.testing.assert_array_equal(path, ref["path"])
    assert ll == ref["loglik"]


@pytest.mark.parametrize("grid_ctas", [0, 7])
@pytest.mark.parametrize("name", golden_names())
def test_grid_window_in_l2_golden(tvlib, name, grid_ctas):
    """The grid kernel with its window in global memory (the layout taken when
    N*D does not fit the workers' shared memory), forced on every fixture."""
    args, z = load_golden(name)
    N, D = args[0], args[5].shape[0]
    if not _grid_ok(N, D):
        pytest.skip("shape outside the grid kernel (D <= 8)")
    ref = orc.decode(*args)
    with tvlib.Model(*args[:6]) as m:
        m.set_path("grid-l2", grid_ctas)
        path, ll = m.decode(args[6], return_loglik=True)
        assert m.last_path() == "grid"
    np.testing.assert_array_equal(path, z["path_cpp"])
    assert ll == ref["loglik"]


def test_grid_large_n_head(tvlib):
    """N = 100: four pairs of critical and upper-half matvec warps beside the
    other roles; both window placements."""
    import tensor_viterbi.synthetic as syn
    p = syn.discrete_problem(100, 40, 700, 24, 5.0, 30.0, seed=11)
    ref = orc.decode(*p.args(), variant="omp")
    with tvlib.Model(*p.model_args()) as m:
        for kind in ("grid", "grid-l2"):
            m.set_path(kind, 0)
            path, ll = m.decode(p.obs_seq, return_loglik=True)
            assert m.last_path() == "grid"
            np.testing.assert_array_equal(path, ref["path"])
            assert ll == ref["loglik"]


def test_grid_max_n_head_with_and_without_split_matvec(tvlib):
    """N = 128, the largest the packed coarse scores take.  With the window in
    shared memory each state is one worker's segment and the upper half of the
    matvec has its own warps; with the window in L2 the contiguous chunks give
    more segments than the block has room for beside a split matvec, so the
    critical lanes scan whole rows."""
    import tensor_viterbi.synthetic as syn
    p = syn.discrete_problem(128, 40, 700, 24, 5.0, 30.0, seed=13)
    ref = orc.decode(*p.args(), variant="omp")
    with tvlib.Model(*p.model_args()) as m:
        for kind in ("grid", "grid-l2"):
            m.set_path(kind, 0)
            path, ll = m.decode(p.obs_seq, return_loglik=True)
            assert m.last_path() == "grid"
            np.testing.assert_array_equal(path, ref["path"])
            assert ll == ref["loglik"]


def _segments_of(path, D):
    starts = np.flatnonzero(np.diff(path, prepend=-1) != 0)
    lengths = np.diff(np.append(starts, path.size))
    seg = np.zeros(path.size, dtype=np.uint8)
    seg[starts] = 1
    return seg, lengths


def test_stress_shape_window_in_l2_properties(tvlib):
    """The stress shape's window (N = 100, D = 1e4: 1e6 cells, too large for
    shared memory, so the grid picks the global-memory window) on a 3e4-step
    sequence.  The oracle's O(T N^2 D) recursion is out of reach at this
    size, so size-independent properties stand in: every segment fits the
    duration range, the returned log-likelihood is the long-double score of
    the returned path within 1e-9 relative, and a second decode is identical.
    Exactness itself is covered by the parity tests of the same kernel on
    smaller shapes above."""
    import tensor_viterbi.synthetic as syn
    p = syn.discrete_problem(100, 10_000, 30_000, 64, 5.0, 50.0, seed=4)
    with tvlib.Model(*p.model_args()) as m:
        path, ll = m.decode(p.obs_seq, return_loglik=True)
        assert m.last_path() == "grid"
        path2, ll2 = m.decode(p.obs_seq, return_loglik=True)
    np.testing.assert_array_equal(path, path2)
    assert ll == ll2
    assert path.min() >= 0 and path.max() < 100
    seg, lengths = _segments_of(path, 10_000)
    assert lengths.max() <= 10_000
    sc = orc.score_segments(p.n_states, p.trans_mat, p.emission_probs, p.start_probs, p.duration_probs,
                            p.obs_seq, path, seg)
    assert abs(ll - sc) <= 1e-9 * abs(sc)


def test_step_floor_probe(tvlib):
    """The latency-floor probe of the head's critical chain and the cross-SM
    round trip: both finish, report positive times, use the plan's matvec
    split, and the chain alone is faster per step than a real decode."""
    import tensor_viterbi.synthetic as syn
    f = tvlib.step_floor(75, 5000, 5000)
    assert f["chain_clocks_per_step"] > 0 and f["chain_us_per_step"] > 0
    assert f["roundtrip_clocks"] > 0 and f["roundtrip_us"] > 0
    assert f["roundtrip_sms"][0] != f["roundtrip_sms"][1]
    import torch
    from tensor_viterbi.viterbi import _lib
    props = torch.cuda.get_device_properties(0)
    optin = getattr(props, "shared_memory_per_block_optin", 232448)
    info = np.zeros(10, dtype=np.int64)
    _lib.check(_lib.lib().tv_grid_plan_info(75, 5000, props.multi_processor_count, optin, 0, info.ctypes.data))
    assert f["matvec_split"] == bool(info[4])
    p = syn.discrete_problem(75, 5000, 30000, 32, 50.0, 2500.0, seed=1)
    with tvlib.Model(*p.model_args()) as m:
        m.set_timing(True)
        m.decode(p.obs_seq)
        step_us = 1e3 * m.kernel_ms() / p.T
    assert f["chain_us_per_step"] < step_us


def test_lost_worker_message_times_out_and_the_next_decode_is_exact(tvlib):
    """Failure handling of the grid kernel without a GPU fault: one worker
    partial message is never sent (tv_model_drop_partial, the worker skips
    that one store).  The bounded wait for it runs out after about a second
    of SM clocks, every CTA leaves at the same step, and the decode returns
    TV_ETIMEOUT naming the wait -- the reference exits the process on any
    device failure (src/hsmm.cu:22-30).  The next decode on the same model
    is exact."""
    import time
    import tensor_viterbi.synthetic as syn
    p = syn.discrete_problem(20, 300, 3000, 16, 20.0, 150.0, seed=21)
    ref = orc.decode(*p.args(), variant="omp")
    with tvlib.Model(*p.model_args()) as m:
        m.set_path("grid", 16)
        m.drop_partial(1500, 0)
        t0 = time.perf_counter()
        with pytest.raises(RuntimeError, match="timed out") as ei:
            m.decode(p.obs_seq)
        waited = time.perf_counter() - t0
        msg = str(ei.value)
        assert "head waiting for worker partials" in msg or "worker waiting for a slot message" in msg, msg
        assert 0.2 < waited < 30.0
        path, ll = m.decode(p.obs_seq, return_loglik=True)
        assert m.last_path() == "grid"
    np.testing.assert_array_equal(path, ref["path"])
    assert ll == ref["loglik"]
