"""GPU tests of the Gaussian emission front-end and of the decode server.

Bar: the device table equals the host expression bit for bit; paths and
log-likelihoods bit-exact against the CPU oracle on the same table; a request
decoded in the server's mix gives exactly what it gives decoded alone.
"""
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _gauss(N, D, T, seed, lo=5.0, hi=50.0):
    import tensor_viterbi.synthetic as syn
    return syn.gaussian_problem(N, D, T, lo, hi, seed=seed)


def test_gaussian_front_end_table_is_bit_exact(tvlib):
    import torch
    import tensor_viterbi.synthetic as syn
    rng = np.random.default_rng(3)
    T, N = 5000, 13
    x = rng.normal(0.0, 3.0, T)
    mu = rng.normal(0.0, 2.0, N)
    sd = rng.uniform(0.5, 2.0, N)
    want = syn.gaussian_loglik_table(x, mu, sd)
    xd = torch.from_numpy(x).cuda()
    table = torch.empty((T, N), dtype=torch.float64, device="cuda")
    tvlib.gaussian_loglik_device(xd.data_ptr(), T, mu, sd, table.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = table.cpu().numpy()
    assert got.view(np.uint64).tolist() == want.view(np.uint64).tolist()


@pytest.mark.parametrize("shape", [(6, 40, 900), (20, 300, 2500), (40, 180, 1200)])
def test_gaussian_model_decode_vs_oracle(tvlib, shape):
    N, D, T = shape
    p = _gauss(N, D, T, seed=N + D)
    ref = orc.decode(*p.args(), variant="omp")
    with tvlib.GaussianModel(N, p.trans_mat, p.duration_probs_linear, p.start_probs, p.duration_probs,
                             p.meta["x"], p.meta["mu"], p.meta["sd"]) as m:
        path, ll = m.decode(return_loglik=True)
    np.testing.assert_array_equal(path, ref["path"])
    assert ll == ref["loglik"]


def _mix(seed):
    """Requests of several shapes: discrete and Gaussian, one-CTA windows and
    windows that need the grid (N*D beyond one CTA's shared memory)."""
    import tensor_viterbi.synthetic as syn
    rng = np.random.default_rng(seed)
    reqs = []
    for k in range(24):
        N = int(rng.choice([10, 15, 25]))
        D = int(rng.choice([20, 60, 100]))
        T = int(rng.integers(D, D + 2000))
        if k % 2:
            reqs.append(("gauss", _gauss(N, D, T, seed=seed * 100 + k)))
        else:
            reqs.append(("disc", syn.discrete_problem(N, D, T, 32, 5.0, 50.0, seed=seed * 100 + k)))
    # two windows beyond one CTA (the grid with a few CTAs)
    reqs.append(("disc", syn.discrete_problem(50, 1000, 2600, 32, 20.0, 400.0, seed=seed * 100 + 90)))
    reqs.append(("gauss", _gauss(25, 1000, 2200, seed=seed * 100 + 91, lo=20.0, hi=400.0)))
    return reqs


def _submit(srv, kind, p):
    if kind == "disc":
        return srv.submit(*p.args())
    return srv.submit_gaussian(p.n_states, p.trans_mat, p.duration_probs_linear, p.start_probs, p.duration_probs,
                               p.meta["x"], p.meta["mu"], p.meta["sd"])


def _alone(tvlib, kind, p):
    if kind == "disc":
        with tvlib.Model(*p.model_args()) as m:
            return m.decode(p.obs_seq, return_loglik=True)
    with tvlib.GaussianModel(p.n_states, p.trans_mat, p.duration_probs_linear, p.start_probs, p.duration_probs,
                             p.meta["x"], p.meta["mu"], p.meta["sd"]) as m:
        return m.decode(return_loglik=True)


def test_server_results_same_alone_and_in_the_mix(tvlib):
    import time
    reqs = _mix(7)
    alone = [_alone(tvlib, k, p) for k, p in reqs]
    with tvlib.Server(max_inflight=16) as srv:
        tickets = []
        for i, (k, p) in enumerate(reqs):
            tickets.append(_submit(srv, k, p))
            if i % 5 == 4:
                time.sleep(0.002)  # later arrivals join while earlier ones run
        results = [srv.wait(t) for t in tickets]
        st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    for (path_a, ll_a), (path_s, ll_s, lat, queue) in zip(alone, results):
        np.testing.assert_array_equal(path_s, path_a)
        assert ll_s == ll_a
        assert lat >= queue >= 0.0
    # and the small ones against the oracle
    for (k, p), (path_s, ll_s, _, _) in zip(reqs[:6], results[:6]):
        ref = orc.decode(*p.args(), variant="omp")
        np.testing.assert_array_equal(path_s, ref["path"])
        assert ll_s == ref["loglik"]


def test_server_admission_respects_the_memory_budget(tvlib):
    import tensor_viterbi.synthetic as syn
    reqs = [syn.discrete_problem(10, 50, 20000, 16, 5.0, 40.0, seed=s) for s in range(12)]
    budget = 4 << 20  # a couple of requests at a time
    with tvlib.Server(budget_bytes=budget, max_inflight=16) as srv:
        tickets = [srv.submit(*p.args()) for p in reqs]
        results = [srv.wait(t) for t in tickets]
        st = srv.stats()
    assert st["completed"] == len(reqs)
    assert st["peak_bytes"] <= budget
    for p, (path, ll, _, _) in zip(reqs[:3], results[:3]):
        ref = orc.decode(*p.args(), variant="omp")
        np.testing.assert_array_equal(path, ref["path"])
        assert ll == ref["loglik"]


def test_server_rejects_bad_requests_at_submission(tvlib):
    import tensor_viterbi.synthetic as syn
    p = syn.discrete_problem(5, 40, 30, 8, 5.0, 20.0, seed=1)  # T < D
    with tvlib.Server(max_inflight=2) as srv:
        with pytest.raises(ValueError):
            srv.submit(*p.args())
        q = syn.discrete_problem(5, 10, 100, 8, 5.0, 9.0, seed=2)
        bad = q.obs_seq.copy()
        bad[5] = 8
        with pytest.raises(ValueError):
            srv.submit(*q.model_args(), bad)
        t = srv.submit(*q.args())
        path, ll, _, _ = srv.wait(t)
    ref = orc.decode(*q.args())
    np.testing.assert_array_equal(path, ref["path"])


def test_models_return_all_device_memory(tvlib):
    """Creating, using and destroying models (grid path, window in shared
    memory and in L2, and the Gaussian front-end) leaves the device's free
    memory where it was."""
    import gc
    import torch
    import tensor_viterbi.synthetic as syn
    p = syn.discrete_problem(20, 600, 30000, 16, 20.0, 300.0, seed=9)
    g = _gauss(15, 500, 20000, seed=10, lo=20.0, hi=300.0)

    def churn():
        for kind in ("grid", "grid-l2"):
            with tvlib.Model(*p.model_args()) as m:
                m.set_path(kind, 0)
                m.decode(p.obs_seq)
        with tvlib.GaussianModel(g.n_states, g.trans_mat, g.duration_probs_linear, g.start_probs,
                                 g.duration_probs, g.meta["x"], g.meta["mu"], g.meta["sd"]) as m:
            m.decode()

    churn()  # first use: context and module state
    torch.cuda.synchronize()
    gc.collect()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        churn()
    torch.cuda.synchronize()
    gc.collect()
    free1, _ = torch.cuda.mem_get_info()
    # each churn allocates well over 100 MB (window-sum table, back-pointers)
    assert free0 - free1 < 32 << 20, (free0, free1)


def test_server_latency_mode_for_a_long_request_alone(tvlib):
    """A long request (T*N*D >= 2e8) that arrives alone at an idle server is
    decoded on a grid of several CTAs instead of one CTA: the same result as
    the decode alone and the oracle, in a fraction of the one-CTA time
    (measured on GB300 at N=50, D=100: 13.2 us per step on one CTA, about
    3.5 us on the 10 CTAs chosen)."""
    import time
    import tensor_viterbi.synthetic as syn
    p = syn.discrete_problem(50, 100, 40000, 32, 5.0, 50.0, seed=17)
    with tvlib.Model(*p.model_args()) as m:
        m.set_path("cta")
        m.decode(p.obs_seq)
        t0 = time.perf_counter()
        path_a, ll_a = m.decode(p.obs_seq, return_loglik=True)
        cta_ms = 1e3 * (time.perf_counter() - t0)
    with tvlib.Server() as srv:
        srv.wait(srv.submit(*p.args()))  # warm-up of the grid kernel
        path_s, ll_s, lat, queue = srv.wait(srv.submit(*p.args()))
    np.testing.assert_array_equal(path_s, path_a)
    assert ll_s == ll_a
    ref = orc.decode(*p.args(), variant="omp")
    np.testing.assert_array_equal(path_s, ref["path"])
    assert ll_s == ref["loglik"]
    assert lat - queue < 0.6 * cta_ms, (lat - queue, cta_ms)
