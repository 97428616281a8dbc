"""The decode entry point that allocates no device memory.

Some callers cannot call cudaMalloc while they decode: code inside a CUDA
graph capture or a stream callback, latency-critical loops where an
allocation can stall on the driver, and processes whose device memory is
reserved up front by a pool.  `tv_decode_device_static` serves them from a
fixed array compiled into the library.  This test calls it through the C ABI
twice in a row, on two different sequences, and checks each result against
the ordinary allocating entry point `tv_decode_device`: paths bit-exact and
log-likelihoods equal, the bar of every other parity test here.  It lives in
its own file, collected last, so a failure here cannot hide another test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _decode_both(tvlib, model, obs_np):
    import torch
    from tensor_viterbi.viterbi import _lib

    L = _lib.lib()
    stream = torch.cuda.current_stream().cuda_stream
    obs = torch.from_numpy(obs_np).cuda()
    T = obs.numel()
    ref_path = torch.full_like(obs, -1)
    ref_ll = torch.zeros(1, dtype=torch.float64, device="cuda")
    _lib.check(L.tv_decode_device(model.handle, C.c_void_p(obs.data_ptr()), T, C.c_void_p(ref_path.data_ptr()),
                                  C.c_void_p(ref_ll.data_ptr()), C.c_void_p(stream)))
    path = torch.full_like(obs, -1)
    ll = torch.zeros(1, dtype=torch.float64, device="cuda")
    status = torch.full((1,), 12345, dtype=torch.int32, device="cuda")
    _lib.check(L.tv_decode_device_static(model.handle, C.c_void_p(obs.data_ptr()), T, C.c_void_p(path.data_ptr()),
                                         C.c_void_p(ll.data_ptr()), C.c_void_p(status.data_ptr()),
                                         C.c_void_p(stream)))
    torch.cuda.synchronize()
    return ref_path.cpu().numpy(), float(ref_ll.item()), path.cpu().numpy(), float(ll.item()), int(status.item())


def test_fixed_scratch_entry_matches_allocating_entry_twice(tvlib):
    import tensor_viterbi.synthetic as syn

    prob, seqs = syn.batch_problem(n_seq=2, N=10, D=120, M=16, lo=2000, hi=6000, seed=31)
    with tvlib.Model(*prob.model_args()) as m:
        results = [_decode_both(tvlib, m, s) for s in seqs]  # two fixed-scratch calls in a row
    for ref_path, ref_ll, path, ll, status in results:
        assert status == 0
        np.testing.assert_array_equal(path, ref_path)
        assert ll == ref_ll
    # the second call did not reuse the first call's back-pointers
    assert not np.array_equal(results[0][2][:50], results[1][2][:50]) or len(seqs[0]) != len(seqs[1])


def test_fixed_scratch_entry_rejects_oversized_problems(tvlib):
    import torch
    import tensor_viterbi.synthetic as syn
    from tensor_viterbi.viterbi import _lib

    # T*N back-pointers beyond the fixed array: refused before any launch
    prob, _ = syn.batch_problem(n_seq=1, N=64, D=20, M=8, lo=1000, hi=1001, seed=1)
    T = _lib.TV_STATIC_SCRATCH_BYTES // (4 * 64) + 16
    obs = torch.zeros(T, dtype=torch.int32, device="cuda")
    out = torch.empty_like(obs)
    with tvlib.Model(*prob.model_args()) as m:
        with pytest.raises(ValueError, match="scratch"):
            m.decode_device_static(obs.data_ptr(), T, out.data_ptr())


def test_fixed_scratch_entry_replays_from_a_cuda_graph(tvlib):
    """A serving loop's form: the decode captured once in a CUDA graph, then
    replayed for new observations copied into the captured input buffer.
    Every replay equals the allocating entry point on the same sequence."""
    import torch
    import tensor_viterbi.synthetic as syn

    prob, seqs = syn.batch_problem(n_seq=4, N=8, D=90, M=12, lo=3000, hi=3001, seed=41)
    T = min(s.size for s in seqs)
    seqs = [np.ascontiguousarray(s[:T]) for s in seqs]
    with tvlib.Model(*prob.model_args()) as m:
        obs = torch.from_numpy(seqs[0]).cuda()
        path = torch.full_like(obs, -1)
        ll = torch.zeros(1, dtype=torch.float64, device="cuda")
        status = torch.full((1,), 12345, dtype=torch.int32, device="cuda")
        # one-time set-up of the fixed scratch, before any capture
        m.decode_device_static(obs.data_ptr(), T, path.data_ptr(), ll.data_ptr(), status.data_ptr(),
                               torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            m.decode_device_static(obs.data_ptr(), T, path.data_ptr(), ll.data_ptr(), status.data_ptr(),
                                   torch.cuda.current_stream().cuda_stream)
        for s in seqs[1:] + seqs[:1]:
            obs.copy_(torch.from_numpy(s))
            path.fill_(-1)
            g.replay()
            torch.cuda.synchronize()
            ref_path, ref_ll = m.decode(s, return_loglik=True)
            assert int(status.item()) == 0
            np.testing.assert_array_equal(path.cpu().numpy(), ref_path)
            assert float(ll.item()) == ref_ll


def test_fixed_scratch_entry_after_allocating_decode_of_smaller_window(tvlib):
    """The kernel's shared-memory limit is process-wide state.  After the
    fixed-scratch set-up, an allocating decode of a model with a small window,
    then a fixed-scratch decode of a model with a much larger window: the
    second must still launch and equal the oracle."""
    import torch
    import tensor_viterbi.synthetic as syn
    from oracle import oracle as orc

    small = syn.discrete_problem(4, 20, 600, 6, 3.0, 12.0, seed=5)
    big = syn.discrete_problem(30, 180, 900, 12, 10.0, 90.0, seed=6)  # 34*N*D + 8*N*N ~ 191 KB
    stream = torch.cuda.current_stream().cuda_stream
    with tvlib.Model(*big.model_args()) as mb, tvlib.Model(*small.model_args()) as ms:
        obs_b = torch.from_numpy(big.obs_seq).cuda()
        path_b = torch.full_like(obs_b, -1)
        ll_b = torch.zeros(1, dtype=torch.float64, device="cuda")
        mb.decode_device_static(obs_b.data_ptr(), obs_b.numel(), path_b.data_ptr(), ll_b.data_ptr(), 0, stream)
        torch.cuda.synchronize()
        ps, lls = ms.decode(small.obs_seq, return_loglik=True)  # small window through the allocating path
        path_b.fill_(-1)
        mb.decode_device_static(obs_b.data_ptr(), obs_b.numel(), path_b.data_ptr(), ll_b.data_ptr(), 0, stream)
        torch.cuda.synchronize()
        got_b, got_llb = path_b.cpu().numpy(), float(ll_b.item())
    ref_s = orc.decode(*small.args())
    ref_b = orc.decode(*big.args(), variant="omp")
    np.testing.assert_array_equal(ps, ref_s["path"])
    assert lls == ref_s["loglik"]
    np.testing.assert_array_equal(got_b, ref_b["path"])
    assert got_llb == ref_b["loglik"]


def test_fixed_scratch_entry_size_limit_is_exact(tvlib):
    """The scratch bound stated in the header, r(8ON) + r(8NN) + r(8ND) + 256
    + 4TN with r() rounding up to 256 bytes: a problem that needs exactly the
    whole array decodes (and equals the allocating entry point); one more
    step is refused."""
    import torch
    import tensor_viterbi.synthetic as syn
    from tensor_viterbi.viterbi import _lib

    N, O, D = 10, 16, 100
    r = lambda x: (x + 255) // 256 * 256
    fixed = r(8 * O * N) + r(8 * N * N) + r(8 * N * D) + 256
    T = (_lib.TV_STATIC_SCRATCH_BYTES - fixed) // (4 * N)
    assert fixed + 4 * T * N == _lib.TV_STATIC_SCRATCH_BYTES  # this shape fills the array exactly
    p = syn.discrete_problem(N, D, T + 1, O, 5.0, 50.0, seed=9)
    with tvlib.Model(*p.model_args()) as m:
        ref_path, ref_ll, path, ll, status = _decode_both(tvlib, m, np.ascontiguousarray(p.obs_seq[:T]))
        obs = torch.from_numpy(p.obs_seq).cuda()
        out = torch.empty_like(obs)
        with pytest.raises(ValueError, match="scratch"):
            m.decode_device_static(obs.data_ptr(), T + 1, out.data_ptr())
    assert status == 0
    np.testing.assert_array_equal(path, ref_path)
    assert ll == ref_ll
