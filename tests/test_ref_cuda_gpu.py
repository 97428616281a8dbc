"""The reference project's own CUDA backend on this GPU: parity and time.

The reference kernels (src/kernels.cu, compiled for sm_103a with the
reference's CUDA flags by oracle/build_ref.sh) run under oracle/ref_cuda.c,
which launches them as src/hsmm.cu:604-791 does.  Checked here:
  * their path, final scores and log-likelihood equal, bit for bit, the CPU
    restatement of the CUDA backend (oracle/tv_oracle_cuda.c, with the
    device's log for the tail's log-survival), on every golden fixture;
  * their agreement with the reference's C++ decoder, case by case, is the
    one recorded in tests/golden/ref_cuda_agreement.json, where each
    disagreement is traced to one of the CUDA backend's four differences;
  * on the single-sequence bench model (N=75, D=5000) at T = 12000, their path
    is the recorded CUDA path, and the time of both decoders is printed
    (REF_CUDA_TIMING lines).
This decoder follows the C++ decoder, so where the two reference backends
disagree it agrees with the C++ one (test_headline_gpu.py, test_decode_gpu.py).
The tests skip when the reference kernels were not built (no reference
checkout where the repository was prepared).
"""
import hashlib
import json
import time

import numpy as np
import pytest

from conftest import GOLDEN, golden_names, load_golden
from oracle import oracle as orc

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(orc.ref_cuda_files() is None,
                                 reason="reference CUDA kernels not built (oracle/build_ref.sh needs the checkout)")]


def _table():
    return json.loads((GOLDEN / "ref_cuda_agreement.json").read_text())["cases"]


def _sha(path):
    return hashlib.sha256(np.ascontiguousarray(path, dtype=np.int32).tobytes()).hexdigest()


def _device_log_suffix(n_states, lin):
    """log of the kernels' linear suffix sums, taken on the device."""
    import torch
    s = torch.from_numpy(orc.lin_suffix(n_states, lin)).cuda()
    return torch.log(s).cpu().numpy()


def _cases():
    import sys
    from conftest import REPO
    sys.path.insert(0, str(REPO / "tests" / "golden"))
    import make_ref_cuda_table as mk
    out = [(n, load_golden(n)[0]) for n in golden_names()]
    return out + mk.tie_cases()


# The reference's tail kernel reduces over 16 shuffle lanes whatever its block
# size (src/kernels.cu:461-465); below one warp (min(T-1, D) <= 16) it reads
# lanes outside the block, whose values are undefined, so those fixtures are
# not run on the reference kernels.
def _tail_block_is_a_warp(args):
    return min(np.asarray(args[6]).size - 1, np.asarray(args[5]).shape[0]) > 16


@pytest.mark.parametrize("name,args", _cases(), ids=[c[0] for c in _cases()])
def test_reference_cuda_kernels_match_their_cpu_restatement(tvlib, name, args):
    if not _tail_block_is_a_warp(args):
        pytest.skip("the reference tail kernel reads shuffle lanes outside a sub-warp block (undefined values)")
    got = orc.ref_cuda_decode(*args)
    want = orc.decode_cuda_semantics(*args, flags=orc.CU_ALL, log_suffix=_device_log_suffix(args[0], args[3]))
    np.testing.assert_array_equal(got["path"], want["path"])
    np.testing.assert_array_equal(got["final"], want["final"])
    assert got["loglik"] == want["loglik"]
    row = _table()[name]
    assert _sha(got["path"]) == row["cuda_path_sha256"]
    cpp = orc.decode(*args)
    assert bool(np.array_equal(got["path"], cpp["path"])) == row["cuda_path_equals_cpp"]


def _best_ms(fn, reps=3):
    best = None
    for _ in range(reps):
        t0 = time.perf_counter()
        out = fn()
        dt = 1e3 * (time.perf_counter() - t0)
        best = dt if best is None or dt < best else best
    return best, out


def test_reference_cuda_on_the_bench_model_and_time(tvlib, c1_case):
    """N=75, D=5000, M=32 at T = 12000 (2D + 2000): the reference kernels'
    path is the recorded CUDA path; ours is the C++ decoder's (the oracle).
    Times: the reference's whole decode call (allocations, uploads, 2 launches
    per step, copies, host backtrace) and its kernels alone, against this
    decoder's drop-in one-shot call and its device-resident decode."""
    import torch
    args, ref = c1_case
    row = _table()["bench_N75_D5000_prefix12000"]
    ms_call, got = _best_ms(lambda: orc.ref_cuda_decode(*args), reps=2)
    assert _sha(got["path"]) == row["cuda_path_sha256"]
    assert bool(np.array_equal(got["path"], ref["path"])) == row["cuda_path_equals_cpp"]

    ours_call, (path, ll) = _best_ms(lambda: tvlib.decode_tensor_viterbi_cuda_loglik(*args))
    np.testing.assert_array_equal(path, ref["path"])
    assert ll == ref["loglik"]
    with tvlib.Model(*args[:6]) as m:
        obs = torch.from_numpy(args[6]).cuda()
        out = torch.empty_like(obs)
        s = torch.cuda.current_stream()
        m.decode_device(obs.data_ptr(), obs.numel(), out.data_ptr(), 0, s.cuda_stream)
        torch.cuda.synchronize()
        dev = []
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            m.decode_device(obs.data_ptr(), obs.numel(), out.data_ptr(), 0, s.cuda_stream)
            e1.record(s)
            e1.synchronize()
            dev.append(e0.elapsed_time(e1))
    T = args[6].size
    rec = {"case": "N75_D5000_M32_T12000", "steps": T,
           "reference_cuda_call_ms": got["ms_call"], "reference_cuda_kernels_ms": got["ms_kernels"],
           "reference_cuda_us_per_step": 1e3 * got["ms_kernels"] / T,
           "ours_dropin_call_ms": ours_call, "ours_device_ms": min(dev), "ours_us_per_step": 1e3 * min(dev) / T}
    print("REF_CUDA_TIMING " + json.dumps(rec))
    assert min(dev) < got["ms_kernels"]


def test_reference_cuda_time_on_config0(tvlib):
    """N=10, D=100, T=1000, M=16 (the reference's CPU-runnable shape): both
    decoders' whole calls, best of five after a warm-up."""
    import tensor_viterbi.synthetic as syn
    p = syn.config0()
    orc.ref_cuda_decode(*p.args())
    tvlib.decode_tensor_viterbi_cuda(*p.args())
    ref_ms, got = _best_ms(lambda: orc.ref_cuda_decode(*p.args()), reps=5)
    ours_ms, path = _best_ms(lambda: tvlib.decode_tensor_viterbi_cuda(*p.args()), reps=5)
    ref = orc.decode(*p.args())
    np.testing.assert_array_equal(path, ref["path"])
    rec = {"case": "N10_D100_M16_T1000", "steps": p.T, "reference_cuda_call_ms": got["ms_call"],
           "reference_cuda_kernels_ms": got["ms_kernels"], "reference_cuda_python_ms": ref_ms,
           "ours_dropin_call_ms": ours_ms,
           "cuda_path_equals_cpp": bool(np.array_equal(got["path"], ref["path"]))}
    print("REF_CUDA_TIMING " + json.dumps(rec))
