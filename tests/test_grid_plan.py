"""The grid kernel's launch plan, checked on the host for many shapes.

`tv_grid_plan_info` runs the same planner the launch uses (tv_host.cu,
plan_grid) without a GPU.  These tests hold its invariants: a plan's block
fits the kernel's 640-thread launch bound and holds every role; the head's
roles add up; the matvec split (two warps per 32 states) stays within the
four pair barriers it has; the dynamic shared memory fits the per-CTA limit;
and the bench's shapes get the plans they were measured with.  A violation
here would launch an invalid block or overrun shared memory on the GPU.
"""
import ctypes as C

import numpy as np
import pytest

SMEM_OPTIN = 232448       # GB300: 227 KB of shared memory per CTA
GRID_THREADS = 640        # the kernel's launch bound
WORKER_SMEM = 256 + 64    # scan threads + certify and intake warps, window in shared memory
WORKER_L2 = 512 + 64      # the same with the window in global memory


def plan(N, D, G, force_l2=0, smem=SMEM_OPTIN):
    from tensor_viterbi.viterbi import _lib
    out = np.zeros(10, dtype=np.int64)
    _lib.check(_lib.lib().tv_grid_plan_info(N, D, G, smem, force_l2, out.ctypes.data_as(C.c_void_p)))
    keys = ("ok", "block", "smem", "l2", "split", "S", "max_seg", "head", "qd_smem", "busy")
    return dict(zip(keys, (int(v) for v in out)))


def round32(x):
    return (x + 31) // 32 * 32


@pytest.mark.parametrize("N", [1, 2, 7, 10, 31, 32, 33, 50, 64, 75, 96, 100, 113, 128])
@pytest.mark.parametrize("D", [9, 10, 57, 250, 1000, 5000, 10000, 65535])
@pytest.mark.parametrize("G", [2, 8, 40, 152])
@pytest.mark.parametrize("force_l2", [0, 1])
def test_plan_invariants(tvlib, N, D, G, force_l2):
    p = plan(N, D, G, force_l2)
    if not p["ok"]:
        return
    assert p["block"] <= GRID_THREADS
    assert p["block"] >= p["head"]
    assert p["block"] >= (WORKER_L2 if p["l2"] else WORKER_SMEM)
    cs = round32(N)
    intake = p["head"] - cs * (1 + p["split"]) - 2 * cs
    assert intake >= round32(N) and intake % 32 == 0
    assert 2 * intake >= p["S"]                 # two segments per intake lane
    if p["split"]:
        assert cs <= 128                        # pair barriers 10..13
    assert p["smem"] + 256 <= SMEM_OPTIN
    assert 1 <= p["max_seg"] <= 32
    assert 1 <= p["busy"] <= G - 1
    if force_l2:
        assert p["l2"] == 1
    if not p["l2"]:
        assert p["qd_smem"] == 0


def test_plan_of_the_default_bench_shape(tvlib):
    """N=75 D=5000 on 152 CTAs: each state's window split over two workers,
    the window in shared memory, the matvec split, 480 threads."""
    p = plan(75, 5000, 152)
    assert p["ok"] and not p["l2"] and p["split"] == 1
    assert p["block"] == 480 and p["head"] == 480
    assert p["S"] == 150 and p["max_seg"] == 1 and p["busy"] == 150


def test_plan_of_the_stress_shape(tvlib):
    """N=100 D=1e4 on 152 CTAs: the window goes to global memory, the
    fixed-point duration rows stay in shared memory; the chunks are of equal
    cost, so workers that span two states hold fewer cells and a few CTAs
    may stay idle."""
    p = plan(100, 10_000, 152)
    assert p["ok"] and p["l2"] == 1 and p["qd_smem"] == 1
    assert p["max_seg"] == 2 and 140 <= p["busy"] <= 151
    assert p["S"] < 151 + 99                   # fewer chunks cross a state boundary than equal cuts would
    assert p["block"] == max(p["head"], WORKER_L2)


def test_plan_refuses_what_the_kernel_cannot_take(tvlib):
    assert not plan(129, 100, 152)["ok"]       # packed coarse scores keep the index in 7 bits
    assert not plan(10, 8, 152)["ok"]          # D must exceed the head's lead L = 8
    assert not plan(10, 100, 1)["ok"]          # a head needs at least one worker


def test_plan_rejects_bad_arguments(tvlib):
    with pytest.raises(ValueError):
        plan(0, 100, 152)
