"""Sharding of independent sequences across ranks (CPU): the LPT assignment
and the gather on rank 0, run as two gloo processes on 127.0.0.1."""
import os
import socket
import sys

import numpy as np
import pytest

from conftest import PKG, REPO


def _sharding():
    sys.path.insert(0, str(PKG))
    from tensor_viterbi import sharding
    return sharding


@pytest.mark.parametrize("ws", [1, 2, 3, 8])
def test_lpt_shards_cover_once_and_balance(ws):
    sh = _sharding()
    rng = np.random.default_rng(ws)
    costs = np.exp(rng.uniform(np.log(1e3), np.log(1e5), 500)).astype(np.int64)
    shards = sh.lpt_shards(costs, ws)
    flat = sorted(k for s in shards for k in s)
    assert flat == list(range(costs.size))
    loads = [costs[s].sum() for s in shards]
    assert max(loads) - min(loads) <= costs.max()
    assert all(s == sorted(s) for s in shards)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, seqs, model_args, out_path):
    import torch.distributed as dist
    sys.path[:0] = [str(REPO), str(PKG)]
    from tensor_viterbi import sharding
    from oracle import oracle as orc
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        res = sharding.decode_sharded(lambda s: orc.decode(*model_args, s)["path"], seqs)
        if rank == 0:
            np.savez(out_path, *res)
        else:
            assert res is None
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_sharded_decode_gathers_every_result_on_rank_0(tmp_path):
    import torch.multiprocessing as mp
    sys.path.insert(0, str(PKG))
    import tensor_viterbi.synthetic as syn
    from oracle import oracle as orc
    prob, seqs = syn.batch_problem(n_seq=9, N=5, D=30, M=8, lo=100, hi=900, seed=4)
    model_args = prob.model_args()
    out = tmp_path / "gathered.npz"
    mp.start_processes(_worker, args=(2, _free_port(), seqs, model_args, str(out)), nprocs=2, join=True,
                       start_method="spawn")
    z = np.load(out)
    got = [z[f"arr_{k}"] for k in range(len(seqs))]
    for s, g in zip(seqs, got):
        np.testing.assert_array_equal(g, orc.decode(*model_args, s)["path"])
