"""Sharding of independent sequences with the GPU decoder: two gloo ranks,
each decoding its longest-processing-time share with one batched launch,
rank 0 gathering the paths and log-likelihoods in input order.  Both ranks
use cuda:0 here (the pool gives one GPU); their kernels are independent
decodes and never wait on each other, as on a multi-GPU node where each rank
has its own device.  The gathered results equal the single-process batched
decode and the oracle."""
import os
import socket
import sys

import numpy as np
import pytest

from conftest import PKG, REPO

pytestmark = pytest.mark.gpu


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, seqs, model_args, out_path):
    import torch
    import torch.distributed as dist
    sys.path[:0] = [str(REPO), str(PKG)]
    from tensor_viterbi import sharding
    from tensor_viterbi.viterbi import native
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    torch.cuda.set_device(0)
    native.configure("gb300", "cuda")
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        with native.Model(*model_args) as m:
            mine = sharding.my_shard([len(s) for s in seqs], ws, rank)
            paths, lls = m.decode_batch([seqs[k] for k in mine], return_loglik=True)
            local = [(k, (p, float(l))) for k, p, l in zip(mine, paths, lls)]
        gathered = [None] * ws if rank == 0 else None
        dist.gather_object(local, gathered, dst=0)
        if rank == 0:
            out = [None] * len(seqs)
            for part in gathered:
                for k, res in part:
                    out[k] = res
            np.savez(out_path, *[r[0] for r in out], lls=np.array([r[1] for r in out]))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_ranks_decode_their_shares_and_gather_on_rank_0(tvlib, tmp_path):
    import torch.multiprocessing as mp
    import tensor_viterbi.synthetic as syn
    from oracle import oracle as orc
    prob, seqs = syn.batch_problem(n_seq=40, N=10, D=60, M=16, lo=200, hi=4000, seed=12)
    model_args = prob.model_args()
    out = tmp_path / "gathered.npz"
    mp.start_processes(_worker, args=(2, _free_port(), seqs, model_args, str(out)), nprocs=2, join=True,
                       start_method="spawn")
    z = np.load(out)
    with tvlib.Model(*model_args) as m:
        paths, lls = m.decode_batch(seqs, return_loglik=True)
    for k, s in enumerate(seqs):
        np.testing.assert_array_equal(z[f"arr_{k}"], paths[k])
        assert float(z["lls"][k]) == float(lls[k])
    for k in range(0, len(seqs), 10):
        ref = orc.decode(*model_args, seqs[k])
        np.testing.assert_array_equal(z[f"arr_{k}"], ref["path"])
        assert float(z["lls"][k]) == ref["loglik"]
