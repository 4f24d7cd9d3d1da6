"""Multi-rank layer on CPU (gloo, world size 2): history shards, disjoint
RANMAR streams per rank, and the single tally reduction."""

import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from ompmc_gb300 import dist as D

    n = D.shard(1001, world, rank)
    acc = np.full(5, float(rank + 1))
    acc2 = acc * acc
    a, a2, e = D.reduce_tallies(acc, acc2, ensrc=10.0 * (rank + 1))
    out[rank] = (n, a.tolist(), a2.tolist(), e)
    dist.destroy_process_group()


def test_two_rank_reduction_and_shards(native):
    import socket

    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    assert out[0][0] + out[1][0] == 1001 and out[0][0] == 501
    for r in range(2):
        assert out[r][1] == [3.0] * 5      # 1 + 2
        assert out[r][2] == [5.0] * 5      # 1 + 4
        assert out[r][3] == 30.0


def test_rank_streams_are_disjoint(native):
    from ompmc_gb300 import api
    from ompmc_gb300 import dist as D

    lanes = 5000
    s0 = D.rank_seeds(97, 33, 0, lanes)
    s1 = D.rank_seeds(97, 33, 1, lanes)
    set0 = {api.stream_seeds(*s0, k) for k in range(lanes)}
    set1 = {api.stream_seeds(*s1, k) for k in range(lanes)}
    assert not (set0 & set1)
    # rank r's lane k is the job's stream r*lanes + k
    assert api.stream_seeds(*s1, 7) == api.stream_seeds(97, 33, lanes + 7)
