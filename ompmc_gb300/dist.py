"""Several GPUs: independent history shards and one tally reduction.

Histories are independent, so a job splits across ranks with no exchange
during transport: rank r takes its share of the histories and the RANMAR
streams that follow the streams of ranks 0..r-1 (stream k of the job is the
seed pair (ixx, jxx + k) continued past 31328, the reference's per-thread
seeding, omc_random.c:72).  At the end the per-rank batch sums are added
once (an all-reduce, or a gather on rank 0).  The reference has no
distributed path at all; this is the data-parallel layer above its
transport call.
"""

from __future__ import annotations

import numpy as np

from . import api


def shard(nperbatch: int, world: int, rank: int) -> int:
    """Histories per batch of rank `rank` (the remainder goes to the first
    ranks)."""
    base, extra = divmod(int(nperbatch), int(world))
    return base + (1 if rank < extra else 0)


def rank_seeds(ixx: int, jxx: int, rank: int, lanes_per_rank: int):
    """Seed pair whose streams 0..lanes_per_rank-1 are the job's streams
    rank*lanes_per_rank ... (rank+1)*lanes_per_rank-1."""
    return api.stream_seeds(ixx, jxx, rank * lanes_per_rank)


def reduce_tallies(acc: np.ndarray, acc2: np.ndarray, ensrc: float):
    """Sum the batch sums of every rank (torch.distributed must be
    initialised; works with the gloo and nccl backends).

    Each (rank, batch) pair is one statistical batch of the job: with W
    ranks of nbatch batches the result holds W*nbatch batches of
    nperbatch/W histories, which is what accumulateResults needs
    (omc_dosxyz.c:739-751); summing the squares of per-rank batches is
    exact under that reading."""
    import torch
    import torch.distributed as dist

    t = torch.from_numpy(np.concatenate([acc, acc2, [ensrc]]).astype(np.float64))
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    t = t.cpu().numpy()
    n = acc.shape[0]
    return t[:n], t[n:2 * n], float(t[-1])
