"""The multi-process path on CPU: two gloo ranks, each with its own shard, reduce exactly as bench.py does on GPUs."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from dcns_gb300 import ranks as R
from dcns_gb300 import workloads as W


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import oracle as O

        pairs = W.batched_pairs(n_pairs=6, seed=R.shard_seed(rank))
        pairs = [(a[:1500], b[:1500]) for a, b in pairs]
        orc = O.Oracle()
        nf, ck, cells = orc.find_batch(pairs, threads=1)
        elapsed_ms = 10.0 * (rank + 1)  # a fake per-rank step time: rank 1 is the slower one
        dist.barrier()
        slowest = R.max_over_ranks(elapsed_ms, dist)
        total_cells = R.sum_over_ranks(sum(cells.values()), dist)
        rate = R.whole_job_rate(len(pairs), world, slowest)
        first = [int(np.asarray(pairs[0][0])[:64].sum()), ck]
        gathered = [None] * world
        dist.all_gather_object(gathered, first)
        q.put((rank, slowest, total_cells, sum(cells.values()), rate, gathered))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_reduce():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=300) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    cells_each = [o[3] for o in out]
    for rank, slowest, total_cells, _, rate, gathered in out:
        assert slowest == 20.0  # max over ranks, seen identically by both
        assert total_cells == sum(cells_each)  # work of the whole job
        assert rate == pytest.approx(2 * 6 / 0.020)
        assert gathered[0] != gathered[1]  # the shards are different batches
