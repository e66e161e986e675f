"""Sharding the 512-problem sweep over ranks (independent problems, no
exchange): two gloo ranks on the CPU each build their share; together the
shares cover every member exactly once, with the same problems (mesh size,
Reynolds number) the single-process sweep draws."""
import os

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp

from goma_gb300 import problem as pb


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = pb.batch_shard(40, 7, rank, world, nmin=2, nmax=6)
    b = pb.batch_sweep_2d(40, seed=7, nmin=2, nmax=6, members=mine)
    work = sum(m.n * m.n for m in b.members)
    got = [None] * world
    dist.all_gather_object(got, (mine, [(m.n, m.re) for m in b.members], work))
    if rank == 0:
        out.put(got)
    dist.destroy_process_group()


def test_two_ranks_partition_the_batch():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    ids = sorted(i for mine, _, _ in got for i in mine)
    assert ids == list(range(40))
    full = pb.batch_sweep_2d(40, seed=7, nmin=2, nmax=6)
    for mine, drawn, _ in got:
        for i, (n, re) in zip(mine, drawn):
            assert full.members[i].n == n and abs(full.members[i].re - re) < 1e-12
    loads = [w for _, _, w in got]
    assert max(loads) - min(loads) <= 6 * 6
