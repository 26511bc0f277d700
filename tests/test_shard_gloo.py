"""The multi-rank split on CPU: two gloo ranks each count their interleaved
share of the engine's first-level tasks (stripes t mod S, restated by the
oracle), the raw 128-bit sums are reduced exactly, and the result equals the
single-process count."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import graphpi_gb300 as gp
from graphpi_gb300 import shard


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from tests import oracle_lib
    orc = oracle_lib.load()
    g = gp.chung_lu(700, 9.0, 2.2, 120, 5)
    tri = orc.triangles(g, 1)
    pats = [gp.Pattern(gp.PatternType.House), gp.Pattern(gp.PatternType.Rectangle), gp.Pattern(4, True)]
    scheds = [gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, tri) for p in pats]
    # the engine's task split (directed edges of the degree-relabelled CSR,
    # or roots), restated by the oracle: rank r takes stripes r, r + N, ...
    g = gp.relabel_by_degree(g)
    stripes = 8
    mine = shard.stripes_of_rank(rank, world, stripes)
    per = orc.stripes_raw(g, [s.tables for s in scheds], stripes, mine, 1)
    raws = [sum(row) for row in per]
    totals = shard.reduce_raw_sums(raws, dist)
    counts = shard.finish(totals, [s.get_in_exclusion_optimize_redundancy() for s in scheds])
    if rank == 0:
        q.put((counts, [orc.count(g, s, 1) for s in scheds]))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.timeout(300)
def test_two_rank_split_equals_single_process(engine):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got, want = q.get(timeout=240)
    for p in procs:
        p.join(timeout=60)
    assert all(p.exitcode == 0 for p in procs)
    assert got == want


def test_stripe_partition_covers_everything():
    for world in (1, 2, 3, 8):
        seen = sorted(s for r in range(world) for s in shard.stripes_of_rank(r, world, 64))
        assert seen == list(range(64))
    assert shard.signed128((1 << 128) - 5) == -5
