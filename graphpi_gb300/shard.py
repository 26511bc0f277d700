"""Splitting one counting job across ranks (one GPU each).

The first-level work of every (pattern, graph) pair is cut into interleaved
stripes (engine options "stripes"/"stripe"); rank r of N takes stripes
r, r + N, ...  Each rank returns undivided signed 128-bit sums
("raw_sums"), the ranks add them exactly, and the total is divided by each
schedule's redundancy — the reference divides its summed long long the same
way (src/graph.cpp:244).  No data-path collective: one reduction at the end.
"""
from __future__ import annotations


def stripes_of_rank(rank: int, world: int, stripes: int) -> list[int]:
    return list(range(rank, stripes, world))


def signed128(v: int) -> int:
    return v - (1 << 128) if v >= (1 << 127) else v


def reduce_raw_sums(raws: list[int], dist=None) -> list[int]:
    """Exact sum of per-rank raw sums (Python ints) over the process group."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return list(raws)
    gathered = [None] * dist.get_world_size()
    dist.all_gather_object(gathered, [int(r) for r in raws])
    return [sum(col) for col in zip(*gathered)]


def finish(raw_totals: list[int], redundancies: list[int]) -> list[int]:
    out = []
    for t, d in zip(raw_totals, redundancies):
        if t < 0:
            raise OverflowError("negative raw total")
        out.append(t // d)
    return out
