"""The standard synthetic workloads, shared by tests and the benchmark.

    chung_lu_7k   Chung-Lu, 7,000 vertices, ~100k undirected edges,
                  exponent 2.1, weights capped at degree 1,000, seed 1
                  (triangle / rectangle / 4-clique, perf=1, restricts=1, IEP off)
    rmat_s20      R-MAT scale 20, edge factor 16, (0.57, 0.19, 0.19, 0.05), seed 2
                  (rectangle and house with IEP, one pattern per launch)
    rmat_s22      R-MAT scale 22, same parameters, seed 3
                  (all 29 connected 3-5-vertex motifs in one launch)
    uneven_256    256 Chung-Lu graphs, n log-uniform in [1k, 200k], average
                  degree uniform in [4, 64], exponent uniform in [2.0, 2.8],
                  seeds 100-355, each paired with one 3-5-vertex motif
    rmat_s24      R-MAT scale 24, seed 4 (6-vertex motifs, learned schedules)

Bounded samples of a job are stripes (the first-level tasks t with
t mod S == s); random_stripes draws the stripe ids the benchmark and the
parity tests use.
"""
from __future__ import annotations

import math

from . import api

RMAT = dict(edge_factor=16, a=0.57, b=0.19, c=0.19)


def chung_lu_7k() -> api.Graph:
    return api.chung_lu(7000, 32.0, 2.1, 1000, 1)


def rmat_scale(scale: int, seed: int) -> api.Graph:
    return api.rmat(scale, RMAT["edge_factor"], RMAT["a"], RMAT["b"], RMAT["c"], seed)


def rmat_s20() -> api.Graph:
    return rmat_scale(20, 2)


def rmat_s22() -> api.Graph:
    return rmat_scale(22, 3)


def rmat_s24() -> api.Graph:
    return rmat_scale(24, 4)


def _unit(seed: int, k: int) -> float:
    """Deterministic uniform [0, 1) from (seed, k) (SplitMix64)."""
    x = (seed * 0x9E3779B97F4A7C15 + k * 0xD1B54A32D192ED03 + 0x632BE59BD9B4E019) & 0xFFFFFFFFFFFFFFFF
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    x ^= x >> 31
    return (x >> 11) / float(1 << 53)


def random_stripes(stripes: int, count: int, seed: int = 20261204) -> list[int]:
    """`count` distinct stripe ids in [0, stripes), uniformly drawn from a
    seeded SplitMix64 stream (the same on every machine and numpy version)."""
    M = 0xFFFFFFFFFFFFFFFF
    out, seen, state = [], set(), seed & M
    while len(out) < min(count, stripes):
        state = (state + 0x9E3779B97F4A7C15) & M
        z = state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        z ^= z >> 31
        s = ((z >> 11) * stripes) >> 53
        if s not in seen:
            seen.add(s)
            out.append(s)
    return out


def uneven_params(count: int = 256, first_seed: int = 100, n_lo: int = 1000, n_hi: int = 200000):
    """(n, avg_degree, gamma, seed, motif index in 0..28) for each graph."""
    out = []
    for i in range(count):
        seed = first_seed + i
        n = int(round(math.exp(math.log(n_lo) + _unit(seed, 0) * (math.log(n_hi) - math.log(n_lo)))))
        avg = 4.0 + 60.0 * _unit(seed, 1)
        gamma = 2.0 + 0.8 * _unit(seed, 2)
        motif = min(28, int(_unit(seed, 3) * 29))
        out.append((n, avg, gamma, seed, motif))
    return out


def uneven_graph(n: int, avg: float, gamma: float, seed: int) -> api.Graph:
    # average degree can't exceed n - 1; cap weights at n / 2
    return api.chung_lu(n, min(avg, (n - 1) / 2.0), gamma, max(2, n // 2), seed)


def uneven_benchmark(count: int = 256, steps: int = 3, step_seconds: float = 2.0) -> dict:
    """The uneven batch: `count` Chung-Lu graphs, one motif each, counted in
    one persistent launch per step against one launch per (pattern, graph)
    pair over the same stripe of the work.  The stripe count is the smallest
    power of two (from 2^16 down) whose batched launch stays near
    `step_seconds`; both legs must give the same raw sums."""
    import ctypes as C
    import statistics
    import time

    from . import native
    from .native import U128, check, lib

    motifs = api.motifs_3_to_5()
    t0 = time.time()
    graphs, scheds = [], []
    for n, avg, gamma, seed, m in uneven_params(count):
        g = uneven_graph(n, avg, gamma, seed)
        graphs.append(g)
        scheds.append(api.Schedule(motifs[m], 1, 1, True, g.v_cnt, g.e_cnt, g.triangle_counting_mt()))
    plans = [api.Plan(s) for s in scheds]
    gh = (C.c_void_p * count)(*[g.device() for g in graphs])
    ph = (C.c_void_p * count)(*[p.handle for p in plans])
    red = [s.get_in_exclusion_optimize_redundancy() for s in scheds]
    setup_s = time.time() - t0

    def batched(S: int, stripe: int) -> tuple[float, list[int]]:
        native.set_option("stripes", S)
        native.set_option("stripe", stripe)
        outs = (U128 * count)()
        check(lib().gpm_batch_count(count, gh, ph, outs), "gpm_batch_count")
        return native.last_launch_stats()[0], [o.value for o in outs]

    native.set_option("raw_sums", 1)
    try:
        S = 1 << 16
        while True:
            t, _ = batched(S, S - 1)
            if t >= step_seconds * 1e3 / 4 or S == 1:
                break
            S //= 2
        while S > 1 and t * 2 <= step_seconds * 1e3:
            S //= 2
            t *= 2
        for i in range(3):
            batched(S, steps + i)
        b_ms, p_ms, emb = [], [], 0.0
        for i in range(steps):
            ms, raw = batched(S, i)
            b_ms.append(ms)
            signed = [r - (1 << 128) if r >= (1 << 127) else r for r in raw]
            emb += sum(r / d for r, d in zip(signed, red))
            tot = 0.0
            for j in range(count):
                o = U128()
                check(lib().gpm_count(gh[j], ph[j], C.byref(o)), "gpm_count")
                tot += native.last_launch_stats()[0]
                if o.value != raw[j]:
                    raise AssertionError(f"pair {j}: one-pair launch and batch differ")
            p_ms.append(tot)
    finally:
        native.set_option("stripes", 1)
        native.set_option("stripe", 0)
        native.set_option("raw_sums", 0)
    return {"workload": f"uneven batch, {count} Chung-Lu graphs (1k-200k vertices), one motif each",
            "stripes": S, "steps": steps, "batched_ms_per_step": statistics.median(b_ms),
            "plain_ms_per_step": statistics.median(p_ms),
            "batched_speedup_vs_plain": statistics.median(p_ms) / statistics.median(b_ms),
            "embeddings_per_s": emb / (sum(b_ms) / 1e3), "vertices": sum(g.v_cnt for g in graphs),
            "directed_edges": sum(g.e_cnt for g in graphs), "setup_s": setup_s}


if __name__ == "__main__":
    import json
    import sys

    if len(sys.argv) > 1 and sys.argv[1] == "uneven":
        print(json.dumps(uneven_benchmark(int(sys.argv[2]) if len(sys.argv) > 2 else 256)))
