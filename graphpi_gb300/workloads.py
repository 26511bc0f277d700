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
