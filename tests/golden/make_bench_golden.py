"""Generates tests/golden/bench_stripes.json from the reference GraphPi itself
(oracle/_ref/libgraphpi_ref.so, built from the reference sources by
oracle/build_ref.sh) at the benchmark sizes.  Run where the reference
checkout exists (takes tens of minutes on 8 cores):

    python tests/golden/make_bench_golden.py

For each benchmark graph it records
  * the graph's identity (generator, size, CSR checksum) and the reference's
    triangle count (Graph::triangle_counting_mt, src/graph.cpp:112-139),
  * the reference Schedule tables (gpm_schedule_build layout) the benchmark
    counts with: performance_modeling_type 1, restricts_type 1, IEP on, built
    for the graph's v_cnt / e_cnt / tri_cnt (src/schedule.cpp:9-253),
  * the reference's undivided sums over seeded random stripes of the
    first-level tasks of the degree-relabelled CSR (the numbering the GPU
    engine counts on): the task split of ref_stripes_raw in
    oracle/ref_shim.cpp, i.e. the reference's own root-loop body, depth-1
    iteration and pattern_matching_aggressive_func.
The CPU oracle's sums are computed too and must agree before anything is
written.

    rmat_s22  R-MAT scale 22, seed 3: all 29 connected 3-5-vertex motifs
    rmat_s20  R-MAT scale 20, seed 2: rectangle and house
"""
from __future__ import annotations

import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import graphpi_gb300 as gp  # noqa: E402
from graphpi_gb300 import workloads  # noqa: E402
from tests import oracle_lib  # noqa: E402

OUT = Path(__file__).resolve().parent / "bench_stripes.json"

BENCH = {
    "rmat_s22": dict(scale=22, seed=3, patterns="motifs", stripes=1 << 23, count=48),
    "rmat_s20": dict(scale=20, seed=2, patterns="c2", stripes=1 << 16, count=16),
}


def patterns(kind: str):
    if kind == "motifs":
        return [(f"m{i}", p) for i, p in enumerate(gp.motifs_3_to_5())]
    return [("rectangle", gp.Pattern(gp.PatternType.Rectangle)), ("house", gp.Pattern(gp.PatternType.House))]


def main() -> None:
    R = oracle_lib.load_ref()
    orc = oracle_lib.load()
    threads = 8
    out = {}
    for name, cfg in BENCH.items():
        t0 = time.time()
        g0 = workloads.rmat_scale(cfg["scale"], cfg["seed"])
        g = gp.relabel_by_degree(g0)
        rg = R.ref_graph_from_csr(g.v_cnt, g.vertex.ctypes.data, g.edge.ctypes.data, -1, threads)
        tri = R.ref_graph_tri(rg)
        S = cfg["stripes"]
        ids = workloads.random_stripes(S, cfg["count"])
        ids_arr = np.ascontiguousarray(ids, dtype=np.int64)
        entry = {"scale": cfg["scale"], "seed": cfg["seed"], "v_cnt": g.v_cnt, "e_cnt": g.e_cnt,
                 "checksum": oracle_lib.csr_checksum(g0), "relabelled_checksum": oracle_lib.csr_checksum(g),
                 "tri_cnt": tri, "flags": [1, 1, 1], "stripes": S, "ids": ids, "names": [], "adj": [],
                 "tables": [], "raw": []}
        print(f"{name}: {g.v_cnt} v, {g.e_cnt} e, tri {tri} ({time.time() - t0:.1f} s)", flush=True)
        for pname, p in patterns(cfg["patterns"]):
            t1 = time.time()
            tabs, ok = oracle_lib.ref_schedule_tables(R, p.adj, 1, 1, True, g.v_cnt, g.e_cnt, tri)
            assert ok, pname
            a = np.ascontiguousarray(p.adj, dtype=np.int32)
            okc = oracle_lib.C.c_int()
            rs = R.ref_schedule_create(a.shape[0], a.ctypes.data, 1, 1, 1, g.v_cnt, g.e_cnt, tri, oracle_lib.C.byref(okc))
            ref = np.zeros(len(ids), dtype=np.int64)
            R.ref_stripes_raw(rg, rs, S, ids_arr.ctypes.data, len(ids), threads, ref.ctypes.data)
            R.ref_schedule_free(rs)
            mine = orc.stripes_raw(g, [tabs], S, ids, threads)[0]
            for j, (x, y) in enumerate(zip(ref.tolist(), mine)):
                assert (x - y) % (1 << 64) == 0, (name, pname, ids[j], x, y)
            entry["names"].append(pname)
            entry["adj"].append(p.adj.reshape(-1).tolist())
            entry["tables"].append(tabs)
            entry["raw"].append(mine)
            print(f"  {pname}: {time.time() - t1:.1f} s, sum {sum(mine)}", flush=True)
        R.ref_graph_free(rg)
        out[name] = entry
        OUT.write_text(json.dumps(out, separators=(",", ":")))


if __name__ == "__main__":
    main()
