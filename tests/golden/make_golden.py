"""Generates the golden fixtures in this folder from the reference GraphPi
itself (oracle/_ref/libgraphpi_ref.so, built from the reference sources by
oracle/build_ref.sh).  Run where the reference checkout exists, naming it:

    GRAPHPI_REFERENCE=<reference checkout> python tests/golden/make_golden.py

Writes
  schedules.json  reference Schedule tables (gpm_schedule_build layout) for
                  every connected 3-5-vertex motif under several
                  (performance_modeling_type, restricts_type, IEP) settings,
                  and every 6-vertex motif under (1, 1, IEP on)
  counts.json     reference Graph::pattern_matching counts on seeded
                  synthetic graphs (generated by this library's own
                  deterministic generators; each graph is identified by a
                  checksum of its CSR) and the Wiki-Vote dataset figures
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import graphpi_gb300 as gp  # noqa: E402
from graphpi_gb300 import workloads  # noqa: E402

REF = ROOT / "oracle" / "_ref" / "libgraphpi_ref.so"
if not os.environ.get("GRAPHPI_REFERENCE"):
    sys.exit("set GRAPHPI_REFERENCE to the reference checkout")
WIKI = Path(os.environ["GRAPHPI_REFERENCE"]) / "dataset" / "wiki-vote_input"
OUT = Path(__file__).resolve().parent


def load_ref():
    R = C.CDLL(str(REF))
    R.ref_graph_from_csr.restype = C.c_void_p
    R.ref_graph_from_csr.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_longlong, C.c_int]
    R.ref_graph_free.argtypes = [C.c_void_p]
    R.ref_graph_tri.restype = C.c_longlong
    R.ref_graph_tri.argtypes = [C.c_void_p]
    R.ref_schedule_create.restype = C.c_void_p
    R.ref_schedule_create.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint,
                                      C.c_longlong, C.POINTER(C.c_int)]
    R.ref_schedule_dump.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    R.ref_schedule_free.argtypes = [C.c_void_p]
    R.ref_pattern_matching.restype = C.c_longlong
    R.ref_pattern_matching.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    R.ref_triangle_counting_mt.restype = C.c_longlong
    R.ref_triangle_counting_mt.argtypes = [C.c_void_p, C.c_int]
    R.ref_motifs.argtypes = [C.c_int, C.c_void_p, C.c_int]
    return R


def csr_checksum(g: gp.Graph) -> str:
    h = hashlib.sha256()
    h.update(np.int64(g.v_cnt).tobytes())
    h.update(g.vertex.astype("<u4").tobytes())
    h.update(g.edge.astype("<i4").tobytes())
    return h.hexdigest()[:16]


def ref_schedule(R, adj, perf, restr, iep, v, e, tri):
    a = np.ascontiguousarray(adj, dtype=np.int32)
    ok = C.c_int()
    s = R.ref_schedule_create(a.shape[0], a.ctypes.data, perf, restr, iep, v, e, tri, C.byref(ok))
    buf = np.zeros(16384, dtype=np.int64)
    k = R.ref_schedule_dump(s, buf.ctypes.data, len(buf)) if ok.value else 0
    return s, bool(ok.value), buf[:k].tolist()


# graphs: name -> (generator call, pattern sets, schedule flags)
GRAPHS = {
    # the reference's own CPU-sized case: triangle, rectangle, 4-clique;
    # perf=1, restricts=1, IEP off
    "chung_lu_7k": (workloads.chung_lu_7k, "c1", (1, 1, 0)),
    # all 29 motifs with IEP, small enough for the reference to finish fast
    "rmat_s10": (lambda: gp.rmat(10, 16, 0.57, 0.19, 0.19, 2), "motifs", (1, 1, 1)),
    "chung_lu_2k": (lambda: gp.chung_lu(2000, 12.0, 2.3, 300, 7), "motifs", (1, 1, 1)),
    "rmat_s12_noiep": (lambda: gp.rmat(12, 8, 0.57, 0.19, 0.19, 5), "motifs4", (1, 1, 0)),
}


def main() -> None:
    R = load_ref()
    # ---- schedule tables ----
    wiki_stats = (7115, 201524, 608389)
    flags = [(1, 1, 1), (0, 0, 0), (1, 1, 0), (0, 1, 1), (1, 0, 1), (2, 2, 0), (3, 1, 1), (0, 2, 1)]
    sched = []
    for k in (3, 4, 5, 6):
        for p in gp.MotifGenerator(k).generate():
            for fl in (flags if k <= 5 else [(1, 1, 1)]):
                s, ok, t = ref_schedule(R, p.adj, *fl, *wiki_stats)
                R.ref_schedule_free(s)
                sched.append({"adj": p.adj.reshape(-1).tolist(), "n": k, "flags": list(fl),
                              "stats": list(wiki_stats), "valid": ok, "tables": t})
    # motif order/count straight from the reference generator
    motif_ref = {}
    for k in (3, 4, 5, 6):
        buf = np.zeros(200 * k * k, dtype=np.int32)
        cnt = R.ref_motifs(k, buf.ctypes.data, 200)
        motif_ref[str(k)] = [buf[i * k * k:(i + 1) * k * k].tolist() for i in range(cnt)]
    (OUT / "schedules.json").write_text(json.dumps({"schedules": sched, "motifs": motif_ref}, separators=(",", ":")))

    # ---- counts ----
    counts = {"graphs": {}}
    pats = {
        "c1": [("triangle", gp.Pattern(3, True)), ("rectangle", gp.Pattern(gp.PatternType.Rectangle)),
               ("clique4", gp.Pattern(4, True))],
        "motifs": [(f"m{k}_{i}", p) for k in (3, 4, 5) for i, p in enumerate(gp.MotifGenerator(k).generate())],
        "motifs4": [(f"m{k}_{i}", p) for k in (3, 4) for i, p in enumerate(gp.MotifGenerator(k).generate())],
    }
    for name, (make, pset, fl) in GRAPHS.items():
        g = make()
        rg = R.ref_graph_from_csr(g.v_cnt, g.vertex.ctypes.data, g.edge.ctypes.data, -1, 8)
        tri = R.ref_graph_tri(rg)
        entry = {"checksum": csr_checksum(g), "v_cnt": g.v_cnt, "e_cnt": g.e_cnt, "tri_cnt": tri,
                 "flags": list(fl), "counts": {}, "adj": {}}
        for pname, p in pats[pset]:
            s, ok, t = ref_schedule(R, p.adj, *fl, g.v_cnt, g.e_cnt, tri)
            assert ok
            c = R.ref_pattern_matching(rg, s, 8)
            R.ref_schedule_free(s)
            entry["counts"][pname] = c
            entry["adj"][pname] = p.adj.reshape(-1).tolist()
        R.ref_graph_free(rg)
        counts["graphs"][name] = entry
        print(name, g.v_cnt, g.e_cnt, tri, len(entry["counts"]), flush=True)
    # Wiki-Vote figures (reference DataLoader + pattern_matching, 24 threads
    # in tianhe/baseline_test.cpp; thread count does not change counts)
    counts["wiki_vote"] = {"tri_cnt": 608389, "rectangle": 57654491, "clique4": 2077903, "house": 9488779111}
    (OUT / "counts.json").write_text(json.dumps(counts, indent=1))


if __name__ == "__main__":
    main()
