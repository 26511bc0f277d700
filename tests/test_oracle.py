"""Pins the CPU oracle: against the reference's recorded outputs (golden
fixtures), against the reference library itself where it was built here,
and against the definition-level brute-force counter."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

import graphpi_gb300 as gp
from graphpi_gb300 import workloads
from tests.oracle_lib import REF_LIB, csr_checksum, golden, reference_root

COUNTS = golden("counts.json")
_REF = reference_root()
WIKI = _REF / "dataset" / "wiki-vote_input" if _REF else None

GEN = {
    "chung_lu_7k": workloads.chung_lu_7k,
    "rmat_s10": lambda: gp.rmat(10, 16, 0.57, 0.19, 0.19, 2),
    "chung_lu_2k": lambda: gp.chung_lu(2000, 12.0, 2.3, 300, 7),
    "rmat_s12_noiep": lambda: gp.rmat(12, 8, 0.57, 0.19, 0.19, 5),
}


@pytest.mark.parametrize("name", list(GEN))
def test_generator_reproduces_golden_graph(engine, name):
    g = GEN[name]()
    e = COUNTS["graphs"][name]
    assert (g.v_cnt, g.e_cnt) == (e["v_cnt"], e["e_cnt"])
    assert csr_checksum(g) == e["checksum"]


@pytest.mark.parametrize("name", list(GEN))
def test_oracle_matches_reference_counts(engine, oracle, name):
    g = GEN[name]()
    e = COUNTS["graphs"][name]
    assert oracle.triangles(g) == e["tri_cnt"]
    perf, restr, iep = e["flags"]
    for pname, want in e["counts"].items():
        n = int(round(len(e["adj"][pname]) ** 0.5))
        p = gp.Pattern.from_adj(np.array(e["adj"][pname]).reshape(n, n))
        s = gp.Schedule(p, perf, restr, bool(iep), g.v_cnt, g.e_cnt, e["tri_cnt"])
        assert oracle.count(g, s) == want, pname


def test_oracle_matches_brute_force(engine, oracle):
    g = gp.chung_lu(250, 10.0, 2.2, 60, 11)
    tri = oracle.triangles(g)
    for k in (3, 4, 5):
        for p in gp.MotifGenerator(k).generate():
            for flags in [(1, 1, True), (0, 0, False), (1, 1, False)]:
                s = gp.Schedule(p, flags[0], flags[1], flags[2], g.v_cnt, g.e_cnt, tri)
                if not s.is_pattern_valid:
                    continue
                want = oracle.brute_force(g, p)
                got = oracle.count(g, s)
                if flags[1] == 0:  # no restrictions: every automorphic copy counted
                    got //= p.multiplicity()
                assert got == want, (p, flags)


def test_oracle_triangles_closed_forms(engine, oracle):
    k = gp.complete_graph(9)
    assert oracle.triangles(k) == 84
    assert oracle.count(k, gp.Schedule(gp.Pattern(4, True), 1, 1, True, 9, k.e_cnt, 84)) == 126


def test_oracle_root_shards_sum_to_total(engine, oracle):
    g = gp.chung_lu(600, 9.0, 2.2, 100, 3)
    tri = oracle.triangles(g)
    for p in [gp.Pattern(gp.PatternType.House), gp.Pattern(gp.PatternType.Rectangle)]:
        s = gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, tri)
        full = oracle.raw_roots(g, s, np.arange(g.v_cnt))
        shards = sum(oracle.raw_roots(g, s, np.arange(r, g.v_cnt, 3)) for r in range(3))
        assert full == shards
        assert full // s.get_in_exclusion_optimize_redundancy() == oracle.count(g, s)


@pytest.mark.skipif(not REF_LIB.exists(), reason="reference library not built here")
def test_oracle_matches_live_reference(engine, oracle):
    R = C.CDLL(str(REF_LIB))
    R.ref_graph_from_csr.restype = C.c_void_p
    R.ref_graph_from_csr.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_longlong, C.c_int]
    R.ref_graph_tri.restype = C.c_longlong
    R.ref_graph_tri.argtypes = [C.c_void_p]
    R.ref_graph_free.argtypes = [C.c_void_p]
    R.ref_schedule_create.restype = C.c_void_p
    R.ref_schedule_create.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint,
                                      C.c_longlong, C.POINTER(C.c_int)]
    R.ref_schedule_free.argtypes = [C.c_void_p]
    R.ref_pattern_matching.restype = C.c_longlong
    R.ref_pattern_matching.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    g = gp.rmat(11, 8, 0.57, 0.19, 0.19, 9)
    rg = R.ref_graph_from_csr(g.v_cnt, g.vertex.ctypes.data, g.edge.ctypes.data, -1, 4)
    tri = R.ref_graph_tri(rg)
    assert tri == oracle.triangles(g)
    for p in gp.motifs_3_to_5()[:12]:
        a = np.ascontiguousarray(p.adj, dtype=np.int32)
        ok = C.c_int()
        rs = R.ref_schedule_create(a.shape[0], a.ctypes.data, 1, 1, 1, g.v_cnt, g.e_cnt, tri, C.byref(ok))
        want = R.ref_pattern_matching(rg, rs, 4)
        R.ref_schedule_free(rs)
        s = gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, tri)
        assert oracle.count(g, s) == want
    R.ref_graph_free(rg)


@pytest.mark.skipif(WIKI is None or not WIKI.exists(),
                    reason="Wiki-Vote dataset: set GRAPHPI_REFERENCE to the reference checkout")
def test_oracle_wiki_vote(engine, oracle):
    g = gp.DataLoader().load_data(gp.DataType.Wiki_Vote, str(WIKI))
    w = COUNTS["wiki_vote"]
    assert (g.v_cnt, g.e_cnt) == (7115, 201524)
    assert oracle.triangles(g) == w["tri_cnt"]
    for name, p in [("rectangle", gp.Pattern(gp.PatternType.Rectangle)), ("clique4", gp.Pattern(4, True))]:
        s = gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, g.tri_cnt)
        assert oracle.count(g, s) == w[name]


def test_oracle_stripes_sum_to_whole_job(engine, oracle):
    """The engine's first-level task split: stripes of every size add up to
    the whole job's undivided sum, for edge-task and root-task plans."""
    g = gp.relabel_by_degree(gp.rmat(10, 12, 0.57, 0.19, 0.19, 4))
    tri = oracle.triangles(g)
    pats = gp.motifs_3_to_5()
    scheds = [gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, tri) for p in pats]
    for S in (1, 5, 64):
        sums = oracle.stripes_raw(g, [s.tables for s in scheds], S, list(range(S)))
        for s, row in zip(scheds, sums):
            assert sum(row) // s.get_in_exclusion_optimize_redundancy() == oracle.count(g, s)


@pytest.mark.skipif(not REF_LIB.exists(), reason="reference library not built here")
def test_oracle_stripes_match_live_reference(engine, oracle):
    """Per-stripe sums of the oracle equal the reference's own code run on
    the same task split (ref_stripes_raw), on all 29 motifs."""
    from tests import oracle_lib
    R = oracle_lib.load_ref()
    g = gp.relabel_by_degree(gp.rmat(11, 8, 0.57, 0.19, 0.19, 9))
    tri = oracle.triangles(g)
    rg = R.ref_graph_from_csr(g.v_cnt, g.vertex.ctypes.data, g.edge.ctypes.data, -1, 4)
    S, ids = 7, np.arange(7, dtype=np.int64)
    for p in gp.motifs_3_to_5():
        tabs, ok = oracle_lib.ref_schedule_tables(R, p.adj, 1, 1, True, g.v_cnt, g.e_cnt, tri)
        a = np.ascontiguousarray(p.adj, dtype=np.int32)
        okc = C.c_int()
        rs = R.ref_schedule_create(a.shape[0], a.ctypes.data, 1, 1, 1, g.v_cnt, g.e_cnt, tri, C.byref(okc))
        ref = np.zeros(S, dtype=np.int64)
        R.ref_stripes_raw(rg, rs, S, ids.ctypes.data, S, 4, ref.ctypes.data)
        R.ref_schedule_free(rs)
        assert oracle.stripes_raw(g, [tabs], S, ids)[0] == ref.tolist(), p
    R.ref_graph_free(rg)


def test_bench_golden_records_reference_tables():
    """The recorded benchmark fixture names its graphs and its stripe ids
    are the seeded ones the benchmark draws."""
    import json
    e = json.loads((Path(__file__).resolve().parent / "golden" / "bench_stripes.json").read_text())
    for name, scale in (("rmat_s22", 22), ("rmat_s20", 20)):
        x = e[name]
        assert x["scale"] == scale and x["flags"] == [1, 1, 1]
        assert x["ids"] == workloads.random_stripes(x["stripes"], len(x["ids"]))
        assert len(x["tables"]) == len(x["raw"]) == len(x["names"])
        assert all(len(r) == len(x["ids"]) for r in x["raw"])


def test_oracle_clique_path_counts_cliques(engine, oracle):
    """The reference's clique function (pattern_matching_func, clique = true)
    counts each k-clique once: it equals the general path and the brute
    force for complete patterns."""
    for g in (gp.chung_lu(300, 14.0, 2.2, 80, 3), gp.rmat(9, 12, 0.57, 0.19, 0.19, 2)):
        tri = oracle.triangles(g)
        for k in (3, 4, 5, 6):
            s = gp.Schedule(gp.Pattern(k, True), 1, 1, True, g.v_cnt, g.e_cnt, tri)
            assert s.is_complete()
            want = oracle.count(g, s)
            assert oracle.count_clique(g, s) == want, k
            if k <= 5:
                assert oracle.brute_force(g, gp.Pattern(k, True)) == want, k


def test_unfolded_cpu_code_matches_oracle(engine, oracle):
    """The unfolded CPU comparison path (oracle/unfolded.py: per-schedule
    nested loops, as the reference's code generator writes them) counts what
    the interpreted oracle counts, with and without inclusion-exclusion."""
    from oracle.unfolded import Unfolded
    g = gp.rmat(10, 12, 0.57, 0.19, 0.19, 6)
    tri = oracle.triangles(g)
    for iep in (True, False):
        scheds = [gp.Schedule(p, 1, 1, iep, g.v_cnt, g.e_cnt, tri) for p in gp.motifs_3_to_5()]
        scheds += [gp.Schedule(p, 1, 1, iep, g.v_cnt, g.e_cnt, tri) for p in gp.MotifGenerator(6).generate()[::23]]
        u = Unfolded(scheds)
        for i, s in enumerate(scheds):
            assert u.count(g, i) == oracle.count(g, s), (i, iep)
