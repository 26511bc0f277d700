"""GPU parity: the sm_103a enumerator against the reference's recorded counts
(golden fixtures) and the CPU oracle on the same seeded graphs.  Integer
counts must match bit for bit."""
import ctypes as C
import math

import numpy as np
import pytest

import graphpi_gb300 as gp
from graphpi_gb300 import workloads
from tests.oracle_lib import csr_checksum, golden

pytestmark = pytest.mark.gpu

COUNTS = golden("counts.json")
GEN = {
    "chung_lu_7k": workloads.chung_lu_7k,
    "rmat_s10": lambda: gp.rmat(10, 16, 0.57, 0.19, 0.19, 2),
    "chung_lu_2k": lambda: gp.chung_lu(2000, 12.0, 2.3, 300, 7),
    "rmat_s12_noiep": lambda: gp.rmat(12, 8, 0.57, 0.19, 0.19, 5),
}


def _pattern(adj):
    n = int(round(len(adj) ** 0.5))
    return gp.Pattern.from_adj(np.array(adj).reshape(n, n))


@pytest.mark.parametrize("name", list(GEN))
def test_triangles_match_reference(engine, oracle, name):
    g = GEN[name]()
    assert g.triangle_counting_mt(0) == COUNTS["graphs"][name]["tri_cnt"] == oracle.triangles(g)


@pytest.mark.parametrize("name", list(GEN))
def test_counts_match_reference_golden(engine, name):
    g = GEN[name]()
    e = COUNTS["graphs"][name]
    assert csr_checksum(g) == e["checksum"]
    perf, restr, iep = e["flags"]
    for pname, want in e["counts"].items():
        s = gp.Schedule(_pattern(e["adj"][pname]), perf, restr, bool(iep), g.v_cnt, g.e_cnt, e["tri_cnt"])
        assert g.pattern_matching(s, 0) == want, pname


@pytest.mark.parametrize("seed", [21, 22])
@pytest.mark.parametrize("flags", [(1, 1, True), (1, 1, False), (0, 0, False), (0, 1, True), (3, 1, True)])
def test_all_motifs_match_oracle(engine, oracle, seed, flags):
    g = gp.chung_lu(1500, 10.0, 2.2, 200, seed) if seed % 2 else gp.rmat(10, 12, 0.57, 0.19, 0.19, seed)
    tri = oracle.triangles(g)
    for p in gp.motifs_3_to_5():
        s = gp.Schedule(p, flags[0], flags[1], flags[2], g.v_cnt, g.e_cnt, tri)
        if not s.is_pattern_valid:
            continue
        assert g.pattern_matching(s) == oracle.count(g, s), (p, flags)


def test_six_vertex_patterns_match_oracle(engine, oracle):
    g = gp.chung_lu(400, 8.0, 2.3, 60, 5)
    tri = oracle.triangles(g)
    pats = gp.MotifGenerator(6).generate()
    for p in pats[::7] + [gp.Pattern(gp.PatternType.Hourglass), gp.Pattern(gp.PatternType.Cycle_6_Tri)]:
        s = gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, tri)
        assert g.pattern_matching(s) == oracle.count(g, s), p


def test_batch_matches_single_launches(engine, oracle):
    g = gp.rmat(11, 10, 0.57, 0.19, 0.19, 8)
    h = gp.chung_lu(3000, 9.0, 2.4, 300, 9)
    tri_g, tri_h = g.triangle_counting_mt(), h.triangle_counting_mt()
    pats = gp.motifs_3_to_5()
    graphs, scheds = [], []
    for i, p in enumerate(pats):
        x, t = (g, tri_g) if i % 2 == 0 else (h, tri_h)
        graphs.append(x)
        scheds.append(gp.Schedule(p, 1, 1, True, x.v_cnt, x.e_cnt, t))
    batched = gp.batch_count(graphs, scheds)
    for x, s, b in zip(graphs, scheds, batched):
        assert b == x.pattern_matching(s) == oracle.count(x, s)


def test_host_buffer_path(engine, oracle):
    g = gp.chung_lu(2500, 11.0, 2.2, 250, 13)
    tri = oracle.triangles(g)
    scheds = [gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, tri) for p in gp.motifs_3_to_5()]
    got = gp.count_host(g, scheds)
    assert got == [oracle.count(g, s) for s in scheds]


def test_relabel_does_not_change_counts(engine):
    g = gp.rmat(10, 8, 0.57, 0.19, 0.19, 31)
    h = gp.Graph(g.v_cnt, g.vertex, g.edge)
    h.device(relabel=False)
    tri = g.triangle_counting_mt()
    assert h.triangle_counting_mt() == tri
    for p in gp.motifs_3_to_5()[::3]:
        s = gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, tri)
        assert g.pattern_matching(s) == h.pattern_matching(s)


def test_complete_graph_closed_forms(engine):
    for n in (5, 9, 16):
        k = gp.complete_graph(n)
        assert k.triangle_counting_mt() == math.comb(n, 3)
        for size in (3, 4, 5):
            s = gp.Schedule(gp.Pattern(size, True), 1, 1, True, n, k.e_cnt, math.comb(n, 3))
            assert k.pattern_matching(s) == math.comb(n, size)


def test_counts_beyond_64_bits(engine):
    # one hub with 150,000 leaves: C(150000, 4) 5-stars > 2^64, which the
    # reference's signed 64-bit accumulation cannot hold
    d = 150000
    g = gp.from_edges(d + 1, np.zeros(d, dtype=np.int32), np.arange(1, d + 1, dtype=np.int32))
    star5 = gp.Pattern(5)
    for i in range(1, 5):
        star5.add_edge(0, i)
    s = gp.Schedule(star5, 1, 1, True, g.v_cnt, g.e_cnt, 0)
    want = math.comb(d, 4)
    assert want > 2 ** 64
    assert g.pattern_matching(s) == want
    star4 = gp.Pattern(4)
    for i in range(1, 4):
        star4.add_edge(0, i)
    s4 = gp.Schedule(star4, 1, 1, True, g.v_cnt, g.e_cnt, 0)
    assert g.pattern_matching(s4) == math.comb(d, 3)


def test_sparse_and_ragged_inputs(engine, oracle):
    # isolated vertices, an edgeless graph, a single edge, a path
    empty = gp.Graph(5, np.zeros(6, dtype=np.uint32), np.zeros(0, dtype=np.int32))
    tri_s = gp.Schedule(gp.Pattern(3, True), 0, 1, False, 5, 0, 0)
    assert empty.triangle_counting_mt() == 0
    assert empty.pattern_matching(tri_s) == 0
    one = gp.from_edges(4, [1], [3])
    wedge = gp.Pattern(3)
    wedge.add_edge(0, 1)
    wedge.add_edge(0, 2)
    assert one.pattern_matching(gp.Schedule(wedge, 1, 1, True, 4, one.e_cnt, 0)) == 0
    path = gp.from_edges(6, [0, 1, 2, 3], [1, 2, 3, 4])
    s = gp.Schedule(wedge, 1, 1, True, 6, path.e_cnt, 0)
    assert path.pattern_matching(s) == 3 == oracle.count(path, s)


def test_malformed_csr_rejected(engine):
    cases = {
        "unsorted": ([0, 2, 3, 4], [2, 1, 0, 0]),
        "self loop": ([0, 1, 2], [0, 0]),
        "asymmetric": ([0, 1, 1], [1]),
        "out of range": ([0, 1, 2], [5, 0]),
    }
    for name, (rp, col) in cases.items():
        g = gp.Graph(len(rp) - 1, np.array(rp, dtype=np.uint32), np.array(col, dtype=np.int32))
        with pytest.raises(gp.GpmError) as ei:
            g.device()
        assert ei.value.code == 1, name


def test_algorithmic_byte_counter(engine):
    g = gp.rmat(10, 16, 0.57, 0.19, 0.19, 2)
    s = gp.Schedule(gp.Pattern(gp.PatternType.House), 1, 1, True, g.v_cnt, g.e_cnt, g.triangle_counting_mt())
    gp.set_option("count_bytes", 1)
    try:
        a = g.pattern_matching(s)
        _, launches, nbytes = gp.last_launch_stats()
    finally:
        gp.set_option("count_bytes", 0)
    assert a == g.pattern_matching(s)
    assert launches == 1 and nbytes > 0


def test_engine_knobs_do_not_change_counts(engine, oracle):
    g = gp.chung_lu(2000, 12.0, 2.3, 300, 7)
    e = COUNTS["graphs"]["chung_lu_2k"]
    scheds = {k: gp.Schedule(_pattern(e["adj"][k]), 1, 1, True, g.v_cnt, g.e_cnt, e["tri_cnt"])
              for k in ("m4_2", "m5_3", "m5_20")}
    for knobs in [{"chunk": 1}, {"warps_per_block": 4, "blocks_per_sm": 1}, {"chunk": 64, "warps_per_block": 16},
                  {"min_blocks": 3, "warps_per_block": 8}]:
        old = {k: gp.get_option(k) for k in knobs}
        for k, v in knobs.items():
            gp.set_option(k, v)
        try:
            for name, s in scheds.items():
                assert g.pattern_matching(s) == e["counts"][name], (knobs, name)
        finally:
            for k, v in old.items():
                gp.set_option(k, v)


def test_cuda_graph_replay_matches_batch(engine, oracle):
    g = gp.rmat(11, 10, 0.57, 0.19, 0.19, 8)
    tri = g.triangle_counting_mt()
    scheds = [gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, tri) for p in gp.motifs_3_to_5()]
    want = gp.batch_count([g] * len(scheds), scheds)
    ex = gp.BatchExec([g] * len(scheds), scheds)
    try:
        assert ex.run() == want
        assert ex.run() == want  # replay
        # replays over stripes sum to the whole job
        gp.set_option("raw_sums", 1)
        gp.set_option("stripes", 4)
        tot = [0] * len(scheds)
        for st in range(4):
            gp.set_option("stripe", st)
            for i, r in enumerate(ex.run()):
                tot[i] += r - (1 << 128) if r >= (1 << 127) else r
        red = [s.get_in_exclusion_optimize_redundancy() for s in scheds]
        assert [t // d for t, d in zip(tot, red)] == want
    finally:
        gp.set_option("stripes", 1)
        gp.set_option("stripe", 0)
        gp.set_option("raw_sums", 0)
        ex.close()


def test_leaf_batch_matches_per_candidate_path(engine, oracle):
    g = gp.chung_lu(3000, 14.0, 2.2, 400, 41)
    tri = g.triangle_counting_mt()
    for flags in [(1, 1, True), (1, 1, False), (0, 1, True)]:
        scheds = [gp.Schedule(p, flags[0], flags[1], flags[2], g.v_cnt, g.e_cnt, tri) for p in gp.motifs_3_to_5()]
        scheds = [s for s in scheds if s.is_pattern_valid]
        pairs = [g] * len(scheds)
        batched = _with_options({"leaf_batch": 1}, lambda: gp.batch_count(pairs, scheds))
        plain = _with_options({"leaf_batch": 0}, lambda: gp.batch_count(pairs, scheds))
        assert batched == plain == [oracle.count(g, s) for s in scheds]
    # tiny staging area forces the global-memory probe path
    assert _with_options({"leaf_batch": 1, "stage_max": 16}, lambda: gp.batch_count(pairs, scheds)) == batched


def test_uneven_multi_graph_batch(engine, oracle):
    # the 256-pair uneven batch, shrunk: 24 seeded Chung-Lu graphs with
    # parameters from the same generator (sizes scaled to 300-3000 vertices),
    # one motif each, all pairs in one persistent launch; per-pair exact
    from graphpi_gb300 import workloads
    motifs = gp.motifs_3_to_5()
    params = workloads.uneven_params(count=24, n_lo=300, n_hi=3000)
    graphs, scheds = [], []
    for n, avg, gamma, seed, m in params:
        g = workloads.uneven_graph(n, min(avg, 24.0), gamma, seed)
        graphs.append(g)
        scheds.append(gp.Schedule(motifs[m], 1, 1, True, g.v_cnt, g.e_cnt, oracle.triangles(g)))
    got = gp.batch_count(graphs, scheds)
    assert got == [oracle.count(g, s) for g, s in zip(graphs, scheds)]


def _with_options(opts: dict, fn):
    old = {k: gp.get_option(k) for k in opts}
    for k, v in opts.items():
        gp.set_option(k, v)
    try:
        return fn()
    finally:
        for k, v in old.items():
            gp.set_option(k, v)


def test_loop_donation_matches_oracle(engine, oracle):
    # skewed graph: hub loops are published and sliced by idle warps; with
    # split=1 every loop at depth >= 2 is shared, the most racy setting
    g = gp.rmat(11, 16, 0.57, 0.19, 0.19, 31)
    tri = g.triangle_counting_mt()
    scheds = [gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, tri) for p in gp.motifs_3_to_5()]
    scheds += [gp.Schedule(p, 1, 1, False, g.v_cnt, g.e_cnt, tri) for p in gp.motifs_3_to_5()[8::4]]
    want = [oracle.count(g, s) for s in scheds]
    pairs = [g] * len(scheds)
    assert _with_options({"split": 0}, lambda: gp.batch_count(pairs, scheds)) == want
    for split in (1, 3, 64):
        for leaf in (0, 1):
            got = _with_options({"split": split, "leaf_batch": leaf}, lambda: gp.batch_count(pairs, scheds))
            assert got == want, (split, leaf)
    # few warps, many slices each
    got = _with_options({"split": 2, "warps_per_block": 4, "blocks_per_sm": 1}, lambda: gp.batch_count(pairs, scheds))
    assert got == want


def test_loop_donation_six_vertex(engine, oracle):
    g = gp.chung_lu(600, 10.0, 2.1, 150, 9)
    tri = oracle.triangles(g)
    pats = gp.MotifGenerator(6).generate()[::9]
    scheds = [gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, tri) for p in pats]
    want = [oracle.count(g, s) for s in scheds]
    got = _with_options({"split": 1}, lambda: gp.batch_count([g] * len(scheds), scheds))
    assert got == want


def test_pair_sum_leaf_matches_oracle(engine, oracle):
    # the pair-sum leaf (sum_x a_x b_x - c_x) against the per-candidate path:
    # a sparse graph whose tables fit, and a dense one whose hub tasks fall
    # back to the loops
    for g in (gp.chung_lu(3000, 8.0, 2.5, 100, 12), gp.rmat(10, 24, 0.57, 0.19, 0.19, 13)):
        tri = oracle.triangles(g)
        scheds = [gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, tri) for p in gp.motifs_3_to_5()]
        scheds = [s for s in scheds if s.plan_info()["pair_ok"]]
        assert scheds, "no plan takes the pair-sum leaf"
        want = [oracle.count(g, s) for s in scheds]
        for split in (0, 1):
            # tables sized to memory; tiny ones that send tasks to the dense
            # counter arrays; tiny ones without arrays (the loops)
            for log2, dense, cap in ((0, 64, 0), (6, 64, 0), (6, 0, 0), (0, 0, 64)):
                opts = {"pair_leaf": 1, "split": split, "pair_log2": log2, "dense_slots": dense, "pair_max_ops": cap}
                got = _with_options(opts, lambda: gp.batch_count([g] * len(scheds), scheds))
                assert got == want, (split, log2, dense, cap)
        assert _with_options({"pair_leaf": 0}, lambda: gp.batch_count([g] * len(scheds), scheds)) == want


def test_stripes_do_not_depend_on_chunk(engine):
    g = gp.rmat(11, 10, 0.57, 0.19, 0.19, 8)
    tri = g.triangle_counting_mt()
    scheds = [gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, tri) for p in gp.motifs_3_to_5()[::3]]
    pairs = [g] * len(scheds)
    runs = []
    for chunk in (1, 8, 64):
        opts = {"raw_sums": 1, "stripes": 8, "stripe": 5, "chunk": chunk}
        runs.append(_with_options(opts, lambda: gp.batch_count(pairs, scheds)))
    assert runs[0] == runs[1] == runs[2]


def test_leaf_bitmaps_match_oracle(engine, oracle):
    # membership in large fixed leaf sets through per-warp bitmaps: forced on
    # for every set that does not fit a tiny stage, and off
    g = gp.rmat(11, 16, 0.57, 0.19, 0.19, 33)
    tri = g.triangle_counting_mt()
    scheds = [gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, tri) for p in gp.motifs_3_to_5()]
    scheds += [gp.Schedule(p, 1, 1, False, g.v_cnt, g.e_cnt, tri) for p in gp.motifs_3_to_5()[9::5]]
    want = [oracle.count(g, s) for s in scheds]
    pairs = [g] * len(scheds)
    for opts in ({"leaf_batch": 1, "bitmap_min": 1, "stage_max": 16},
                 {"leaf_batch": 1, "bitmap_min": 1, "stage_max": 16, "split": 1},
                 {"leaf_batch": 1, "bitmap_min": 0}):
        assert _with_options(opts, lambda: gp.batch_count(pairs, scheds)) == want, opts


def test_gpu_csr_builder_matches_host(engine, oracle):
    # edge list -> CSR on the GPU against the host builder: same offsets and
    # neighbours (caller's ids), same counts; bad ids rejected
    rng = np.random.default_rng(5)
    for v, m in ((1, 0), (50, 400), (3000, 40000)):
        src = rng.integers(0, v, m).astype(np.int32)
        dst = rng.integers(0, v, m).astype(np.int32)
        if m:
            src[:5], dst[:5] = 0, 0  # self loops
            src[5:9], dst[5:9] = src[9:13], dst[9:13]  # duplicates
        h = gp.from_edges(v, src, dst)
        d = gp.from_edges(v, src, dst, on_device=True)
        assert np.array_equal(h.vertex, d.vertex) and np.array_equal(h.edge, d.edge)
        if m:
            s = gp.Schedule(gp.Pattern(gp.PatternType.House), 1, 1, True, d.v_cnt, d.e_cnt, oracle.triangles(d))
            assert d.pattern_matching(s) == h.pattern_matching(s) == oracle.count(h, s)
    with pytest.raises(gp.GpmError):
        gp.from_edges(10, np.array([1, 2], np.int32), np.array([3, 10], np.int32), on_device=True)
