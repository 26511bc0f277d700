"""GPU parity at the benchmark sizes.

The whole job of a 5-vertex motif on R-MAT scale 22 is hours of CPU time, so
parity there is pinned on bounded, uniformly random parts of the job:
stripes of the engine's first-level tasks (tasks t with t mod S == s; the
undivided 128-bit sums of the stripes add up to the whole job).
  * tests/golden/bench_stripes.json holds the reference's own schedule
    tables and its undivided sums over 48 seeded random stripes of R-MAT
    scale 22 (all 29 motifs) and 16 of R-MAT scale 20 (rectangle, house),
    recorded by tests/golden/make_bench_golden.py from the reference library;
  * further stripes are checked against the CPU oracle live;
  * whole-graph star counts are checked against the closed form
    sum_v C(deg v, k) in Python integers (above 2^64 at scale 22).
Counts must match bit for bit.
"""
import ctypes as C
import json
import math
from pathlib import Path

import numpy as np
import pytest

import graphpi_gb300 as gp
from graphpi_gb300 import native, workloads
from tests.oracle_lib import csr_checksum

pytestmark = pytest.mark.gpu

GOLDEN = json.loads((Path(__file__).resolve().parent / "golden" / "bench_stripes.json").read_text())


def _signed(v: int) -> int:
    return v - (1 << 128) if v >= (1 << 127) else v


def _raw_stripes(g, scheds, S, ids, batched=True):
    """Engine raw sums [pattern][stripe] over stripes ids of S."""
    plans = [gp.Plan(s) for s in scheds]
    n = len(plans)
    gh = (C.c_void_p * n)(*([g.device()] * n))
    ph = (C.c_void_p * n)(*[p.handle for p in plans])
    out = [[0] * len(ids) for _ in plans]
    gp.set_option("raw_sums", 1)
    gp.set_option("stripes", S)
    try:
        for j, s in enumerate(ids):
            gp.set_option("stripe", s)
            if batched:
                outs = (native.U128 * n)()
                native.check(gp.lib().gpm_batch_count(n, gh, ph, outs), "gpm_batch_count")
                for i in range(n):
                    out[i][j] = _signed(outs[i].value)
            else:
                for i, p in enumerate(plans):
                    o = native.U128()
                    native.check(gp.lib().gpm_count(g.device(), p.handle, C.byref(o)), "gpm_count")
                    out[i][j] = _signed(o.value)
    finally:
        gp.set_option("stripes", 1)
        gp.set_option("stripe", 0)
        gp.set_option("raw_sums", 0)
        for p in plans:
            p.close()
    return out


@pytest.fixture(scope="module")
def s22():
    e = GOLDEN["rmat_s22"]
    g = workloads.rmat_scale(22, 3)
    assert csr_checksum(g) == e["checksum"]
    tri = g.triangle_counting_mt()
    assert tri == e["tri_cnt"]
    scheds = [gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, tri) for p in gp.motifs_3_to_5()]
    yield g, scheds, e
    g.close()


def test_s22_schedules_equal_reference(engine, s22):
    g, scheds, e = s22
    for s, want, name in zip(scheds, e["tables"], e["names"]):
        assert [int(x) for x in s.tables] == want, name


def test_s22_random_stripes_match_reference_sums(engine, s22):
    """All 29 motifs, batched, on the 48 recorded stripes of 2^23."""
    g, scheds, e = s22
    got = _raw_stripes(g, scheds, e["stripes"], e["ids"])
    for i, name in enumerate(e["names"]):
        assert got[i] == e["raw"][i], name


def test_s22_stripes_one_pattern_per_launch(engine, s22):
    """Plain launches agree with the recorded sums too (first 4 stripes)."""
    g, scheds, e = s22
    got = _raw_stripes(g, scheds, e["stripes"], e["ids"][:4], batched=False)
    for i, name in enumerate(e["names"]):
        assert got[i] == e["raw"][i][:4], name


def test_s22_stripes_match_live_oracle(engine, oracle, s22):
    """Two more random stripes, outside the recorded set, against the CPU
    oracle run now; the device's degree relabel must number the tasks as the
    host relabel does (a host-relabelled upload without relabelling gives the
    same sums)."""
    g, scheds, e = s22
    S = e["stripes"]
    ids = [s for s in workloads.random_stripes(S, 64) if s not in set(e["ids"])][:2]
    got = _raw_stripes(g, scheds, S, ids)
    gr = gp.relabel_by_degree(g)
    want = oracle.stripes_raw(gr, [s.tables for s in scheds], S, ids)
    assert got == want
    h = gp.Graph(gr.v_cnt, gr.vertex, gr.edge)
    h.device(relabel=False)
    assert _raw_stripes(h, scheds, S, ids) == want
    h.close()


def _star(k: int):
    p = gp.Pattern(k + 1)
    for i in range(1, k + 1):
        p.add_edge(0, i)
    return p


@pytest.mark.parametrize("scale,seed", [(20, 2), (22, 3)])
def test_star_counts_closed_form(engine, scale, seed):
    """Whole-graph counts of the stars with 2, 3 and 4 leaves equal
    sum_v C(deg v, k) exactly; at scale 22 the 4-leaf count exceeds 2^64."""
    g = workloads.rmat_scale(scale, seed)
    deg = np.diff(g.vertex.astype(np.int64)).tolist()
    tri = g.triangle_counting_mt()
    for k in (2, 3, 4):
        s = gp.Schedule(_star(k), 1, 1, True, g.v_cnt, g.e_cnt, tri)
        want = sum(math.comb(d, k) for d in deg)
        assert g.pattern_matching(s) == want, k
    if scale == 22:
        assert sum(math.comb(d, 4) for d in deg) > 1 << 64
    g.close()


def test_s20_rectangle_house_match_reference_sums(engine):
    e = GOLDEN["rmat_s20"]
    g = workloads.rmat_scale(20, 2)
    assert csr_checksum(g) == e["checksum"]
    tri = g.triangle_counting_mt()
    assert tri == e["tri_cnt"]
    pats = [gp.Pattern(gp.PatternType.Rectangle), gp.Pattern(gp.PatternType.House)]
    scheds = [gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, tri) for p in pats]
    for s, want in zip(scheds, e["tables"]):
        assert [int(x) for x in s.tables] == want
    got = _raw_stripes(g, scheds, e["stripes"], e["ids"], batched=False)
    assert got == e["raw"]
    g.close()
