"""The clique fast path (gpm_clique_count; Graph::pattern_matching with
clique=True on a complete pattern) against the oracle's restatement of the
reference's clique function and its general path, bit for bit."""
import ctypes as C
import math

import pytest

import graphpi_gb300 as gp
from graphpi_gb300 import native

pytestmark = pytest.mark.gpu


def _clique(g, k: int) -> int:
    out = native.U128()
    native.check(gp.lib().gpm_clique_count(g.device(), k, C.byref(out)), "gpm_clique_count")
    return out.value


@pytest.mark.parametrize("make", [
    lambda: gp.chung_lu(3000, 16.0, 2.1, 400, 41),
    lambda: gp.rmat(13, 16, 0.57, 0.19, 0.19, 7),
])
def test_clique_counts_match_oracle(engine, oracle, make):
    g = make()
    tri = oracle.triangles(g)
    for k in (3, 4, 5, 6):
        s = gp.Schedule(gp.Pattern(k, True), 1, 1, True, g.v_cnt, g.e_cnt, tri)
        want = oracle.count_clique(g, s)
        assert want == oracle.count(g, s)
        assert _clique(g, k) == want, k
        assert g.pattern_matching(s, 0, True) == want
    assert _clique(g, 3) == g.triangle_counting_mt()


def test_clique_complete_graph_and_stripes(engine):
    k16 = gp.complete_graph(16)
    for k in range(3, 9):
        assert _clique(k16, k) == math.comb(16, k)
    g = gp.rmat(12, 16, 0.57, 0.19, 0.19, 3)
    whole = _clique(g, 5)
    gp.set_option("stripes", 7)
    try:
        parts = 0
        for s in range(7):
            gp.set_option("stripe", s)
            parts += _clique(g, 5)
    finally:
        gp.set_option("stripes", 1)
        gp.set_option("stripe", 0)
    assert parts == whole


def test_clique_flag_ignored_for_other_patterns(engine, oracle):
    """clique=True on a pattern that is not complete counts it normally (the
    reference's pattern_matching takes its general path for any flag)."""
    g = gp.chung_lu(1500, 10.0, 2.2, 150, 43)
    tri = oracle.triangles(g)
    s = gp.Schedule(gp.Pattern(gp.PatternType.House), 1, 1, True, g.v_cnt, g.e_cnt, tri)
    assert g.pattern_matching(s, 0, True) == oracle.count(g, s)
