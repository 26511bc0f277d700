"""Schedule compiler parity: the engine's tables equal the reference
Schedule's (golden tables from the reference built from source, see
tests/golden/make_golden.py)."""
import numpy as np
import pytest

import graphpi_gb300 as gp
from tests.oracle_lib import golden

SCHED = golden("schedules.json")


def test_motif_generator_matches_reference(engine):
    # counts 2 / 6 / 21 / 112 and the same generation order
    # (reference test/schedule_test.cpp:57,64 asserts 2 and 6)
    for k, mats in SCHED["motifs"].items():
        ours = [p.adj.reshape(-1).tolist() for p in gp.MotifGenerator(int(k)).generate()]
        assert ours == mats
    assert [len(SCHED["motifs"][str(k)]) for k in (3, 4, 5, 6)] == [2, 6, 21, 112]


@pytest.mark.parametrize("chunk", range(8))
def test_schedule_tables_equal_reference(engine, chunk):
    entries = SCHED["schedules"][chunk::8]
    for e in entries:
        n = e["n"]
        p = gp.Pattern.from_adj(np.array(e["adj"]).reshape(n, n))
        perf, restr, iep = e["flags"]
        v, ecnt, tri = e["stats"]
        s = gp.Schedule(p, perf, restr, bool(iep), v, ecnt, tri)
        assert s.is_pattern_valid == e["valid"], (n, e["flags"])
        if e["valid"]:
            assert s.tables.tolist() == e["tables"], (n, e["adj"], e["flags"])


def test_prefix_tree_shape(engine):
    # reference test/schedule_test.cpp:27-49: 5-vertex pattern with
    # prefixes N(0), N(1), N(0)N(1), N(0)N(1)N(2)
    p = gp.Pattern(5)
    p.add_edge(0, 1)
    p.add_edge(1, 2)
    for i in (3, 4):
        for j in range(3):
            p.add_edge(i, j)
    s = gp.Schedule(p, 0, 0, False, 10, 20, 0)
    assert s.get_total_prefix_num() == 4
    assert [s.get_loop_set_prefix_id(i) for i in range(1, 5)] == [0, 1, 3, 3]
    assert s.get_father_prefix_id(3) == 2 and s.get_father_prefix_id(2) == 0


def test_iep_tables_and_redundancy(engine):
    # 5-star: four independent leaves -> IEP over 4 loops, 15 set partitions
    star = gp.Pattern(5)
    for i in range(1, 5):
        star.add_edge(0, i)
    s = gp.Schedule(star, 1, 1, True, 1000, 10000, 100)
    assert s.get_in_exclusion_optimize_num() == 4
    assert len(s.in_exclusion_optimize_group) == 15
    # all-singleton group first with coefficient 1
    assert s.in_exclusion_optimize_group[0] == [[0], [1], [2], [3]]
    assert s.in_exclusion_optimize_val[0] == 1
    assert s.get_in_exclusion_optimize_redundancy() >= 1


def test_multiplicity(engine):
    assert gp.Pattern(4, True).multiplicity() == 24
    assert gp.Pattern(gp.PatternType.Rectangle).multiplicity() == 8
    assert gp.Pattern(gp.PatternType.House).multiplicity() == 2


def test_perf_modeling_requires_triangles(engine):
    with pytest.raises(gp.GpmError):
        gp.Schedule(gp.Pattern(3, True), 1, 1, False, 100, 1000, -1)


def test_invalid_order_reported(engine):
    # path 0-2-1 in identity order: vertex 1 has no earlier neighbour
    p = gp.Pattern(3)
    p.add_edge(0, 2)
    p.add_edge(1, 2)
    s = gp.Schedule(p, 0, 0, False, 10, 10, 0)
    assert not s.is_pattern_valid


def test_builtin_patterns(engine):
    for t in gp.PatternType:
        p = gp.Pattern(t)
        assert p.check_connected()
        s = gp.Schedule(p, 0, 1, True, 1000, 10000, 0)
        assert s.is_pattern_valid


def test_label_sensitive_schedules_flagged(engine):
    # schedules whose reference count depends on labels (checked against the
    # brute-force count: these differ from it) must be flagged
    wrong = ["011100100011100011100011011100011100", "011100101010110001100011010101001110",
             "011110101110110101111001110001001110", "011111101100110010110001101001100110"]
    for adj in wrong:
        s = gp.Schedule(gp.Pattern(6, adj), 1, 1, True, 400, 3000, 2000)
        assert s.label_sensitive(), adj
    # without inclusion-exclusion nothing is skipped
    for p in gp.motifs_3_to_5():
        assert not gp.Schedule(p, 1, 1, False, 400, 3000, 2000).label_sensitive()


def test_candidates_reproduce_the_constructors_choice(engine):
    # the first candidate of minimal analytic cost, rebuilt from its order,
    # gives exactly the tables of the Schedule constructor
    stats = (7115, 201524, 608389)
    for p in gp.motifs_3_to_5()[::2] + [gp.Pattern(gp.PatternType.House)]:
        cands = gp.schedule_candidates(p, 1, 1, *stats)
        assert cands
        best = min(range(len(cands)), key=lambda i: (cands[i]["cost"], i))
        s = gp.schedule_from_order(p, cands[best]["order"], cands[best]["pairs"], True, 1)
        ref = gp.Schedule(p, 1, 1, True, *stats)
        assert s.tables.tolist() == ref.tables.tolist(), p
