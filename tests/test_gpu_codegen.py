"""Per-schedule generated kernels (graphpi_gb300/codegen.py) against the
oracle and the reference's recorded stripe sums, bit for bit: every one of
the 29 connected 3-5-vertex motifs, with and without inclusion-exclusion,
with the long depth-2 loops run as queued slices, and stripes that add up."""
import json
from pathlib import Path

import pytest

import graphpi_gb300 as gp
from graphpi_gb300 import codegen, workloads
from tests.oracle_lib import csr_checksum

pytestmark = pytest.mark.gpu

GOLDEN = json.loads((Path(__file__).resolve().parent / "golden" / "bench_stripes.json").read_text())


@pytest.mark.parametrize("iep", [True, False])
def test_generated_motifs_match_oracle(engine, oracle, iep):
    g = gp.rmat(11, 12, 0.57, 0.19, 0.19, 17)
    tri = oracle.triangles(g)
    scheds = [gp.Schedule(p, 1, 1, iep, g.v_cnt, g.e_cnt, tri) for p in gp.motifs_3_to_5()]
    gen = codegen.Generated(scheds)
    for i, s in enumerate(scheds):
        want = oracle.count(g, s)
        assert gen.count(g, i) == want, i
        # every task with a depth-2 loop longer than 2 candidates as slices
        assert gen.raw(g, i, split2=2) // s.get_in_exclusion_optimize_redundancy() == want, i


def test_generated_six_vertex_and_stripes(engine, oracle):
    g = gp.chung_lu(1200, 9.0, 2.2, 150, 19)
    tri = oracle.triangles(g)
    pats = gp.MotifGenerator(6).generate()[::9]
    scheds = [gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, tri) for p in pats]
    gen = codegen.Generated(scheds)
    for i, s in enumerate(scheds):
        assert gen.count(g, i) == oracle.count(g, s), i
        parts = sum(gen.raw(g, i, stripes=5, stripe=k, split2=4) for k in range(5))
        assert parts == gen.raw(g, i)


def test_generated_s22_stripes_match_reference_sums(engine):
    """All 29 generated kernels on four of the reference-recorded stripes of
    R-MAT scale 22 (the same first-level tasks the interpreter counts)."""
    e = GOLDEN["rmat_s22"]
    g = workloads.rmat_scale(22, 3)
    assert csr_checksum(g) == e["checksum"]
    scheds = [gp.Schedule.from_tables(t) for t in e["tables"]]
    gen = codegen.Generated(scheds)
    for j in range(4):
        for i, name in enumerate(e["names"]):
            assert gen.raw(g, i, stripes=e["stripes"], stripe=e["ids"][j]) == e["raw"][i][j], (name, e["ids"][j])
    g.close()
