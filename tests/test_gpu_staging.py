"""Staging fixed leaf sets into shared memory with bulk copies
(cp.async.bulk into the warp's stage, completion on an mbarrier; option
"stage_tma") against plain loads and the oracle, on the batched leaf that
stages them, with sets at every 16-byte alignment."""
import pytest

import graphpi_gb300 as gp

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("stage_max", [1024, 37])
def test_bulk_copy_staging_matches_oracle(engine, oracle, stage_max):
    g = gp.rmat(11, 14, 0.57, 0.19, 0.19, 23)
    tri = oracle.triangles(g)
    scheds = [gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, tri) for p in gp.motifs_3_to_5()]
    want = [oracle.count(g, s) for s in scheds]
    old = {k: gp.get_option(k) for k in ("leaf_batch", "stage_tma", "stage_max")}
    try:
        gp.set_option("leaf_batch", 1)
        gp.set_option("stage_max", stage_max)
        for tma in (0, 1):
            gp.set_option("stage_tma", tma)
            assert gp.batch_count([g] * len(scheds), scheds) == want, tma
    finally:
        for k, v in old.items():
            gp.set_option(k, v)
