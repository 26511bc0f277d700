"""The autotuner changes speed only: counts stay identical under the tuned
knobs, and the table round-trips through its JSON store."""
import pytest

import graphpi_gb300 as gp
from graphpi_gb300 import autotune


def test_table_store_roundtrip(engine, tmp_path):
    p = tmp_path / "tune.json"
    autotune.save({"chunk": 4, "warps_per_block": 8}, p, "abc")
    autotune.save({"chunk": 16}, p, "def")
    assert autotune.load(p, "abc") == {"chunk": 4, "warps_per_block": 8}
    assert autotune.load(p, "def") == {"chunk": 16}
    assert autotune.load(p, "zzz") is None


@pytest.mark.gpu
def test_autotune_keeps_counts(engine, oracle):
    g = gp.rmat(12, 12, 0.57, 0.19, 0.19, 14)
    tri = g.triangle_counting_mt()
    scheds = [gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, tri) for p in gp.motifs_3_to_5()[::4]]
    before = autotune.current()
    try:
        space = {"chunk": [2, 16], "warps_per_block": [4, 8], "merge_alpha4_mid": [0, 8], "stage_max": [256, 1024]}
        table = autotune.autotune(g, scheds, stripes=16, sample_stripes=2, repeats=1, budget_s=60, space=space)
        assert table["_ms"] <= table["_default_ms"] * 1.05
        assert gp.batch_count([g] * len(scheds), scheds) == [oracle.count(g, s) for s in scheds]
    finally:
        autotune.apply(before)


def test_stored_table_applies_by_signature(engine, tmp_path):
    g = gp.rmat(8, 8, 0.57, 0.19, 0.19, 3)
    scheds = [gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, 100) for p in gp.motifs_3_to_5()[:3]]
    p = tmp_path / "tables.json"
    autotune.save({"chunk": 3, "_ms": 1.0}, p, autotune.signature(g, scheds))
    before = autotune.current()
    try:
        assert autotune.apply_stored(g, scheds[:2], p) is None  # another pattern set
        t = autotune.apply_stored(g, scheds, p)
        assert t["chunk"] == 3 and gp.get_option("chunk") == 3
    finally:
        autotune.apply(before)
