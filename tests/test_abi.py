"""The C ABI library: loads, exports every declared symbol, validates
arguments and reports errors without touching a GPU."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import graphpi_gb300 as gp
from graphpi_gb300 import native

INCLUDE = Path(__file__).resolve().parents[1] / "include"


def declared_symbols():
    names = set()
    for h in INCLUDE.glob("*.h"):
        for m in re.finditer(r"GPM_API\s+[\w\s\*]+?\b(gpm_\w+)\s*\(", h.read_text()):
            names.add(m.group(1))
    return sorted(names)


def test_every_declared_symbol_is_exported(engine):
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(engine, s), s
        assert s in native.SIGNATURES, f"{s} has no Python binding"


def test_generator_library_stands_alone():
    """libgpm_gen.so exports every gpm_gen.h entry point and loads without
    the engine (the CPU reference arm generates its graphs with it)."""
    names = [m.group(1) for m in re.finditer(r"GPM_API\s+[\w\s\*]+?\b(gpm_\w+)\s*\(",
                                             (INCLUDE / "gpm_gen.h").read_text())]
    L = native.gen_lib()
    for s in names:
        assert hasattr(L, s), s
    g = gp.rmat(8, 8, 0.57, 0.19, 0.19, 1)
    h = gp.relabel_by_degree(g)
    assert h.e_cnt == g.e_cnt and sorted(np.diff(h.vertex.astype(np.int64)).tolist(), reverse=True) == \
        np.diff(h.vertex.astype(np.int64)).tolist()


def test_plan_rejects_bad_tables(engine):
    bad = np.array([3, 0, 1], dtype=np.int64)
    h = C.c_void_p()
    rc = engine.gpm_plan_create(bad.ctypes.data, len(bad), C.byref(h))
    assert rc == 1 and engine.gpm_last_error()
    # a valid table stream cut short
    s = gp.Schedule(gp.Pattern(gp.PatternType.House), 0, 1, True, 100, 1000, 0)
    t = np.ascontiguousarray(s.tables[:-3])
    assert engine.gpm_plan_create(t.ctypes.data, len(t), C.byref(h)) == 1


def test_plan_rejects_oversized_pattern(engine):
    t = np.array([9], dtype=np.int64)
    h = C.c_void_p()
    assert engine.gpm_plan_create(t.ctypes.data, 1, C.byref(h)) == 6


def test_options_roundtrip(engine):
    old = gp.get_option("chunk")
    gp.set_option("chunk", 4)
    assert gp.get_option("chunk") == 4
    gp.set_option("chunk", old)
    with pytest.raises(gp.GpmError):
        gp.set_option("no_such_knob", 1)
    with pytest.raises(gp.GpmError):
        gp.set_option("warps_per_block", 0)


def test_schedule_argument_errors(engine):
    adj = np.zeros((3, 3), dtype=np.int32)
    nw, valid = C.c_int32(), C.c_int32()
    assert engine.gpm_schedule_build(1, adj.ctypes.data, 0, 0, 0, 10, 10, 0, None, 0, C.byref(nw), C.byref(valid)) == 1
    asym = np.array([[0, 1, 0], [0, 0, 1], [0, 1, 0]], dtype=np.int32)
    buf = np.zeros(512, dtype=np.int64)
    assert engine.gpm_schedule_build(3, asym.ctypes.data, 0, 0, 0, 10, 10, 0, buf.ctypes.data, 512, C.byref(nw),
                                     C.byref(valid)) == 1


def test_generators_deterministic(engine):
    a = gp.rmat(9, 8, 0.57, 0.19, 0.19, 42)
    b = gp.rmat(9, 8, 0.57, 0.19, 0.19, 42)
    c = gp.rmat(9, 8, 0.57, 0.19, 0.19, 43)
    assert np.array_equal(a.vertex, b.vertex) and np.array_equal(a.edge, b.edge)
    assert not np.array_equal(a.edge, c.edge)
    # symmetric, sorted, no self loops
    for g in (a, gp.chung_lu(500, 6.0, 2.3, 50, 1)):
        for v in range(g.v_cnt):
            nb = g.edge[g.vertex[v]:g.vertex[v + 1]]
            assert np.all(np.diff(nb) > 0) and not np.any(nb == v)
        src = np.repeat(np.arange(g.v_cnt), np.diff(g.vertex.astype(np.int64)))
        fwd = set(zip(src.tolist(), g.edge.tolist()))
        assert all((b_, a_) in fwd for a_, b_ in fwd)


def test_relabel_host_keeps_degree_sequence(engine):
    g = gp.chung_lu(800, 8.0, 2.2, 100, 5)
    r = gp.relabel_by_degree(g)
    d0 = np.sort(np.diff(g.vertex.astype(np.int64)))[::-1]
    d1 = np.diff(r.vertex.astype(np.int64))
    assert np.array_equal(d0, d1)


def test_workload_params_stable():
    from graphpi_gb300 import workloads
    ps = workloads.uneven_params()
    assert len(ps) == 256
    assert all(1000 <= n <= 200000 and 4 <= avg <= 64 and 2.0 <= gm <= 2.8 and 0 <= m < 29
               for n, avg, gm, _, m in ps)
    assert ps == workloads.uneven_params()


def test_engine_defaults_and_option_checks(engine):
    # the shipped defaults (each chosen by measurement) and the range checks
    want = {"split": 64, "pair_leaf": 1, "leaf_batch": 0, "dense_slots": 64, "pair_max_ops": 0, "bitmap_min": 4096,
            "min_blocks": 1, "stripes": 1, "stripe": 0, "raw_sums": 0, "pair_log2": 0, "stage_tma": 1,
            "merge_vec": 1, "schedule_gpu": 1, "pool": 1}
    for k, v in want.items():
        assert gp.get_option(k) == v, k
    for bad in (("min_blocks", 2), ("split", -1), ("pair_log2", 25), ("stripes", 0), ("no_such_knob", 1)):
        with pytest.raises(gp.GpmError):
            gp.set_option(*bad)
    for k, v in want.items():
        assert gp.get_option(k) == v, k
