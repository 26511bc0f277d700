"""The allocation-free entry point (gpm_count_noalloc), for callers that
cannot call cudaMalloc (GPU memory owned by another allocator, loops that
cannot take cudaMalloc's synchronisation).
It counts from a CSR the caller already holds in device memory, with scratch
in a fixed file-scope device array.  Checked through the C ABI against the
regular entry point, twice in a row (the array keeps the previous call's
contents, so the second call proves it clears what must start at zero).
This file sorts last so a failure here leaves every other test already run."""
import ctypes as C

import numpy as np
import pytest
import torch

import graphpi_gb300 as gp
from graphpi_gb300 import native

pytestmark = pytest.mark.gpu


def _noalloc(g, s) -> int:
    rp = torch.from_numpy(g.vertex.view(np.int32)).cuda()
    col = torch.from_numpy(g.edge).cuda()
    torch.cuda.synchronize()
    t = np.ascontiguousarray(s.tables, dtype=np.int64)
    out = native.U128()
    native.check(gp.lib().gpm_count_noalloc(g.v_cnt, rp.data_ptr(), col.data_ptr(), t.ctypes.data, len(t),
                                            C.byref(out)), "gpm_count_noalloc")
    return out.value


def test_noalloc_matches_gpm_count_twice(engine):
    gp.lib().gpm_set_device(0)
    torch.cuda.set_device(0)
    cases = [
        (gp.chung_lu(3000, 12.0, 2.2, 300, 17), [gp.Pattern(3, True), gp.Pattern(gp.PatternType.House)]),
        (gp.rmat(11, 8, 0.57, 0.19, 0.19, 4), [gp.Pattern(gp.PatternType.Rectangle), gp.Pattern(4, True)]),
    ]
    for g, pats in cases:
        tri = g.triangle_counting_mt()
        for p in pats:
            s = gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, tri)
            want = g.pattern_matching(s)
            assert _noalloc(g, s) == want
            assert _noalloc(g, s) == want


def test_noalloc_hub_cut_grid_matches_oracle(engine, oracle):
    """A hub of degree 19,999: one warp's sets need about 320 KB, so the grid
    is cut to the warps the fixed array holds (far fewer than a full grid)
    and long loops are shared with idle warps; counts equal the oracle's."""
    rng = np.random.default_rng(5)
    n = 20000
    src = np.concatenate([np.zeros(n - 1, dtype=np.int32), rng.integers(1, n, 60000, dtype=np.int32)])
    dst = np.concatenate([np.arange(1, n, dtype=np.int32), rng.integers(1, n, 60000, dtype=np.int32)])
    g = gp.from_edges(n, src, dst)
    tri = oracle.triangles(g)
    for p in (gp.Pattern(gp.PatternType.House), gp.Pattern(gp.PatternType.Rectangle)):
        s = gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, tri)
        want = oracle.count(g, s)
        assert _noalloc(g, s) == want
        assert _noalloc(g, s) == want


def test_noalloc_rejects_malformed_csr(engine):
    """The caller's CSR is checked like gpm_graph_create's: a one-way edge and
    an unsorted list are invalid arguments, not silently wrong counts."""
    s = gp.Schedule(gp.Pattern(3, True), 0, 0, False, 3, 2, 0)
    for rowptr, col in (([0, 1, 1, 1], [1]), ([0, 2, 3, 4], [2, 1, 0, 0])):
        rp = torch.tensor(rowptr, dtype=torch.int32, device="cuda")
        cl = torch.tensor(col, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        t = np.ascontiguousarray(s.tables, dtype=np.int64)
        out = native.U128()
        rc = gp.lib().gpm_count_noalloc(3, rp.data_ptr(), cl.data_ptr(), t.ctypes.data, len(t), C.byref(out))
        assert rc == 1, gp.lib().gpm_last_error()


def test_noalloc_rejects_oversized(engine):
    # one hub of degree 2,000,000: a warp's sets cannot fit the fixed scratch
    d = 2_000_000
    g = gp.from_edges(d + 1, np.zeros(d, dtype=np.int32), np.arange(1, d + 1, dtype=np.int32))
    s = gp.Schedule(gp.Pattern(gp.PatternType.House), 1, 1, True, g.v_cnt, g.e_cnt, 0)
    with pytest.raises(gp.GpmError) as ei:
        _noalloc(g, s)
    assert ei.value.code == 6
