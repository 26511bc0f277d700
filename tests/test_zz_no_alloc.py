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


def test_noalloc_rejects_oversized(engine):
    # one hub of degree 2,000,000: a warp's sets cannot fit the fixed scratch
    d = 2_000_000
    g = gp.from_edges(d + 1, np.zeros(d, dtype=np.int32), np.arange(1, d + 1, dtype=np.int32))
    s = gp.Schedule(gp.Pattern(gp.PatternType.House), 1, 1, True, g.v_cnt, g.e_cnt, 0)
    with pytest.raises(gp.GpmError) as ei:
        _noalloc(g, s)
    assert ei.value.code == 6
