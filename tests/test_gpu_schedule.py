"""Schedule construction on the GPU (schedule_gpu.cu): every candidate's
analytic cost computed by one GPU thread must give the host's tables word
for word — all 2 + 6 + 21 connected 3-5-vertex motifs and a sample of the
112 six-vertex ones, under every performance model and both restriction
generators."""
import numpy as np
import pytest

import graphpi_gb300 as gp

pytestmark = pytest.mark.gpu


def test_gpu_scoring_gives_the_host_tables(engine):
    pats = gp.motifs_3_to_5() + gp.MotifGenerator(6).generate()[::5]
    stats = [(7115, 201524, 608389), (4194304, 128306732, 2112625082)]
    old = gp.get_option("schedule_gpu")
    try:
        for v, e, tri in stats:
            for perf, restr in ((1, 1), (2, 2), (3, 1), (1, 2)):
                for p in pats:
                    gp.set_option("schedule_gpu", 1)
                    a = gp.Schedule(p, perf, restr, True, v, e, tri)
                    gp.set_option("schedule_gpu", 0)
                    b = gp.Schedule(p, perf, restr, True, v, e, tri)
                    assert a.is_pattern_valid == b.is_pattern_valid
                    assert np.array_equal(a.tables, b.tables), (p, perf, restr)
    finally:
        gp.set_option("schedule_gpu", old)
