"""Unfolded CPU code for a schedule: the CPU comparison path.  TEST
INFRASTRUCTURE ONLY (tests/ and the benchmark's CPU legs use it; the engine
never does).

The reference's code generator (tianhe/code_generator.cpp:47-132) writes,
for one schedule, C++ in which the recursion of
pattern_matching_aggressive_func (src/graph.cpp:246-398) is unrolled into
nested loops, one per depth, and compiles it into the reference as
Graph::unfold_pattern_matching.  This module writes the same kind of code in
plain C from the schedule tables (decoded as graphpi_gb300.codegen decodes
them): one loop per depth over its loop set below the restriction bound,
injectivity checks, scalar merge intersections (VertexSet::intersection,
src/vertex_set.cpp:105-119) for the prefix sets, the last level's
lower_bound and subtraction (:346-364) or the inclusion-exclusion tail
(:306-344) in 128-bit integers; roots are spread over OpenMP threads.  It is
compiled with gcc -O3 -fopenmp into oracle/_gen/ and returns the undivided
sum, so it checks against the oracle and times the unfolded CPU code beside
the interpreted one.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
OUT = ROOT / "oracle" / "_gen"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from graphpi_gb300.codegen import _Sched  # noqa: E402  (the shared table decoding)

_PRELUDE = r'''/* generated by oracle/unfolded.py: unfolded CPU loops per schedule */
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
typedef __int128 i128;

static int lb(const int* a, int n, int x) {
    int lo = 0, hi = n;
    while (lo < hi) { int m = (lo + hi) >> 1; if (a[m] < x) lo = m + 1; else hi = m; }
    return lo;
}
static int merge(const int* a, int na, const int* b, int nb, int* out) {
    int i = 0, j = 0, w = 0;
    while (i < na && j < nb) {
        if (a[i] < b[j]) ++i; else if (a[i] > b[j]) ++j; else { out[w++] = a[i]; ++i; ++j; }
    }
    return w;
}
/* |S[0, n) \ ch[0, nch)| */
static long long outside(const int* S, int n, const int* ch, int nch) {
    long long r = n;
    for (int j = 0; j < nch; ++j) { int p = lb(S, n, ch[j]); if (p < n && S[p] == ch[j]) --r; }
    return r;
}
'''


def _bound(sc, d):
    r = sc.restr[d]
    if not r:
        return None
    e = f"ch[{r[0]}]"
    for j in r[1:]:
        e = f"(ch[{j}] < {e} ? ch[{j}] : {e})"
    return e


def _chain(sc, d, ind):
    out = []
    for p in sc.chains[d]:
        f = sc.father[p]
        if f == -1:
            out.append(f"{ind}S{p} = nv; N{p} = dv;")
        else:
            out.append(f"{ind}S{p} = buf + (size_t){sc.slot[p]} * cap;")
            out.append(f"{ind}N{p} = merge(S{f}, N{f}, nv, dv, (int*)S{p});")
            out.append(f"{ind}if (N{p} == 0) continue;")
    return out


def _tail(sc, ind):
    T = sc.T
    out = []
    if sc.k == 0:
        q = sc.ls[T]
        b = _bound(sc, T)
        if b is not None and sc.any_restr:
            out.append(f"{ind}acc += outside(S{q}, lb(S{q}, N{q}, {b}), ch, {T});")
        else:
            out.append(f"{ind}acc += outside(S{q}, N{q}, ch, {T});")
        return out
    out.append(f"{ind}{{")
    i2 = ind + "    "
    for val, grp in sc.groups:
        out.append(f"{i2}{{ i128 v = {val};")
        for blk in grp:
            sets = [sc.ls[T + m] for m in blk]
            if len(sets) == 1:
                out.append(f"{i2}  if (v) v *= outside(S{sets[0]}, N{sets[0]}, ch, {T});")
            else:
                out.append(f"{i2}  if (v) {{ const int* A = S{sets[0]}; int na = N{sets[0]}; int* dst = tmp;")
                for q in sets[1:]:
                    out.append(f"{i2}    na = merge(A, na, S{q}, N{q}, dst); A = dst; dst = (dst == tmp) ? tmp2 : tmp;")
                out.append(f"{i2}    v *= outside(A, na, ch, {T}); }}")
        out.append(f"{i2}  acc += v; }}")
    out.append(f"{ind}}}")
    return out


def _level(sc, d, ind):
    out = []
    ls = sc.ls[d]
    b = _bound(sc, d)
    out.append(f"{ind}{{")
    i1 = ind + "    "
    out.append(f"{i1}const int* L{d} = S{ls};")
    n_expr = f"lb(S{ls}, N{ls}, {b})" if b is not None else f"N{ls}"
    out.append(f"{i1}const int n{d} = {n_expr};")
    out.append(f"{i1}for (int i{d} = 0; i{d} < n{d}; ++i{d}) {{")
    i2 = i1 + "    "
    out.append(f"{i2}const int v = L{d}[i{d}];")
    dup = " || ".join(f"v == ch[{j}]" for j in range(d))
    out.append(f"{i2}if ({dup}) continue;")
    out.append(f"{i2}const int* nv = col + rp[v]; const int dv = (int)(rp[v + 1] - rp[v]);")
    out.extend(_chain(sc, d, i2))
    out.append(f"{i2}ch[{d}] = v;")
    if d + 1 == sc.T:
        out.extend(_tail(sc, i2))
    else:
        out.extend(_level(sc, d + 1, i2))
    out.append(f"{i1}}}")
    out.append(f"{ind}}}")
    return out


def _function(sc, i):
    P = sc.P
    L = [f"/* schedule {i}: {sc.n} vertices, tail at depth {sc.T} */",
         f"int unf{i}(int V, const uint32_t* rp, const int32_t* col, int cap, int threads, uint64_t* out) {{",
         "    i128 total = 0;",
         "    int bad = 0;",
         "#pragma omp parallel num_threads(threads > 0 ? threads : omp_get_max_threads()) reduction(| : bad)",
         "    {",
         f"        int* buf = (int*)malloc(sizeof(int) * (size_t)cap * {max(1, len(sc.slot))});",
         "        int* tmp = (int*)malloc(sizeof(int) * (size_t)cap);",
         "        int* tmp2 = (int*)malloc(sizeof(int) * (size_t)cap);",
         "        i128 acc = 0;",
         "        if (!buf || !tmp || !tmp2) bad = 1;",
         "        if (!bad) {",
         "#pragma omp for schedule(dynamic, 16)",
         "        for (int v0 = 0; v0 < V; ++v0) {",
         "            int ch[8];",
         "            " + " ".join(f"const int* S{p} = 0; int N{p} = 0;" for p in range(P)),
         "            ch[0] = v0;",
         "            {",
         "                const int* nv = col + rp[v0]; const int dv = (int)(rp[v0 + 1] - rp[v0]);"]
    # depth 0: every prefix aliases N(v0) (no father)
    L.extend(_chain(sc, 0, "                "))
    L.append("            }")
    if sc.T == 1:
        L.extend(_tail(sc, "            "))
    else:
        L.extend(_level(sc, 1, "            "))
    L += ["        }",
          "        }",
          "#pragma omp critical",
          "        total += acc;",
          "        free(buf); free(tmp); free(tmp2);",
          "    }",
          "    if (bad) return -2;",
          "    out[0] = (uint64_t)total;",
          "    out[1] = (uint64_t)(total >> 64);",
          "    return 0;",
          "}"]
    return "\n".join(L)


def generate(schedules) -> str:
    scs = [_Sched(s) for s in schedules]
    return "\n".join([_PRELUDE] + [_function(sc, i) for i, sc in enumerate(scs)])


class Unfolded:
    """The unfolded CPU functions of a list of schedules, compiled."""

    def __init__(self, schedules):
        self.schedules = list(schedules)
        src = generate(self.schedules)
        key = hashlib.sha256(src.encode()).hexdigest()[:16]
        OUT.mkdir(parents=True, exist_ok=True)
        so = OUT / f"unfolded_{key}.so"
        if not so.exists():
            c = OUT / f"unfolded_{key}.c"
            c.write_text(src)
            tmp = OUT / f"unfolded_{key}.so.tmp{os.getpid()}"
            subprocess.run(["gcc", "-O3", "-std=gnu11", "-fPIC", "-fopenmp", "-shared", str(c), "-o", str(tmp)],
                           check=True)
            os.replace(tmp, so)
        self.lib = C.CDLL(str(so))
        for i in range(len(self.schedules)):
            f = getattr(self.lib, f"unf{i}")
            f.restype = C.c_int
            f.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]

    def raw(self, g, which: int, threads: int = 0) -> int:
        """Undivided signed sum of schedule `which` over every root."""
        deg = np.diff(g.vertex.astype(np.int64))
        cap = max(1, int(deg.max()) if len(deg) else 1)
        out = np.zeros(2, dtype=np.uint64)
        rc = getattr(self.lib, f"unf{which}")(g.v_cnt, g.vertex.ctypes.data, g.edge.ctypes.data, cap, threads,
                                              out.ctypes.data)
        assert rc == 0, rc
        v = int(out[0]) | (int(out[1]) << 64)
        return v - (1 << 128) if v >= (1 << 127) else v

    def count(self, g, which: int, threads: int = 0) -> int:
        return self.raw(g, which, threads) // self.schedules[which].get_in_exclusion_optimize_redundancy()
