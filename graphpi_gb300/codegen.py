"""Per-schedule kernels from a code generator.

The engine's matcher (match_core.cuh) interprets a compiled plan: one
kernel runs every schedule, reading loop sets, restriction masks, prefix
chains and inclusion-exclusion groups from tables.  This module instead
emits, for each schedule, CUDA source whose nested loops carry those tables
as constants — the schedule's loop nest written out the way the reference's
code generator writes it for the CPU (tianhe/code_generator.cpp:47-132,
print_block :15-38), but with warp-cooperative set operations — and compiles
it with nvcc for sm_103a at run time (cached in-tree by content hash).

What one generated schedule does (Graph::pattern_matching and
pattern_matching_aggressive_func, reference src/graph.cpp:199-398):
  * a task is a first-level edge (v0, v1) of the device CSR (or a root v0
    when the inclusion-exclusion tail starts at depth 1), taken from stripes
    exactly as the interpreter takes them, so raw sums compare stripe by
    stripe;
  * depth d >= 2 is a for-loop over its loop set clipped below the
    restriction bound, skipping chosen vertices, building the depth's prefix
    sets (warp intersections into per-warp scratch slots), with early exit
    on an empty set;
  * the last loop's set is never written: its size below the bound and
    minus the chosen vertices is counted during the intersection;
  * an inclusion-exclusion tail evaluates each distinct block once and
    combines the groups in 128-bit integers.
Load balance without waits: a task whose depth-2 loop is longer than a
threshold is not run in the first launch; it is cut into slices of its
depth-2 candidates, queued, and a second launch runs the slices (the sum
over a loop is the sum over its parts).
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import subprocess
from pathlib import Path

import numpy as np

from . import native

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
GEN_DIR = PKG / "_build" / "gen"


class _Sched:
    """The schedule tables decoded into the lists the generator walks."""

    def __init__(self, s):
        self.n = s.size
        self.father = list(s.father_prefix_id)
        self.P = s.total_prefix_num
        self.ls = list(s.loop_set_prefix_id)
        self.k = s.in_exclusion_optimize_num
        self.T = self.n - self.k if self.k else self.n - 1
        self.chains = []
        for d in range(self.n):
            c, p = [], s.last[d]
            while p != -1:
                c.append(p)
                p = s.next[p]
            self.chains.append(c)
        self.restr = []
        self.any_restr = s.total_restrict_num > 0
        for d in range(self.n):
            r, i = [], s.restrict_last[d]
            while i != -1:
                r.append(s.restrict_index[i])
                i = s.restrict_next[i]
            self.restr.append(r)
        self.groups = [(int(v), [list(b) for b in g]) for v, g in
                       zip(s.in_exclusion_optimize_val, s.in_exclusion_optimize_group)]
        self.redundancy = s.in_exclusion_optimize_redundancy
        # scratch slots: one per prefix with a father, then two temporaries
        self.slot = {}
        for p in range(self.P):
            if self.father[p] != -1:
                self.slot[p] = len(self.slot)
        self.nslots = len(self.slot) + 2
        self.tmp0 = len(self.slot)
        # the last loop's set, counted without being written (no tail)
        self.fused = None
        if self.k == 0 and self.n >= 3:
            q = self.ls[self.n - 1]
            L = self.n - 2
            used = [self.ls[d] for d in range(self.n) if d != self.n - 1]
            if q in self.chains[L] and q not in self.father and q not in used and self.father[q] != -1:
                self.fused = q


def _bound(sc: _Sched, d: int) -> str | None:
    r = sc.restr[d]
    if not r:
        return None
    terms = [f"ch[{j}]" for j in r]
    e = terms[0]
    for t in terms[1:]:
        e = f"min({e}, {t})"
    return e


def _chain(sc: _Sched, d: int, ind: str, skip: str) -> list[str]:
    """Builds the prefix sets of depth d for the candidate (nv, dv)."""
    out = []
    for p in sc.chains[d]:
        if p == sc.fused:
            continue
        f = sc.father[p]
        if f == -1:
            out.append(f"{ind}S{p} = nv; N{p} = dv;")
        else:
            out.append(f"{ind}S{p} = scr + (size_t){sc.slot[p]} * cap;")
            out.append(f"{ind}N{p} = isect_store(S{f}, N{f}, nv, dv, (int*)S{p}, lane);")
            out.append(f"{ind}if (N{p} == 0) {skip}")
    return out


def _tail(sc: _Sched, ind: str) -> list[str]:
    """The work at depth T once chosen[0, T) and every set exist."""
    T, out = sc.T, []
    if sc.k == 0:
        q = sc.ls[T]
        b = _bound(sc, T)
        if b is not None and sc.any_restr:
            out.append(f"{ind}acc += count_outside(S{q}, lower_bound_u(S{q}, N{q}, {b}), ch, {T}, lane);")
        else:
            out.append(f"{ind}acc += count_outside(S{q}, N{q}, ch, {T}, lane);")
        return out
    # inclusion-exclusion: each distinct block once
    out.append(f"{ind}{{")
    i2 = ind + "    "
    blocks = {}
    for _, grp in sc.groups:
        for blk in grp:
            blocks.setdefault(tuple(blk), len(blocks))
    for i in range(sc.k):
        q = sc.ls[T + i]
        out.append(f"{i2}const long long u{i} = count_outside(S{q}, N{q}, ch, {T}, lane);")
    cond = " || ".join(f"u{i} == 0" for i in range(sc.k))
    out.append(f"{i2}if (!({cond})) {{")
    i3 = i2 + "    "
    for blk, b in blocks.items():
        if len(blk) == 1:
            out.append(f"{i3}const long long w{b} = u{blk[0]};")
            continue
        sets = [sc.ls[T + m] for m in blk]
        out.append(f"{i3}long long w{b} = 0;")
        out.append(f"{i3}{{")
        i4 = i3 + "    "
        out.append(f"{i4}const int* A = S{sets[0]}; int na = N{sets[0]};")
        for j, q in enumerate(sets[1:-1]):
            out.append(f"{i4}if (na > 0) {{ int* dst = scr + (size_t){sc.tmp0 + (j & 1)} * cap; "
                       f"na = isect_store(A, na, S{q}, N{q}, dst, lane); A = dst; }}")
        out.append(f"{i4}if (na > 0) w{b} = isect_count(A, na, S{sets[-1]}, N{sets[-1]}, INT_MAX, ch, {T}, lane);")
        out.append(f"{i3}}}")
    for v, grp in sc.groups:
        prod = " * ".join(f"(__int128)w{blocks[tuple(b)]}" for b in grp)
        out.append(f"{i3}acc += (__int128)({v}) * {prod};")
    out.append(f"{i2}}}")
    out.append(f"{ind}}}")
    return out


def _level(sc: _Sched, d: int, ind: str) -> list[str]:
    """The loop of depth d (2 <= d < T) and everything below it."""
    out = []
    ls = sc.ls[d]
    b = _bound(sc, d)
    out.append(f"{ind}{{")
    i1 = ind + "    "
    out.append(f"{i1}const int* L{d} = S{ls};")
    if b is not None:
        out.append(f"{i1}const int n{d} = lower_bound_u(S{ls}, N{ls}, {b});")
    else:
        out.append(f"{i1}const int n{d} = N{ls};")
    if d == 2:
        out.append(f"{i1}n2_out = n2;")
        out.append(f"{i1}if (split2 > 0 && n2 > split2) return 0;  // deferred: run as slices")
        out.append(f"{i1}const int e2 = min(n2, hi2);")
        loop = f"for (int i2 = lo2; i2 < e2; ++i2)"
    else:
        loop = f"for (int i{d} = 0; i{d} < n{d}; ++i{d})"
    out.append(f"{i1}{loop} {{")
    i2 = i1 + "    "
    out.append(f"{i2}const int v = L{d}[i{d}];")
    dup = " || ".join(f"v == ch[{j}]" for j in range(d))
    out.append(f"{i2}if ({dup}) continue;")
    out.append(f"{i2}const int* nv = g.col + g.rowptr[v];")
    out.append(f"{i2}const int dv = (int)(g.rowptr[v + 1] - g.rowptr[v]);")
    out.extend(_chain(sc, d, i2, "continue;"))
    out.append(f"{i2}ch[{d}] = v;")
    if sc.fused is not None and d == sc.n - 2:
        q = sc.fused
        f = sc.father[q]
        bt = _bound(sc, sc.n - 1)
        bnd = bt if (bt is not None and sc.any_restr) else "INT_MAX"
        out.append(f"{i2}acc += isect_count(S{f}, N{f}, nv, dv, {bnd}, ch, {sc.n - 1}, lane);")
    elif d + 1 == sc.T:
        out.extend(_tail(sc, i2))
    else:
        out.extend(_level(sc, d + 1, i2))
    out.append(f"{i1}}}")
    out.append(f"{ind}}}")
    return out


def _task(sc: _Sched, i: int) -> str:
    P = sc.P
    L = [f"// schedule {i}: {sc.n} vertices, tail at depth {sc.T}, inclusion-exclusion length {sc.k}",
         f"__device__ __int128 g{i}_task(const GraphView& g, int* scr, int cap, int v0, int v1, int lo2, int hi2,",
         "                              int split2, int& n2_out, int lane) {",
         "    int ch[kMaxN];",
         "    __int128 acc = 0;",
         "    n2_out = 0;",
         "    (void)lo2; (void)hi2; (void)split2; (void)scr; (void)cap;"]
    L.append("    " + " ".join(f"const int* S{p} = nullptr; int N{p} = 0;" for p in range(P)))
    L.append("    ch[0] = v0;")
    L.append("    {")
    L.append("        const int* nv = g.col + g.rowptr[v0];")
    L.append("        const int dv = (int)(g.rowptr[v0 + 1] - g.rowptr[v0]);")
    L.extend(_chain(sc, 0, "        ", "return 0;"))
    L.append("    }")
    if sc.T == 1:
        L.extend(_tail(sc, "    "))
        L.append("    return acc;")
        L.append("}")
        return "\n".join(L)
    b = _bound(sc, 1)
    if b is not None:
        L.append(f"    if (v1 >= {b}) return 0;")
    L.append("    if (v1 == v0) return 0;")
    L.append("    {")
    L.append("        const int* nv = g.col + g.rowptr[v1];")
    L.append("        const int dv = (int)(g.rowptr[v1 + 1] - g.rowptr[v1]);")
    L.extend(_chain(sc, 1, "        ", "return 0;"))
    L.append("        ch[1] = v1;")
    if sc.fused is not None and sc.n - 2 == 1:
        # the last loop (depth 2) counted during the intersection of depth 1
        q = sc.fused
        f = sc.father[q]
        bt = _bound(sc, 2)
        bnd = bt if (bt is not None and sc.any_restr) else "INT_MAX"
        L.append(f"        acc += isect_count(S{f}, N{f}, nv, dv, {bnd}, ch, 2, lane);")
        L.append("        return acc;")
    L.append("    }")
    if sc.fused is not None and sc.n - 2 == 1:
        pass  # counted above
    elif sc.T == 2:
        L.extend(_tail(sc, "    "))
    else:
        L.extend(_level(sc, 2, "    "))
    L.append("    return acc;")
    L.append("}")
    return "\n".join(L)


_KERNELS = r'''
// first launch: whole tasks; tasks with a long depth-2 loop become queued slices
__global__ void __launch_bounds__(256) g{i}_first(GraphView g, int* scratch, long long per_warp, int cap,
        unsigned long long* cursor, unsigned long long* out, unsigned long long stripes, unsigned long long stripe,
        int chunk, GenItem* queue, unsigned long long* qtail, unsigned long long qcap, int split2) {
    const int lane = threadIdx.x & 31;
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int* scr = scratch + gw * per_warp;
    const unsigned long long ntasks = {root} ? (unsigned long long)g.v_cnt : g.e_cnt;
    __int128 acc = 0;
    int cur_v = -1;
    unsigned cur_lo = 0, cur_hi = 0;
    for (;;) {
        unsigned long long q = 0;
        if (lane == 0) q = atomicAdd(cursor, 1ull);
        q = __shfl_sync(kFull, q, 0);
        const unsigned long long i0 = q * (unsigned long long)chunk;
        if (i0 * stripes + stripe >= ntasks) break;
        for (unsigned long long i = i0; i < i0 + (unsigned long long)chunk; ++i) {
            const unsigned long long t = i * stripes + stripe;
            if (t >= ntasks) break;
            int v0 = (int)t, v1 = -1;
            if (!{root}) {
                const unsigned e = (unsigned)t;
                if (cur_v < 0 || e < cur_lo || e >= cur_hi) {
                    int lo = 0, hi = g.v_cnt;
                    while (lo < hi) {
                        int mid = (lo + hi + 1) >> 1;
                        if (g.rowptr[mid] <= e) lo = mid;
                        else hi = mid - 1;
                    }
                    cur_v = lo;
                    cur_lo = g.rowptr[lo];
                    cur_hi = g.rowptr[lo + 1];
                }
                v0 = cur_v;
                v1 = g.col[e];
            }
            int n2 = 0;
            acc += g{i}_task(g, scr, cap, v0, v1, 0, INT_MAX, split2, n2, lane);
            if (split2 > 0 && n2 > split2) {
                // slices of about n2 / 1024 candidates, queued when they fit
                const int slice = max(1, (n2 + 1023) / 1024);
                const unsigned long long m = (unsigned long long)((n2 + slice - 1) / slice);
                unsigned long long at = ~0ull;
                if (lane == 0) {
                    unsigned long long old = *(volatile unsigned long long*)qtail;
                    for (int tries = 0; tries < (1 << 20) && old + m <= qcap; ++tries) {
                        const unsigned long long got = atomicCAS(qtail, old, old + m);
                        if (got == old) {
                            at = old;
                            break;
                        }
                        old = got;
                    }
                }
                at = __shfl_sync(kFull, at, 0);
                if (at == ~0ull) {
                    int dummy = 0;
                    acc += g{i}_task(g, scr, cap, v0, v1, 0, INT_MAX, 0, dummy, lane);
                } else {
                    for (unsigned long long j = lane; j < m; j += 32) {
                        GenItem it;
                        it.t = t;
                        it.lo = (int)(j * slice);
                        it.hi = (int)min((unsigned long long)n2, (j + 1) * slice);
                        queue[at + j] = it;
                    }
                }
            }
        }
    }
    if (lane == 0 && acc != 0) add128(out, acc);
}

// second launch: the queued slices
__global__ void __launch_bounds__(256) g{i}_slices(GraphView g, int* scratch, long long per_warp, int cap,
        unsigned long long* head, unsigned long long* out, const GenItem* queue, const unsigned long long* qtail) {
    const int lane = threadIdx.x & 31;
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int* scr = scratch + gw * per_warp;
    const unsigned long long n = *qtail;
    __int128 acc = 0;
    for (;;) {
        unsigned long long q = 0;
        if (lane == 0) q = atomicAdd(head, 1ull);
        q = __shfl_sync(kFull, q, 0);
        if (q >= n) break;
        const GenItem it = queue[q];
        const unsigned e = (unsigned)it.t;
        int lo = 0, hi = g.v_cnt;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (g.rowptr[mid] <= e) lo = mid;
            else hi = mid - 1;
        }
        int dummy = 0;
        acc += g{i}_task(g, scr, cap, lo, g.col[e], it.lo, it.hi, 0, dummy, lane);
    }
    if (lane == 0 && acc != 0) add128(out, acc);
}
'''

_PRELUDE = r'''// Generated by graphpi_gb300/codegen.py: one specialised loop nest per
// schedule.  Do not edit; regenerated from the schedule tables.
#include <cuda_runtime.h>
#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstring>
#include "gpm_internal.h"

namespace gpm {
#include "match_core.cuh"

struct GenItem {
    unsigned long long t;  // first-level task
    int lo, hi;            // depth-2 candidates [lo, hi)
};
'''

_HOST = r'''
}  // namespace gpm

using namespace gpm;

namespace {
struct Buffers {
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    GenItem* queue = nullptr;
    unsigned long long* small = nullptr;  // cursor, head, qtail, out[2]
    cudaEvent_t e0 = nullptr, e1 = nullptr;
};
Buffers buf;
const unsigned long long kQueueCap = 1ull << 22;
const int kNslots[] = {@NSLOTS@};
const int kRoot[] = {@ROOTS@};
}  // namespace

extern "C" __attribute__((visibility("default"))) int gen_count(int which, int v_cnt, unsigned long long e_cnt,
        const unsigned* rowptr, const int* col, int max_degree, unsigned long long stripes, unsigned long long stripe,
        int chunk, int split2, unsigned long long* raw, float* ms) {
    if (which < 0 || which >= @COUNT@ || v_cnt < 1 || stripes < 1 || stripe >= stripes) return 1;
    int dev = 0, sms = 0, occ = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 3;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int threads = 256;
    const void* kfn = nullptr;
    switch (which) {
@OCC_CASES@
    }
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kfn, threads, 0) != cudaSuccess || occ < 1) return 3;
    const long long blocks = (long long)sms * std::min(occ, 2);
    const long long warps = blocks * (threads / 32);
    const int cap = max_degree > 0 ? max_degree : 1;
    const long long per_warp = (long long)kNslots[which] * cap;
    const size_t need = (size_t)warps * (size_t)per_warp * sizeof(int);
    if (buf.scratch_bytes < need) {
        if (buf.scratch) cudaFree(buf.scratch);
        buf.scratch = nullptr;
        buf.scratch_bytes = 0;
        if (cudaMalloc(&buf.scratch, need) != cudaSuccess) return 2;
        buf.scratch_bytes = need;
    }
    if (!buf.queue) {
        if (cudaMalloc(&buf.queue, sizeof(GenItem) * kQueueCap) != cudaSuccess) return 2;
        if (cudaMalloc(&buf.small, 8 * sizeof(unsigned long long)) != cudaSuccess) return 2;
        cudaEventCreate(&buf.e0);
        cudaEventCreate(&buf.e1);
    }
    cudaMemset(buf.small, 0, 8 * sizeof(unsigned long long));
    unsigned long long* cursor = buf.small;
    unsigned long long* head = buf.small + 1;
    unsigned long long* qtail = buf.small + 2;
    unsigned long long* out = buf.small + 3;
    GraphView g;
    g.rowptr = rowptr;
    g.col = col;
    g.v_cnt = v_cnt;
    g.pad_ = 0;
    g.e_cnt = e_cnt;
    const unsigned long long ntasks = kRoot[which] ? (unsigned long long)v_cnt : e_cnt;
    const unsigned long long per_stripe = (ntasks + stripes - 1) / stripes;
    const int ch = (int)std::max<unsigned long long>(1, std::min<unsigned long long>((unsigned long long)chunk, per_stripe / (unsigned long long)warps));
    cudaEventRecord(buf.e0);
    switch (which) {
@LAUNCH_CASES@
    }
    cudaEventRecord(buf.e1);
    cudaError_t e = cudaGetLastError();
    unsigned long long h[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(h, out, sizeof h, cudaMemcpyDeviceToHost);
    unsigned long long chk[8] = {0};
    if (e == cudaSuccess) e = cudaMemcpyFromSymbol(chk, g_check, sizeof chk);
    if (e != cudaSuccess) {
        fprintf(stderr, "gen_count: %s\n", cudaGetErrorString(e));
        return 3;
    }
    if (chk[0]) {
        fprintf(stderr, "gen_count: internal check %llu (%lld %lld %lld %lld)\n", chk[0], (long long)chk[1],
                (long long)chk[2], (long long)chk[3], (long long)chk[4]);
        const unsigned long long zero[8] = {0};
        cudaMemcpyToSymbol(g_check, zero, sizeof zero);
        return 3;
    }
    cudaEventElapsedTime(ms, buf.e0, buf.e1);
    raw[0] = h[0];
    raw[1] = h[1];
    return 0;
}
'''


def generate(schedules) -> str:
    """CUDA source with one loop nest, first-launch and slice kernels per
    schedule, and the host launcher gen_count(which, ...)."""
    scs = [_Sched(s) for s in schedules]
    parts = [_PRELUDE]
    for i, sc in enumerate(scs):
        parts.append(_task(sc, i))
        parts.append(_KERNELS.replace("{i}", str(i)).replace("{root}", "true" if sc.T == 1 else "false"))
    occ_cases = "\n".join(f"        case {i}: kfn = (const void*)g{i}_first; break;" for i in range(len(scs)))
    launch_cases = "\n".join(
        f"        case {i}:\n"
        f"            g{i}_first<<<(unsigned)blocks, threads>>>(g, (int*)buf.scratch, per_warp, cap, cursor, out, "
        f"stripes, stripe, ch, buf.queue, qtail, kQueueCap, {'0' if sc.T <= 2 else 'split2'});\n"
        f"            g{i}_slices<<<(unsigned)blocks, threads>>>(g, (int*)buf.scratch, per_warp, cap, head, out, "
        f"buf.queue, qtail);\n"
        f"            break;" for i, sc in enumerate(scs))
    host = _HOST
    for key, val in (("@COUNT@", str(len(scs))), ("@NSLOTS@", ", ".join(str(sc.nslots) for sc in scs)),
                     ("@ROOTS@", ", ".join("1" if sc.T == 1 else "0" for sc in scs)),
                     ("@OCC_CASES@", occ_cases), ("@LAUNCH_CASES@", launch_cases)):
        host = host.replace(key, val)
    parts.append(host)
    return "\n".join(parts)


def _nvcc() -> str:
    from .build import _nvcc as find
    return find()


class Generated:
    """Compiled per-schedule kernels for a list of schedules."""

    def __init__(self, schedules, verbose: bool = False):
        self.schedules = list(schedules)
        src = generate(self.schedules)
        deps = (CSRC / "match_core.cuh").read_text() + (CSRC / "gpm_internal.h").read_text()
        key = hashlib.sha256((src + deps).encode()).hexdigest()[:16]
        GEN_DIR.mkdir(parents=True, exist_ok=True)
        so = GEN_DIR / f"gen_{key}.so"
        if not so.exists():
            cu = GEN_DIR / f"gen_{key}.cu"
            cu.write_text(src)
            tmp = GEN_DIR / f"gen_{key}.so.tmp{os.getpid()}"
            cmd = [_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-lineinfo",
                   "-shared", "-Xcompiler", "-fPIC", f"-I{ROOT / 'include'}", f"-I{CSRC}", str(cu), "-o", str(tmp)]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"generated kernels failed to compile:\n{r.stdout}\n{r.stderr[-4000:]}")
            os.replace(tmp, so)
        self.path = so
        self.lib = C.CDLL(str(so))
        self.lib.gen_count.restype = C.c_int
        self.lib.gen_count.argtypes = [C.c_int, C.c_int, C.c_uint64, C.c_void_p, C.c_void_p, C.c_int, C.c_uint64,
                                       C.c_uint64, C.c_int, C.c_int, C.c_void_p, C.POINTER(C.c_float)]
        self.last_ms = 0.0

    def raw(self, graph, which: int, stripes: int = 1, stripe: int = 0, split2: int = 256, chunk: int = 8) -> int:
        """Undivided signed 128-bit sum of schedule `which` over the stripe
        (the engine's first-level tasks t with t mod stripes == stripe) on the
        graph's device CSR (degree-relabelled, as the interpreter counts)."""
        rp, cl = C.c_void_p(), C.c_void_p()
        # label-sensitive schedules count on the caller's ids, as the interpreter does
        caller_ids = 1 if self.schedules[which].label_sensitive() else 0
        native.check(native.lib().gpm_graph_device_csr(graph.device(), caller_ids, C.byref(rp), C.byref(cl)),
                     "gpm_graph_device_csr")
        st = graph.stats()
        out = np.zeros(2, dtype=np.uint64)
        ms = C.c_float()
        rc = self.lib.gen_count(which, graph.v_cnt, graph.e_cnt, rp, cl, st["max_degree"], stripes, stripe, chunk,
                                split2, out.ctypes.data, C.byref(ms))
        if rc != 0:
            raise native.GpmError(rc, "gen_count", "generated kernel failed (see stderr)")
        self.last_ms = ms.value
        v = int(out[0]) | (int(out[1]) << 64)
        return v - (1 << 128) if v >= (1 << 127) else v

    def count(self, graph, which: int) -> int:
        """Embeddings of schedule `which` in the graph (whole job)."""
        r = self.raw(graph, which)
        if r < 0:
            raise OverflowError("negative raw total")
        return r // self.schedules[which].get_in_exclusion_optimize_redundancy()
