"""Python mirror of the reference GraphPi API over the C ABI.

Same class and method names as the reference's C++ API
(include/pattern.h, include/schedule.h, include/graph.h,
include/dataloader.h, include/motif_generator.h of thu-pacman/GraphPi), so a
script reads like the reference's drivers (tianhe/baseline_test.cpp):

    g = DataLoader().load_data(DataType.Wiki_Vote, path)
    s = Schedule(Pattern(PatternType.House), 1, 1, True, g.v_cnt, g.e_cnt, g.tri_cnt)
    assert s.is_pattern_valid
    n = g.pattern_matching(s, 0)

Counting runs on the GPU through libgraphpi_gb300.so; there is no CPU path.
Counts are exact Python ints (the engine sums in 128 bits).
"""
from __future__ import annotations

import ctypes as C
import enum
import itertools
from dataclasses import dataclass, field

import numpy as np

from . import native
from .native import U128, check, check_gen, gen_lib, lib


class PatternType(enum.IntEnum):
    Rectangle = 0
    QG3 = 1
    Pentagon = 2
    House = 3
    Hourglass = 4
    Cycle_6_Tri = 5
    Clique_7_Minus = 6


_BUILTIN_EDGES = {
    PatternType.Rectangle: (4, [(0, 1), (0, 2), (1, 3), (2, 3)]),
    PatternType.QG3: (4, [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3)]),
    PatternType.Pentagon: (5, [(0, 1), (0, 2), (1, 3), (2, 4), (3, 4)]),
    PatternType.House: (5, [(0, 1), (0, 2), (0, 3), (1, 3), (1, 4), (2, 4)]),
    PatternType.Hourglass: (6, [(0, 1), (0, 2), (0, 4), (1, 2), (1, 5), (2, 3), (3, 4), (3, 5), (4, 5)]),
    PatternType.Cycle_6_Tri: (6, [(0, 1), (0, 2), (1, 2), (1, 3), (1, 4), (2, 3), (2, 5), (0, 4), (0, 5)]),
    PatternType.Clique_7_Minus: (7, [(j, i) for i in range(7) for j in range(i) if not (i == 6 and j == 5)]),
}


class Pattern:
    """Dense adjacency matrix of a query graph (reference include/pattern.h)."""

    def __init__(self, size, clique: bool | str = False):
        if isinstance(size, PatternType):
            n, edges = _BUILTIN_EDGES[size]
            self.adj = np.zeros((n, n), dtype=np.int32)
            for a, b in edges:
                self.add_edge(a, b)
            return
        n = int(size)
        self.adj = np.zeros((n, n), dtype=np.int32)
        if isinstance(clique, str):  # Pattern(size, "0110...") row-major matrix
            if len(clique) < n * n:
                raise ValueError("adjacency string shorter than size*size")
            for i in range(n):
                for j in range(n):
                    if clique[i * n + j] == "1":
                        self.add_edge(i, j)
        elif clique:
            for i in range(n):
                for j in range(i):
                    self.add_edge(i, j)

    @classmethod
    def from_adj(cls, adj) -> "Pattern":
        a = np.asarray(adj, dtype=np.int32)
        p = cls(a.shape[0])
        p.adj[:] = ((a + a.T) > 0).astype(np.int32)
        np.fill_diagonal(p.adj, 0)
        return p

    def add_edge(self, x: int, y: int) -> None:
        self.adj[x, y] = self.adj[y, x] = 1

    def del_edge(self, x: int, y: int) -> None:
        self.adj[x, y] = self.adj[y, x] = 0

    def add_ordered_edge(self, x: int, y: int) -> None:
        self.adj[x, y] = 1

    def get_size(self) -> int:
        return self.adj.shape[0]

    def get_adj_mat_ptr(self) -> np.ndarray:
        return self.adj.reshape(-1)

    def check_connected(self) -> bool:
        n = self.get_size()
        seen, stack = {0}, [0]
        while stack:
            x = stack.pop()
            for y in np.nonzero(self.adj[x])[0]:
                if int(y) not in seen:
                    seen.add(int(y))
                    stack.append(int(y))
        return len(seen) == n

    def multiplicity(self) -> int:
        out = C.c_int64()
        a = np.ascontiguousarray(self.adj, dtype=np.int32)
        check(lib().gpm_pattern_multiplicity(self.get_size(), a.ctypes.data, C.byref(out)), "multiplicity")
        return out.value

    def __repr__(self) -> str:
        return "Pattern(" + "".join(map(str, self.adj.reshape(-1).tolist())) + ")"


class MotifGenerator:
    """All connected k-vertex patterns (reference src/motif_generator.cpp)."""

    def __init__(self, size: int):
        self.size = int(size)

    def generate(self) -> list[Pattern]:
        k = self.size
        cnt = C.c_int32()
        check(lib().gpm_motifs(k, None, 0, C.byref(cnt)), "gpm_motifs")
        buf = np.zeros(cnt.value * k * k, dtype=np.int32)
        check(lib().gpm_motifs(k, buf.ctypes.data, cnt.value, C.byref(cnt)), "gpm_motifs")
        return [Pattern.from_adj(buf[i * k * k:(i + 1) * k * k].reshape(k, k)) for i in range(cnt.value)]


def motifs_3_to_5() -> list[Pattern]:
    """The 29 connected 3-, 4- and 5-vertex motifs (2 + 6 + 21)."""
    return [p for k in (3, 4, 5) for p in MotifGenerator(k).generate()]


class Schedule:
    """Schedule tables built by the engine's schedule compiler
    (reference Schedule(pattern, valid, perf, restricts, iep, v, e, tri),
    include/schedule.h:13)."""

    def __init__(self, pattern: Pattern, performance_modeling_type: int = 1, restricts_type: int = 1,
                 use_in_exclusion_optimize: bool = True, v_cnt: int = 1, e_cnt: int = 0, tri_cnt: int = 0):
        n = pattern.get_size()
        a = np.ascontiguousarray(pattern.adj, dtype=np.int32)
        cap = 8192
        buf = np.zeros(cap, dtype=np.int64)
        nw, valid = C.c_int32(), C.c_int32()
        check(lib().gpm_schedule_build(n, a.ctypes.data, int(performance_modeling_type), int(restricts_type),
                                       1 if use_in_exclusion_optimize else 0, int(v_cnt), int(e_cnt), int(tri_cnt),
                                       buf.ctypes.data, cap, C.byref(nw), C.byref(valid)), "Schedule")
        self.is_pattern_valid = bool(valid.value)
        self.tables = buf[:nw.value].copy()
        self.pattern = pattern
        if self.is_pattern_valid:
            self._decode()

    @classmethod
    def from_tables(cls, tables) -> "Schedule":
        s = cls.__new__(cls)
        s.tables = np.asarray(tables, dtype=np.int64).copy()
        s.is_pattern_valid = True
        s.pattern = None
        s._decode()
        return s

    def _decode(self) -> None:
        t = [int(x) for x in self.tables]
        pos = 0

        def take(k=1):
            nonlocal pos
            out = t[pos:pos + k]
            pos += k
            return out

        n = take()[0]
        self.size = n
        self.adj_mat = np.array(take(n * n), dtype=np.int32).reshape(n, n)
        P = take()[0]
        self.total_prefix_num = P
        self.father_prefix_id = take(P)
        self.last = take(n)
        self.next = take(P)
        self.loop_set_prefix_id = take(n)
        R = take()[0]
        self.total_restrict_num = R
        self.restrict_last = take(n)
        self.restrict_next = take(R)
        self.restrict_index = take(R)
        npairs = take()[0]
        pr = take(2 * npairs)
        self.restrict_pair = [(pr[2 * i], pr[2 * i + 1]) for i in range(npairs)]
        self.in_exclusion_optimize_num = take()[0]
        ng = take()[0]
        self.in_exclusion_optimize_group, self.in_exclusion_optimize_val = [], []
        for _ in range(ng):
            self.in_exclusion_optimize_val.append(take()[0])
            nb = take()[0]
            grp = []
            for _ in range(nb):
                ln = take()[0]
                grp.append(take(ln))
            self.in_exclusion_optimize_group.append(grp)
        self.in_exclusion_optimize_redundancy = take()[0]
        self.multiplicity = take()[0]
        if pos != len(t):
            raise ValueError("schedule tables have trailing words")

    def label_sensitive(self) -> bool:
        """True when the count depends on vertex labels (gpm_schedule_analyze)."""
        t = np.ascontiguousarray(self.tables, dtype=np.int64)
        out = C.c_int32()
        check(lib().gpm_schedule_analyze(t.ctypes.data, len(t), C.byref(out)), "gpm_schedule_analyze")
        return bool(out.value)

    def plan_info(self) -> dict:
        """How the engine evaluates this schedule (gpm_plan_info)."""
        t = np.ascontiguousarray(self.tables, dtype=np.int64)
        info = np.zeros(6, dtype=np.int32)
        check(lib().gpm_plan_info(t.ctypes.data, len(t), info.ctypes.data, 6), "gpm_plan_info")
        keys = ("T", "L", "k", "leaf_kind", "pair_ok", "label_sensitive")
        return dict(zip(keys, map(int, info)))

    # reference getters (include/schedule.h:23-37)
    def get_size(self): return self.size

    def is_complete(self) -> bool:
        """True for a clique pattern (every pair of vertices adjacent)."""
        n = self.size
        a = np.asarray(self.adj_mat).reshape(n, n)
        return n >= 3 and bool(np.all(a + np.eye(n, dtype=a.dtype) >= 1))
    def get_total_prefix_num(self): return self.total_prefix_num
    def get_father_prefix_id(self, i): return self.father_prefix_id[i]
    def get_loop_set_prefix_id(self, i): return self.loop_set_prefix_id[i]
    def get_last(self, i): return self.last[i]
    def get_next(self, i): return self.next[i]
    def get_in_exclusion_optimize_num(self): return self.in_exclusion_optimize_num
    def get_total_restrict_num(self): return self.total_restrict_num
    def get_restrict_last(self, i): return self.restrict_last[i]
    def get_restrict_next(self, i): return self.restrict_next[i]
    def get_restrict_index(self, i): return self.restrict_index[i]
    def get_in_exclusion_optimize_redundancy(self): return self.in_exclusion_optimize_redundancy
    def get_multiplicity(self): return self.multiplicity
    def get_adj_mat_ptr(self): return self.adj_mat.reshape(-1)


MAX_PAIRS = 28


def schedule_candidates(pattern: "Pattern", performance_modeling_type: int, restricts_type: int, v_cnt: int,
                        e_cnt: int, tri_cnt: int) -> list[dict]:
    """Every (loop order, restriction set) the Schedule constructor scores,
    with its analytic cost (gpm_schedule_candidates)."""
    n = pattern.get_size()
    a = np.ascontiguousarray(pattern.adj, dtype=np.int32)
    cnt = C.c_int32()
    check(lib().gpm_schedule_candidates(n, a.ctypes.data, performance_modeling_type, restricts_type, v_cnt, e_cnt,
                                        tri_cnt, None, None, None, None, 0, C.byref(cnt)), "candidates")
    k = cnt.value
    orders = np.zeros(k * n, dtype=np.int32)
    npairs = np.zeros(k, dtype=np.int32)
    pairs = np.zeros(k * 2 * MAX_PAIRS, dtype=np.int32)
    costs = np.zeros(k, dtype=np.float64)
    check(lib().gpm_schedule_candidates(n, a.ctypes.data, performance_modeling_type, restricts_type, v_cnt, e_cnt,
                                        tri_cnt, orders.ctypes.data, npairs.ctypes.data, pairs.ctypes.data,
                                        costs.ctypes.data, k, C.byref(cnt)), "candidates")
    out = []
    for i in range(k):
        pr = pairs[i * 2 * MAX_PAIRS: i * 2 * MAX_PAIRS + 2 * npairs[i]].reshape(-1, 2)
        out.append({"order": orders[i * n:(i + 1) * n].tolist(), "pairs": [tuple(map(int, x)) for x in pr],
                    "cost": float(costs[i])})
    return out


def schedule_from_order(pattern: "Pattern", order, pairs, use_in_exclusion_optimize: bool = True,
                        restricts_type: int = 1) -> "Schedule":
    """The schedule for one candidate (gpm_schedule_from_order)."""
    n = pattern.get_size()
    a = np.ascontiguousarray(pattern.adj, dtype=np.int32)
    o = np.ascontiguousarray(order, dtype=np.int32)
    pr = np.ascontiguousarray(np.array(pairs, dtype=np.int32).reshape(-1))
    buf = np.zeros(8192, dtype=np.int64)
    nw, valid = C.c_int32(), C.c_int32()
    check(lib().gpm_schedule_from_order(n, a.ctypes.data, o.ctypes.data, len(pr) // 2, pr.ctypes.data if len(pr) else None,
                                        1 if use_in_exclusion_optimize else 0, restricts_type, buf.ctypes.data,
                                        len(buf), C.byref(nw), C.byref(valid)), "schedule_from_order")
    if not valid.value:
        raise ValueError("order is not prefix-connected")
    s = Schedule.from_tables(buf[:nw.value])
    s.pattern = pattern
    return s


class Plan:
    """A schedule compiled for the device (gpm_plan)."""

    def __init__(self, schedule: Schedule):
        if not schedule.is_pattern_valid:
            raise ValueError("invalid schedule")
        self.schedule = schedule
        self._t = np.ascontiguousarray(schedule.tables, dtype=np.int64)
        h = C.c_void_p()
        check(lib().gpm_plan_create(self._t.ctypes.data, len(self._t), C.byref(h)), "gpm_plan_create")
        self.handle = h

    def close(self) -> None:
        if getattr(self, "handle", None):
            lib().gpm_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Graph:
    """Data graph as a host CSR (`vertex` = offsets, `edge` = sorted
    neighbours, reference include/graph.h:14-15) with a lazily created device
    copy relabelled by degree."""

    def __init__(self, v_cnt: int, vertex, edge, tri_cnt: int = -1):
        self.v_cnt = int(v_cnt)
        self.vertex = np.ascontiguousarray(vertex, dtype=np.uint32)
        self.edge = np.ascontiguousarray(edge, dtype=np.int32)
        if len(self.vertex) != self.v_cnt + 1:
            raise ValueError("vertex offsets need v_cnt + 1 entries")
        self.e_cnt = int(self.vertex[-1])
        deg = np.diff(self.vertex.astype(np.int64))
        self.max_degree = int(deg.max()) if len(deg) else 0
        self.tri_cnt = int(tri_cnt)
        self._dev = None

    # -- device copy --------------------------------------------------------
    def device(self, relabel: bool = True):
        if self._dev is None:
            h = C.c_void_p()
            check(lib().gpm_graph_create(self.v_cnt, self.vertex.ctypes.data, self.edge.ctypes.data,
                                         1 if relabel else 0, C.byref(h)), "gpm_graph_create")
            self._dev = h
        return self._dev

    def close(self) -> None:
        if self._dev is not None:
            lib().gpm_graph_destroy(self._dev)
            self._dev = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def stats(self) -> dict:
        v, e, md, mi = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        check(lib().gpm_graph_stats(self.device(), C.byref(v), C.byref(e), C.byref(md), C.byref(mi)), "stats")
        return {"v_cnt": v.value, "e_cnt": e.value, "max_degree": md.value, "max_intersection_size": mi.value}

    # -- reference methods --------------------------------------------------
    def triangle_counting_mt(self, thread_count: int = 0) -> int:
        out = C.c_uint64()
        check(lib().gpm_tri_count(self.device(), C.byref(out)), "gpm_tri_count")
        return out.value

    def triangle_counting(self) -> int:
        return self.triangle_counting_mt(1)

    def ensure_tri_cnt(self) -> int:
        if self.tri_cnt < 0:
            self.tri_cnt = self.triangle_counting_mt()
        return self.tri_cnt

    def pattern_matching(self, schedule: Schedule, thread_count: int = 0, clique: bool = False) -> int:
        """Embeddings of the schedule's pattern (Graph::pattern_matching,
        reference src/graph.cpp:199-245).  clique=True on a complete pattern
        takes the clique fast path (gpm_clique_count); the count is the same
        (the reference accepts the flag and counts the same way)."""
        if clique and schedule.is_complete():
            out = U128()
            check(lib().gpm_clique_count(self.device(), schedule.get_size(), C.byref(out)), "gpm_clique_count")
            return out.value
        plan = Plan(schedule)
        try:
            out = U128()
            check(lib().gpm_count(self.device(), plan.handle, C.byref(out)), "gpm_count")
            return out.value
        finally:
            plan.close()

    def schedule(self, pattern: Pattern, performance_modeling_type: int = 1, restricts_type: int = 1,
                 use_in_exclusion_optimize: bool = True) -> Schedule:
        tri = self.ensure_tri_cnt() if performance_modeling_type else 0
        return Schedule(pattern, performance_modeling_type, restricts_type, use_in_exclusion_optimize,
                        self.v_cnt, self.e_cnt, tri)


def batch_count(graphs: list[Graph], schedules: list[Schedule]) -> list[int]:
    """All (graph, schedule) pairs in one persistent launch (gpm_batch_count)."""
    if len(graphs) != len(schedules):
        raise ValueError("graphs and schedules differ in length")
    plans = [Plan(s) for s in schedules]
    try:
        n = len(plans)
        gh = (C.c_void_p * n)(*[g.device() for g in graphs])
        ph = (C.c_void_p * n)(*[p.handle for p in plans])
        outs = (U128 * n)()
        check(lib().gpm_batch_count(n, gh, ph, outs), "gpm_batch_count")
        return [o.value for o in outs]
    finally:
        for p in plans:
            p.close()


class BatchExec:
    """A batched launch captured once in a CUDA graph and replayed
    (gpm_batch_exec_run).  Options in force at the first run (grid, chunk,
    staging) are baked in; the stripe options are read at every replay."""

    def __init__(self, graphs: list[Graph], schedules: list[Schedule]):
        if len(graphs) != len(schedules):
            raise ValueError("graphs and schedules differ in length")
        self.graphs = graphs
        self.plans = [Plan(s) for s in schedules]
        self.n = len(self.plans)
        self._gh = (C.c_void_p * self.n)(*[g.device() for g in graphs])
        self._ph = (C.c_void_p * self.n)(*[p.handle for p in self.plans])
        self._exec = C.c_void_p()

    def run(self) -> list[int]:
        outs = (U128 * self.n)()
        check(lib().gpm_batch_exec_run(C.byref(self._exec), self.n, self._gh, self._ph, outs), "gpm_batch_exec_run")
        return [o.value for o in outs]

    def close(self) -> None:
        if self._exec:
            lib().gpm_batch_exec_destroy(self._exec)
            self._exec = C.c_void_p()
        for p in self.plans:
            p.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def count_host(graph: Graph, schedules: list[Schedule]) -> list[int]:
    """One-shot host-buffer path (gpm_count_host): upload, relabel, batched
    count, download, free."""
    tabs = [np.ascontiguousarray(s.tables, dtype=np.int64) for s in schedules]
    flat = np.ascontiguousarray(np.concatenate(tabs))
    nw = np.array([len(t) for t in tabs], dtype=np.int32)
    outs = (U128 * len(tabs))()
    check(lib().gpm_count_host(graph.v_cnt, graph.vertex.ctypes.data, graph.edge.ctypes.data, len(tabs),
                               flat.ctypes.data, nw.ctypes.data, outs), "gpm_count_host")
    return [o.value for o in outs]


# ---------------------------------------------------------------------------
# data graphs

def _take_csr(rp, cl, n) -> tuple[np.ndarray, np.ndarray]:
    e = rp[n]
    vertex = np.ctypeslib.as_array(rp, shape=(n + 1,)).copy()
    edge = np.ctypeslib.as_array(cl, shape=(max(e, 1),))[:e].copy()
    gen_lib().gpm_free(C.cast(rp, C.c_void_p))
    gen_lib().gpm_free(C.cast(cl, C.c_void_p))
    return vertex, edge


def rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
         seed: int = 2) -> Graph:
    rp, cl, n = C.POINTER(C.c_uint32)(), C.POINTER(C.c_int32)(), C.c_int32()
    check_gen(gen_lib().gpm_gen_rmat(scale, edge_factor, a, b, c, seed, C.byref(rp), C.byref(cl), C.byref(n)), "rmat")
    vertex, edge = _take_csr(rp, cl, n.value)
    return Graph(n.value, vertex, edge)


def chung_lu(n: int, avg_degree: float, gamma: float, max_degree: int = 0, seed: int = 1) -> Graph:
    rp, cl, nv = C.POINTER(C.c_uint32)(), C.POINTER(C.c_int32)(), C.c_int32()
    check_gen(gen_lib().gpm_gen_chung_lu(n, avg_degree, gamma, max_degree, seed, C.byref(rp), C.byref(cl),
                                         C.byref(nv)), "chung_lu")
    vertex, edge = _take_csr(rp, cl, nv.value)
    return Graph(nv.value, vertex, edge)


def from_edges(v_cnt: int, src, dst, on_device: bool = False) -> Graph:
    """Graph from undirected edges (self loops and duplicates dropped).
    on_device: sort and deduplicate on the GPU (gpm_graph_from_edges); the
    device copy is kept and the host CSR downloaded."""
    s = np.ascontiguousarray(src, dtype=np.int32)
    d = np.ascontiguousarray(dst, dtype=np.int32)
    if on_device:
        h = C.c_void_p()
        check(lib().gpm_graph_from_edges(v_cnt, len(s), s.ctypes.data, d.ctypes.data, 1, C.byref(h)),
              "gpm_graph_from_edges")
        e = C.c_int64()
        check(lib().gpm_graph_stats(h, None, C.byref(e), None, None), "gpm_graph_stats")
        vertex = np.zeros(v_cnt + 1, dtype=np.uint32)
        edge = np.zeros(max(1, e.value), dtype=np.int32)
        check(lib().gpm_graph_download(h, vertex.ctypes.data, edge.ctypes.data), "gpm_graph_download")
        g = Graph(v_cnt, vertex, edge[:e.value])
        g._dev = h
        return g
    rp, cl = C.POINTER(C.c_uint32)(), C.POINTER(C.c_int32)()
    check_gen(gen_lib().gpm_csr_from_edges(v_cnt, len(s), s.ctypes.data, d.ctypes.data, C.byref(rp), C.byref(cl)),
              "from_edges")
    vertex, edge = _take_csr(rp, cl, v_cnt)
    return Graph(v_cnt, vertex, edge)


def relabel_by_degree(g: Graph) -> Graph:
    rp, cl = C.POINTER(C.c_uint32)(), C.POINTER(C.c_int32)()
    check_gen(gen_lib().gpm_csr_relabel_degree(g.v_cnt, g.vertex.ctypes.data, g.edge.ctypes.data, C.byref(rp),
                                               C.byref(cl)), "relabel")
    vertex, edge = _take_csr(rp, cl, g.v_cnt)
    return Graph(g.v_cnt, vertex, edge, g.tri_cnt)


def complete_graph(n: int) -> Graph:
    src, dst = zip(*[(i, j) for i in range(n) for j in range(i)])
    g = from_edges(n, src, dst)
    g.tri_cnt = n * (n - 1) * (n - 2) // 6
    return g


class DataType(enum.IntEnum):
    Patents = 0
    Orkut = 1
    complete8 = 2
    LiveJournal = 3
    MiCo = 4
    Twitter = 5
    CiteSeer = 6
    Wiki_Vote = 7
    Invalid = 8


_TRI = {DataType.Patents: 7515023, DataType.LiveJournal: 177820130, DataType.MiCo: 12534960,
        DataType.CiteSeer: 1166, DataType.Wiki_Vote: 608389, DataType.Orkut: 627584181,
        DataType.Twitter: 34824916864}


class DataLoader:
    """Text edge lists and the raw binary CSR format
    (reference src/dataloader.cpp:20-190)."""

    def load_data(self, data_type: DataType, path: str, oriented_type: int = 0) -> Graph | None:
        if data_type == DataType.Twitter:
            # header {v_cnt, e_cnt, max_degree}, vertex[v_cnt + 1], edge[e_cnt],
            # little-endian uint32 (src/dataloader.cpp:165-190)
            raw = np.fromfile(path, dtype="<u4")
            if len(raw) < 4:
                return None
            v, e = int(raw[0]), int(raw[1])
            if len(raw) < 4 + v + e:
                return None
            vertex = raw[3:4 + v].astype(np.uint32)
            edge = raw[4 + v:4 + v + e].astype(np.int32)
            if int(vertex[0]) != 0 or int(vertex[-1]) != e:
                return None
            return Graph(v, vertex, edge, _TRI[data_type])
        with open(path) as f:
            ints = np.array(f.read().split(), dtype=np.int64)
        v_hdr, e_hdr = int(ints[0]), int(ints[1])
        pairs = ints[2:2 + 2 * ((len(ints) - 2) // 2)].reshape(-1, 2)
        if len(pairs) != e_hdr:
            return None
        pairs = pairs[pairs[:, 0] != pairs[:, 1]]
        # ids by first appearance (src/dataloader.cpp:79-81)
        flat = pairs.reshape(-1)
        uniq, first = np.unique(flat, return_index=True)
        order = np.argsort(first, kind="stable")
        remap = np.empty(len(uniq), dtype=np.int64)
        remap[order] = np.arange(len(uniq))
        ids = remap[np.searchsorted(uniq, flat)].reshape(-1, 2)
        if len(uniq) != v_hdr:
            return None
        if oriented_type:
            deg = np.bincount(ids.reshape(-1), minlength=v_hdr)
            key = -deg if oriented_type == 1 else deg
            rank = np.argsort(key, kind="stable")
            new_id = np.empty(v_hdr, dtype=np.int64)
            new_id[rank] = np.arange(v_hdr)
            ids = new_id[ids]
        # the CSR is built on the GPU (gpm_graph_from_edges), on the host
        # only when no CUDA device is present
        try:
            g = from_edges(v_hdr, ids[:, 0], ids[:, 1], on_device=True)
        except native.GpmError as e:
            if e.code != 7:  # GPM_ERR_NO_DEVICE
                raise
            g = from_edges(v_hdr, ids[:, 0], ids[:, 1])
        g.tri_cnt = _TRI.get(data_type, -1)
        return g

    def load_complete(self, clique_size: int) -> Graph:
        return complete_graph(clique_size)
