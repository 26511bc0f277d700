"""Loads the CPU oracle (oracle/liboracle.so) for tests: the checker, never
the thing under test."""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
REF_LIB = ROOT / "oracle" / "_ref" / "libgraphpi_ref.so"


def reference_root() -> Path | None:
    """The reference checkout named by GRAPHPI_REFERENCE (None when unset or
    absent): tests that read its dataset skip without it."""
    v = os.environ.get("GRAPHPI_REFERENCE")
    return Path(v) if v and Path(v).is_dir() else None


class Oracle:
    def __init__(self, lib: C.CDLL):
        self.L = lib
        lib.oracle_pattern_matching.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                                C.c_void_p]
        lib.oracle_pattern_matching_roots.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                                      C.c_void_p, C.c_int64, C.c_int, C.c_void_p]
        lib.oracle_pattern_matching_roots_timed.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                                            C.c_void_p, C.c_int64, C.c_int, C.c_double,
                                                            C.c_void_p, C.c_void_p]
        lib.oracle_brute_force.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                           C.c_void_p]
        lib.oracle_triangle_count.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int]
        lib.oracle_triangle_count.restype = C.c_longlong
        lib.oracle_pattern_matching_clique.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                                       C.c_int, C.c_void_p]
        lib.oracle_stripes_raw.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                           C.c_int64, C.c_void_p, C.c_int, C.c_int, C.c_void_p]

    def count(self, g, schedule, threads: int = 0) -> int:
        t = np.ascontiguousarray(schedule.tables, dtype=np.int64)
        out = np.zeros(2, dtype=np.uint64)
        rc = self.L.oracle_pattern_matching(g.v_cnt, g.vertex.ctypes.data, g.edge.ctypes.data, t.ctypes.data,
                                            len(t), threads, out.ctypes.data)
        assert rc == 0, f"oracle failed ({rc})"
        return int(out[0]) | (int(out[1]) << 64)

    def count_clique(self, g, schedule, threads: int = 0) -> int:
        """The reference's clique function (pattern_matching_func with
        clique = true) on the schedule's loops."""
        t = np.ascontiguousarray(schedule.tables, dtype=np.int64)
        out = np.zeros(2, dtype=np.uint64)
        rc = self.L.oracle_pattern_matching_clique(g.v_cnt, g.vertex.ctypes.data, g.edge.ctypes.data, t.ctypes.data,
                                                   len(t), threads, out.ctypes.data)
        assert rc == 0, f"oracle failed ({rc})"
        return int(out[0]) | (int(out[1]) << 64)

    def raw_roots(self, g, schedule, roots, threads: int = 0) -> int:
        """Undivided signed sum over the given root vertices."""
        t = np.ascontiguousarray(schedule.tables, dtype=np.int64)
        r = np.ascontiguousarray(roots, dtype=np.int32)
        out = np.zeros(2, dtype=np.uint64)
        rc = self.L.oracle_pattern_matching_roots(g.v_cnt, g.vertex.ctypes.data, g.edge.ctypes.data, t.ctypes.data,
                                                  len(t), r.ctypes.data, len(r), threads, out.ctypes.data)
        assert rc == 0, f"oracle failed ({rc})"
        v = int(out[0]) | (int(out[1]) << 64)
        return v - (1 << 128) if v >= (1 << 127) else v

    def raw_roots_timed(self, g, schedule, roots, seconds: float, threads: int = 0) -> tuple[int, int]:
        """(undivided signed sum over the roots finished within `seconds`, how many)."""
        t = np.ascontiguousarray(schedule.tables, dtype=np.int64)
        r = np.ascontiguousarray(roots, dtype=np.int32)
        out = np.zeros(2, dtype=np.uint64)
        done = np.zeros(1, dtype=np.int64)
        rc = self.L.oracle_pattern_matching_roots_timed(g.v_cnt, g.vertex.ctypes.data, g.edge.ctypes.data,
                                                        t.ctypes.data, len(t), r.ctypes.data, len(r), threads,
                                                        seconds, done.ctypes.data, out.ctypes.data)
        assert rc == 0, f"oracle failed ({rc})"
        v = int(out[0]) | (int(out[1]) << 64)
        return (v - (1 << 128) if v >= (1 << 127) else v), int(done[0])

    def stripes_raw(self, g, tables_list, stripes: int, ids, threads: int = 0) -> list[list[int]]:
        """Undivided signed sums of the engine's first-level tasks: result[i][j]
        = schedule i (tables) over stripe ids[j] of `stripes` (tasks t with
        t mod stripes == ids[j]).  `g` must carry the numbering the engine
        counts on (the degree-relabelled CSR unless the graph was uploaded
        without relabelling)."""
        tabs = [np.ascontiguousarray(t, dtype=np.int64) for t in tables_list]
        flat = np.ascontiguousarray(np.concatenate(tabs))
        nw = np.array([len(t) for t in tabs], dtype=np.int32)
        ids = np.ascontiguousarray(ids, dtype=np.int64)
        out = np.zeros(2 * len(tabs) * len(ids), dtype=np.uint64)
        rc = self.L.oracle_stripes_raw(g.v_cnt, g.vertex.ctypes.data, g.edge.ctypes.data, len(tabs), flat.ctypes.data,
                                       nw.ctypes.data, int(stripes), ids.ctypes.data, len(ids), threads,
                                       out.ctypes.data)
        assert rc == 0, f"oracle failed ({rc})"
        res = []
        for i in range(len(tabs)):
            row = []
            for j in range(len(ids)):
                q = i * len(ids) + j
                v = int(out[2 * q]) | (int(out[2 * q + 1]) << 64)
                row.append(v - (1 << 128) if v >= (1 << 127) else v)
            res.append(row)
        return res

    def brute_force(self, g, pattern, threads: int = 0) -> int:
        a = np.ascontiguousarray(pattern.adj, dtype=np.int32)
        out = np.zeros(2, dtype=np.uint64)
        rc = self.L.oracle_brute_force(g.v_cnt, g.vertex.ctypes.data, g.edge.ctypes.data, a.shape[0], a.ctypes.data,
                                       threads, out.ctypes.data)
        assert rc == 0
        return int(out[0]) | (int(out[1]) << 64)

    def triangles(self, g, threads: int = 0) -> int:
        return self.L.oracle_triangle_count(g.v_cnt, g.vertex.ctypes.data, g.edge.ctypes.data, threads)


def load_ref() -> C.CDLL:
    """The reference library built from its own sources (oracle/_ref)."""
    R = C.CDLL(str(REF_LIB))
    R.ref_graph_from_csr.restype = C.c_void_p
    R.ref_graph_from_csr.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_longlong, C.c_int]
    R.ref_graph_free.argtypes = [C.c_void_p]
    R.ref_graph_tri.restype = C.c_longlong
    R.ref_graph_tri.argtypes = [C.c_void_p]
    R.ref_schedule_create.restype = C.c_void_p
    R.ref_schedule_create.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint,
                                      C.c_longlong, C.POINTER(C.c_int)]
    R.ref_schedule_dump.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    R.ref_schedule_free.argtypes = [C.c_void_p]
    R.ref_pattern_matching.restype = C.c_longlong
    R.ref_pattern_matching.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    R.ref_triangle_counting_mt.restype = C.c_longlong
    R.ref_triangle_counting_mt.argtypes = [C.c_void_p, C.c_int]
    R.ref_motifs.argtypes = [C.c_int, C.c_void_p, C.c_int]
    R.ref_stripes_raw.argtypes = [C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    return R


def ref_schedule_tables(R, adj, perf: int, restr: int, iep: bool, v_cnt: int, e_cnt: int, tri: int):
    """(tables, valid) of the reference's own Schedule, gpm_schedule_build layout."""
    a = np.ascontiguousarray(adj, dtype=np.int32)
    ok = C.c_int()
    s = R.ref_schedule_create(a.shape[0], a.ctypes.data, perf, restr, 1 if iep else 0, v_cnt, e_cnt, tri, C.byref(ok))
    buf = np.zeros(1 << 16, dtype=np.int64)
    n = R.ref_schedule_dump(s, buf.ctypes.data, len(buf))
    R.ref_schedule_free(s)
    assert n > 0
    return [int(x) for x in buf[:n]], bool(ok.value)


def load() -> Oracle:
    from graphpi_gb300 import build
    lib_path = build.build_oracle()
    return Oracle(C.CDLL(str(lib_path)))


def csr_checksum(g) -> str:
    h = hashlib.sha256()
    h.update(np.int64(g.v_cnt).tobytes())
    h.update(g.vertex.astype("<u4").tobytes())
    h.update(g.edge.astype("<i4").tobytes())
    return h.hexdigest()[:16]


def golden(name: str) -> dict:
    return json.loads((GOLDEN / name).read_text())
