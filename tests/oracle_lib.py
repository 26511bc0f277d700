"""Loads the CPU oracle (oracle/liboracle.so) for tests: the checker, never
the thing under test."""
from __future__ import annotations

import ctypes as C
import hashlib
import json
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
REF_LIB = ROOT / "oracle" / "_ref" / "libgraphpi_ref.so"


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

    def count(self, g, schedule, threads: int = 0) -> int:
        t = np.ascontiguousarray(schedule.tables, dtype=np.int64)
        out = np.zeros(2, dtype=np.uint64)
        rc = self.L.oracle_pattern_matching(g.v_cnt, g.vertex.ctypes.data, g.edge.ctypes.data, t.ctypes.data,
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

    def brute_force(self, g, pattern, threads: int = 0) -> int:
        a = np.ascontiguousarray(pattern.adj, dtype=np.int32)
        out = np.zeros(2, dtype=np.uint64)
        rc = self.L.oracle_brute_force(g.v_cnt, g.vertex.ctypes.data, g.edge.ctypes.data, a.shape[0], a.ctypes.data,
                                       threads, out.ctypes.data)
        assert rc == 0
        return int(out[0]) | (int(out[1]) << 64)

    def triangles(self, g, threads: int = 0) -> int:
        return self.L.oracle_triangle_count(g.v_cnt, g.vertex.ctypes.data, g.edge.ctypes.data, threads)


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
