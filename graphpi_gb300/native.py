"""ctypes bindings of the C ABI (include/gpm.h, include/gpm_gen.h)."""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libgraphpi_gb300.so"
GEN_LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libgpm_gen.so"

GPM_OK = 0
STATUS = {
    0: "GPM_OK",
    1: "GPM_ERR_INVALID_ARG",
    2: "GPM_ERR_OOM",
    3: "GPM_ERR_CUDA",
    4: "GPM_ERR_TIMEOUT",
    5: "GPM_ERR_OVERFLOW",
    6: "GPM_ERR_UNSUPPORTED",
    7: "GPM_ERR_NO_DEVICE",
}


class GpmError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str):
        super().__init__(f"{where}: {STATUS.get(code, code)}: {msg}")
        self.code = code


class U128(C.Structure):
    _fields_ = [("lo", C.c_uint64), ("hi", C.c_uint64)]

    @property
    def value(self) -> int:
        return (self.hi << 64) | self.lo


P = C.c_void_p
I32, I64, U64 = C.c_int32, C.c_int64, C.c_uint64
PI32, PI64, PU64 = C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_uint64)
PU32 = C.POINTER(C.c_uint32)

# name: (restype, argtypes)
SIGNATURES = {
    "gpm_last_error": (C.c_char_p, []),
    "gpm_set_device": (I32, [I32]),
    "gpm_graph_create": (I32, [I32, P, P, I32, C.POINTER(P)]),
    "gpm_graph_from_edges": (I32, [I32, C.c_int64, P, P, I32, C.POINTER(P)]),
    "gpm_graph_download": (I32, [P, P, P]),
    "gpm_graph_destroy": (I32, [P]),
    "gpm_graph_device_csr": (I32, [P, I32, C.POINTER(P), C.POINTER(P)]),
    "gpm_graph_stats": (I32, [P, PI64, PI64, PI64, PI64]),
    "gpm_tri_count": (I32, [P, PU64]),
    "gpm_clique_count": (I32, [P, I32, C.POINTER(U128)]),
    "gpm_motifs": (I32, [I32, P, I32, PI32]),
    "gpm_pattern_multiplicity": (I32, [I32, P, PI64]),
    "gpm_schedule_build": (I32, [I32, P, I32, I32, I32, I64, U64, I64, P, I32, PI32, PI32]),
    "gpm_schedule_analyze": (I32, [P, I32, PI32]),
    "gpm_plan_info": (I32, [P, I32, P, I32]),
    "gpm_schedule_candidates": (I32, [I32, P, I32, I32, I64, U64, I64, P, P, P, P, I32, PI32]),
    "gpm_schedule_from_order": (I32, [I32, P, P, I32, P, I32, I32, P, I32, PI32, PI32]),
    "gpm_plan_create": (I32, [P, I32, C.POINTER(P)]),
    "gpm_plan_destroy": (I32, [P]),
    "gpm_count": (I32, [P, P, C.POINTER(U128)]),
    "gpm_batch_count": (I32, [I32, P, P, P]),
    "gpm_batch_exec_run": (I32, [C.POINTER(P), I32, P, P, P]),
    "gpm_batch_exec_destroy": (I32, [P]),
    "gpm_count_host": (I32, [I32, P, P, I32, P, P, P]),
    "gpm_count_noalloc": (I32, [I32, P, P, P, I32, C.POINTER(U128)]),
    "gpm_set_option": (I32, [C.c_char_p, I64]),
    "gpm_get_option": (I32, [C.c_char_p, PI64]),
    "gpm_last_launch_stats": (I32, [C.POINTER(C.c_double), PI64, PU64]),
    "gpm_gen_rmat": (I32, [I32, I32, C.c_double, C.c_double, C.c_double, U64, C.POINTER(PU32), C.POINTER(PI32), PI32]),
    "gpm_gen_chung_lu": (I32, [I32, C.c_double, C.c_double, I32, U64, C.POINTER(PU32), C.POINTER(PI32), PI32]),
    "gpm_csr_from_edges": (I32, [I32, I64, P, P, C.POINTER(PU32), C.POINTER(PI32)]),
    "gpm_csr_relabel_degree": (I32, [I32, P, P, C.POINTER(PU32), C.POINTER(PI32)]),
    "gpm_free": (None, [P]),
    "gpm_mlp_create": (I32, [I32, I32, U64, C.POINTER(P)]),
    "gpm_mlp_destroy": (I32, [P]),
    "gpm_mlp_params": (I32, [P, P, I32, I32]),
    "gpm_mlp_forward": (I32, [P, P, I32, P]),
    "gpm_mlp_gradients": (I32, [P, P, P, I32, P, C.POINTER(C.c_float)]),
    "gpm_mlp_train": (I32, [P, P, P, I32, I32, C.c_float, C.c_float, C.POINTER(C.c_float)]),
}

GEN_SIGNATURES = {name: SIGNATURES[name] for name in (
    "gpm_last_error", "gpm_gen_rmat", "gpm_gen_chung_lu", "gpm_csr_from_edges", "gpm_csr_relabel_degree",
    "gpm_free")}

_lib = None
_gen_lib = None


def lib() -> C.CDLL:
    """Loads the engine library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -m graphpi_gb300.build` "
                "(or __graft_entry__.build())")
        L = C.CDLL(str(LIB_PATH), mode=os.RTLD_LOCAL if hasattr(os, "RTLD_LOCAL") else 0)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def gen_lib() -> C.CDLL:
    """Loads the generator library (include/gpm_gen.h) alone: seeded graphs and
    host CSR utilities without the engine or the CUDA runtime."""
    global _gen_lib
    if _gen_lib is None:
        if not GEN_LIB_PATH.exists():
            raise RuntimeError(f"{GEN_LIB_PATH} is missing: build it with `python -m graphpi_gb300.build`")
        L = C.CDLL(str(GEN_LIB_PATH), mode=os.RTLD_LOCAL if hasattr(os, "RTLD_LOCAL") else 0)
        for name, (res, args) in GEN_SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _gen_lib = L
    return _gen_lib


def check(code: int, where: str, L: C.CDLL | None = None) -> None:
    if code != GPM_OK:
        msg = (L or lib()).gpm_last_error().decode(errors="replace")
        raise GpmError(code, where, msg)


def check_gen(code: int, where: str) -> None:
    check(code, where, gen_lib())


def set_option(key: str, value: int) -> None:
    check(lib().gpm_set_option(key.encode(), int(value)), f"gpm_set_option({key})")


def get_option(key: str) -> int:
    v = C.c_int64()
    check(lib().gpm_get_option(key.encode(), C.byref(v)), f"gpm_get_option({key})")
    return v.value


def last_launch_stats() -> tuple[float, int, int]:
    ms, n, b = C.c_double(), C.c_int64(), C.c_uint64()
    lib().gpm_last_launch_stats(C.byref(ms), C.byref(n), C.byref(b))
    return ms.value, n.value, b.value
