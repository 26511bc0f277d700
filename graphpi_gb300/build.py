"""Builds the native library in-tree.

    graphpi_gb300/_lib/libgraphpi_gb300.so   engine: host C++ + sm_103a CUDA
    graphpi_gb300/_lib/libgpm_gen.so         the seeded graph generators and host
                                             CSR utilities alone (include/gpm_gen.h),
                                             for processes that must not load the
                                             engine (the CPU reference arm)
    oracle/liboracle.so                      CPU oracle (test infrastructure)
    oracle/_ref/libgraphpi_ref.so            reference GraphPi built from its own
                                             sources (only where they exist)

Translation units compile in parallel; one -gencode (sm_103a).  Object files
go to graphpi_gb300/_build/.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "libgraphpi_gb300.so"
GEN_LIB = LIBDIR / "libgpm_gen.so"
GEN_SOURCES = ("gen", "errors")  # seeded generators + host CSR utilities (include/gpm_gen.h)
ORACLE_SRC = ROOT / "oracle" / "oracle.c"
ORACLE_LIB = ROOT / "oracle" / "liboracle.so"
REF_SCRIPT = ROOT / "oracle" / "build_ref.sh"
# the reference checkout the oracle/_ref recipe compiles from: GRAPHPI_REFERENCE,
# else the checkout's usual location in the build container
REFERENCE = Path(os.environ.get("GRAPHPI_REFERENCE", "/root/reference"))

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CXXFLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]
INCLUDES = [f"-I{ROOT / 'include'}", f"-I{CSRC}"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build graphpi_gb300")


def _run_all(cmds: list[list[str]]) -> None:
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)) for c in cmds]
    failed = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((c, out))
    if failed:
        msg = "\n\n".join(" ".join(c) + "\n" + out for c, out in failed)
        raise RuntimeError(f"native build failed:\n{msg}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_engine(force: bool = False) -> Path:
    nvcc = _nvcc()
    OBJ.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    headers = list((ROOT / "include").rglob("*.h")) + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh"))
    cmds, objs = [], []
    for src in sorted(CSRC.glob("*.cpp")):
        obj = OBJ / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmds.append(["g++", *CXXFLAGS, *INCLUDES, "-c", str(src), "-o", str(obj)])
    for src in sorted(CSRC.glob("*.cu")):
        obj = OBJ / (src.stem + ".cu.o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmds.append([nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                         *INCLUDES, "-c", str(src), "-o", str(obj)])
    _run_all(cmds)
    if force or cmds or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run_all([[nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-Xcompiler", "-fopenmp",
                   "-Xlinker", "-Bsymbolic", "-lgomp"]])
        os.replace(tmp, LIB)
    gen_objs = [OBJ / (name + ".o") for name in GEN_SOURCES]
    if force or _stale(GEN_LIB, gen_objs):
        tmp = GEN_LIB.with_suffix(".so.tmp")
        _run_all([["g++", "-shared", "-fopenmp", "-o", str(tmp), *map(str, gen_objs)]])
        os.replace(tmp, GEN_LIB)
    return LIB


def build_oracle(force: bool = False) -> Path:
    if force or _stale(ORACLE_LIB, [ORACLE_SRC]):
        tmp = ORACLE_LIB.with_suffix(".so.tmp")
        _run_all([["gcc", "-O3", "-std=gnu11", "-fPIC", "-fopenmp", "-shared", str(ORACLE_SRC), "-o", str(tmp)]])
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_reference() -> Path | None:
    """Compiles the reference library where its sources exist (not on GPU hosts)."""
    if not (REFERENCE / "src").is_dir():
        return None
    out = ROOT / "oracle" / "_ref" / "libgraphpi_ref.so"
    srcs = list((REFERENCE / "src").glob("*.cpp")) + [ROOT / "oracle" / "ref_shim.cpp"]
    if _stale(out, srcs):
        _run_all([["bash", str(REF_SCRIPT), str(REFERENCE)]])
    return out if out.exists() else None


def build_all(force: bool = False) -> None:
    build_engine(force)
    build_oracle(force)
    build_reference()


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print(f"built {LIB}")
