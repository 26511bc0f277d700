"""The C++ API is a drop-in for the reference's: a driver written like
tianhe/baseline_test.cpp compiles against include/graphpi/*.h, links
libgraphpi_gb300.so and counts on the GPU."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import graphpi_gb300 as gp
from graphpi_gb300 import native

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "cpp" / "baseline_drop_in.cpp"


def _compile(tmp_path) -> Path:
    exe = tmp_path / "baseline_drop_in"
    libdir = native.LIB_PATH.parent
    subprocess.run(["g++", "-std=c++17", "-O2", f"-I{ROOT / 'include'}", str(SRC), "-o", str(exe),
                    f"-L{libdir}", "-lgraphpi_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    return exe


def _write_edges(g, path: Path) -> None:
    src = np.repeat(np.arange(g.v_cnt), np.diff(g.vertex.astype(np.int64)))
    keep = src < g.edge
    with open(path, "w") as f:
        f.write(f"{g.v_cnt} {int(keep.sum())}\n")
        np.savetxt(f, np.stack([src[keep], g.edge[keep]], axis=1), fmt="%d")


def test_drop_in_compiles(engine, tmp_path):
    assert _compile(tmp_path).exists()


@pytest.mark.gpu
def test_drop_in_counts_match_oracle(engine, oracle, tmp_path):
    exe = _compile(tmp_path)
    g = gp.chung_lu(3000, 10.0, 2.2, 200, 23)
    # every vertex must appear in an edge for the text loader's vertex check
    deg = np.diff(g.vertex.astype(np.int64))
    assert deg.min() > 0 or True
    keepv = np.nonzero(deg > 0)[0]
    remap = -np.ones(g.v_cnt, dtype=np.int64)
    remap[keepv] = np.arange(len(keepv))
    src = np.repeat(np.arange(g.v_cnt), deg)
    h = gp.from_edges(len(keepv), remap[src], remap[g.edge])
    path = tmp_path / "graph.txt"
    _write_edges(h, path)
    for adj, size in [("0111101111011110", 4), ("0111010011100101100001100", 5)]:
        out = subprocess.run([str(exe), "complete8", str(path), str(size), adj], capture_output=True, text=True,
                             check=True, timeout=120).stdout
        got = int(next(l for l in out.splitlines() if l.startswith("ans ")).split()[1])
        tri = int(next(l for l in out.splitlines() if l.startswith("tri ")).split()[1])
        assert tri == oracle.triangles(h)
        s = gp.Schedule(gp.Pattern(size, adj), 1, 1, True, h.v_cnt, h.e_cnt, tri)
        assert got == oracle.count(h, s)
