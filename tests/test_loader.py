"""The reference's on-disk formats (DataLoader::load_data,
src/dataloader.cpp:20-190): text edge lists and the raw binary CSR
("Twitter") format, through the Python mirror and the C++ API.  Without a
GPU the text loader builds the CSR on the host; with one it builds it on the
device (gpm_graph_from_edges) — both must give the reference's CSR."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import graphpi_gb300 as gp
from graphpi_gb300 import native

ROOT = Path(__file__).resolve().parents[1]


def _write_binary(g, path: Path) -> None:
    deg = np.diff(g.vertex.astype(np.int64))
    hdr = np.array([g.v_cnt, g.e_cnt, int(deg.max())], dtype="<u4")
    np.concatenate([hdr, g.vertex.astype("<u4"), g.edge.astype("<u4")]).tofile(path)


def _write_text(g, path: Path, shuffle_seed: int = 3) -> None:
    src = np.repeat(np.arange(g.v_cnt), np.diff(g.vertex.astype(np.int64)))
    keep = src < g.edge
    pairs = np.stack([src[keep], g.edge[keep]], axis=1)
    rng = np.random.default_rng(shuffle_seed)
    pairs = pairs[rng.permutation(len(pairs))]
    with open(path, "w") as f:
        f.write(f"{g.v_cnt} {len(pairs)}\n")
        np.savetxt(f, pairs, fmt="%d")


def _dump(tmp_path, dataset: str, path: Path, oriented: int = 0):
    exe = tmp_path / "load_dump"
    if not exe.exists():
        libdir = native.LIB_PATH.parent
        subprocess.run(["g++", "-std=c++17", "-O2", f"-I{ROOT / 'include'}", str(ROOT / "tests" / "cpp" / "load_dump.cpp"),
                        "-o", str(exe), f"-L{libdir}", "-lgraphpi_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    out = subprocess.run([str(exe), dataset, str(path), str(oriented)], capture_output=True, text=True, check=True,
                         timeout=120).stdout.splitlines()
    out = [l for l in out if not l.startswith("Success")]
    v, e, md, tri = map(int, out[0].split())
    vertex = np.array(out[1].split(), dtype=np.int64)
    edge = np.array(out[2].split(), dtype=np.int64) if e else np.zeros(0, dtype=np.int64)
    return v, e, md, tri, vertex, edge


def _connected_part(g):
    """The graph without isolated vertices (the text format needs every
    vertex to appear in an edge)."""
    deg = np.diff(g.vertex.astype(np.int64))
    keep = np.nonzero(deg > 0)[0]
    remap = -np.ones(g.v_cnt, dtype=np.int64)
    remap[keep] = np.arange(len(keep))
    src = np.repeat(np.arange(g.v_cnt), deg)
    return gp.from_edges(len(keep), remap[src], remap[g.edge])


def test_binary_format_python(engine, tmp_path):
    g = gp.rmat(10, 8, 0.57, 0.19, 0.19, 3)
    path = tmp_path / "g.bin"
    _write_binary(g, path)
    h = gp.DataLoader().load_data(gp.DataType.Twitter, str(path))
    assert h.v_cnt == g.v_cnt and np.array_equal(h.vertex, g.vertex) and np.array_equal(h.edge, g.edge)
    assert h.tri_cnt == 34824916864  # the reference's table value for this data type
    raw = np.fromfile(path, dtype="<u4")
    raw[:-5].tofile(path)  # truncated
    assert gp.DataLoader().load_data(gp.DataType.Twitter, str(path)) is None


def test_binary_format_cpp(engine, tmp_path):
    g = gp.rmat(10, 8, 0.57, 0.19, 0.19, 3)
    path = tmp_path / "g.bin"
    _write_binary(g, path)
    v, e, md, tri, vertex, edge = _dump(tmp_path, "Twitter", path)
    assert (v, e, md) == (g.v_cnt, g.e_cnt, g.max_degree)
    assert np.array_equal(vertex, g.vertex) and np.array_equal(edge, g.edge)


@pytest.mark.parametrize("oriented", [0, 1])
def test_text_format_cpp_matches_python(engine, tmp_path, oriented):
    g = _connected_part(gp.chung_lu(1500, 8.0, 2.3, 150, 29))
    path = tmp_path / "g.txt"
    _write_text(g, path)
    v, e, md, tri, vertex, edge = _dump(tmp_path, "complete8", path, oriented)
    h = gp.DataLoader().load_data(gp.DataType.complete8, str(path), oriented)
    assert (v, e) == (h.v_cnt, h.e_cnt) == (g.v_cnt, g.e_cnt)
    assert np.array_equal(vertex, h.vertex) and np.array_equal(edge, h.edge)


@pytest.mark.gpu
def test_text_loader_gpu_build_matches_host(engine, tmp_path):
    """With a GPU the loaders build the CSR on the device; the result equals
    the host builder's, and counting uses the device copy the loader made."""
    g = _connected_part(gp.rmat(12, 8, 0.57, 0.19, 0.19, 6))
    path = tmp_path / "g.txt"
    _write_text(g, path)
    for oriented in (0, 1):
        h = gp.DataLoader().load_data(gp.DataType.complete8, str(path), oriented)
        assert h._dev is not None  # built on the device
        v, e, md, tri, vertex, edge = _dump(tmp_path, "complete8", path, oriented)
        assert np.array_equal(vertex, h.vertex) and np.array_equal(edge, h.edge)
        host = gp.from_edges(h.v_cnt, np.repeat(np.arange(h.v_cnt), np.diff(h.vertex.astype(np.int64))), h.edge)
        assert np.array_equal(host.vertex, h.vertex) and np.array_equal(host.edge, h.edge)
        assert tri == h.triangle_counting_mt() == g.triangle_counting_mt()
