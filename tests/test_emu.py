"""The matcher's device core on the CPU: graphpi_gb300/csrc/match_core.cuh
compiled as host C++ against the warp emulator (tests/emu/warp_emu.h) with
AddressSanitizer, run on small skewed graphs and compared with the oracle.

Covers, without a GPU: loop donation with every loop shared (split=1, the
most racy setting) with and without the batched leaf, the pair-sum leaf and
its dense counter arrays (every phase shared, in one-element slices), leaf
bitmaps, stripes that do not depend on the
grab size and that add up to the whole job (the multi-rank split); any
out-of-bounds access, any lane that meets a different shuffle/ballot/syncwarp
than its warp, and any internal check stops the run.  After every launch the
dense counters and leaf bitmaps must be zero again and every donation slot
released with no visitor left (the claim protocol's bookkeeping).  The
upload kernels' row search (csr_rows.cuh) runs on one emulated warp over
CSRs with long runs of empty rows and with hubs."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "graphpi_gb300" / "csrc"
EMU = ROOT / "tests" / "emu"
OUT = ROOT / "graphpi_gb300" / "_build" / "emu"

HOST_SOURCES = ["capi_host.cpp", "errors.cpp", "schedule.cpp", "pattern.cpp", "gen.cpp"]
FLAGS = ["-O1", "-g", "-fsanitize=address", "-fno-omit-frame-pointer", "-fopenmp", "-ffp-contract=off"]
INCLUDES = [f"-I{ROOT / 'include'}", f"-I{CSRC}", f"-I{EMU}"]


def _build() -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    # pair sums shared from one block of candidates on, in one-element units
    stress = ["-DGPM_PAIR_SHARE_BLOCKS=1", "-DGPM_PAIR_UNIT_LOG2=0"]
    jobs = [(["g++", "-std=c++20", *FLAGS, *stress, *INCLUDES, "-c", str(EMU / "emu_match.cpp"),
              "-o", str(OUT / "emu.o")])]
    for src in HOST_SOURCES:
        jobs.append(["g++", "-std=c++17", *FLAGS, "-DGPM_HOST_ONLY", *INCLUDES, "-c", str(CSRC / src),
                     "-o", str(OUT / (src + ".o"))])
    jobs.append(["gcc", *FLAGS, "-c", str(ROOT / "oracle" / "oracle.c"), "-o", str(OUT / "oracle.o")])
    procs = [subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True) for j in jobs]
    for j, p in zip(jobs, procs):
        out, _ = p.communicate()
        assert p.returncode == 0, " ".join(j) + "\n" + out
    exe = OUT / "emu_match"
    objs = [str(OUT / "emu.o")] + [str(OUT / (s + ".o")) for s in HOST_SOURCES] + [str(OUT / "oracle.o")]
    r = subprocess.run(["g++", "-fsanitize=address", "-fopenmp", *objs, "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


# the cases, in three groups of similar length run as concurrent processes
CASE_GROUPS = [["quick", "stripes", "rows"], ["vec", "pair"], ["pairhub", "pairtags"]]


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_device_core_on_emulated_warps():
    exe = _build()
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0")
    procs = [subprocess.Popen([str(exe), *cases], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, env=env)
             for cases in CASE_GROUPS]
    try:
        outs = [p.communicate(timeout=900) for p in procs]
    finally:
        for p in procs:
            if p.poll() is None:
                p.kill()
    for cases, p, (out, err) in zip(CASE_GROUPS, procs, outs):
        tail = " ".join(cases) + ":\n" + (out[-3000:] + "\n" + err[-3000:]).strip()
        assert p.returncode == 0, tail
        assert "PASSED (0 mismatches)" in out, tail
