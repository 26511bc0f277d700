"""Autotuner for the engine's launch and intersection knobs.

Counts never depend on these knobs; only speed does.  The tuner times
batched launches over a fixed sample of the work (interleaved stripes, raw
sums) and walks the knobs one at a time (coordinate descent), keeping a
value only when it is faster.  Every trial's raw sums must equal the first
trial's, otherwise it raises.  The result is a small table
{knob: value} that `apply` installs and `save`/`load` keep on disk, keyed
by the graph and pattern set it was tuned on.

Knobs (gpm_set_option):
  chunk                     first-level tasks per work-queue grab
  warps_per_block           warps per persistent block
  blocks_per_sm             persistent blocks per SM
  merge_vec                 merges over 128-bit windows of the longer list
  min_blocks                3 / 4: the kernel variants compiled for three / four 8-warp
                            blocks per SM (80 registers) instead of 122
  stage_max                 largest fixed set staged in shared memory (ints)
  stage_tma                 stage those sets with bulk copies (cp.async.bulk)
  leaf_batch                batched deepest loop level on/off
  pair_leaf                 pair sums over the last two loops on/off
  bitmap_min                smallest fixed leaf set tested through a bitmap
                            (the bitmap-vs-search threshold by set size)
  split                     shortest loop (depth >= 2) shared with idle warps
  merge_alpha4_{small,mid,large}
                            merge vs binary-search weight for lists shorter
                            than 256, 8192, and longer (degree buckets)
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import statistics
import time
from pathlib import Path

from . import native
from .native import U128, check, lib

SPACE = {
    "chunk": [1, 2, 4, 8, 16, 32],
    "warps_per_block": [4, 8, 16],
    "blocks_per_sm": [1, 2, 3],
    "min_blocks": [1, 3, 4],
    "merge_vec": [0, 1],
    "stage_max": [0, 256, 1024, 2048],
    "stage_tma": [0, 1],
    "leaf_batch": [0, 1],
    "pair_leaf": [0, 1],
    "bitmap_min": [0, 1024, 4096, 16384],
    "split": [0, 16, 64, 256],
    "merge_alpha4_small": [0, 2, 4, 8, 32],
    "merge_alpha4_mid": [0, 2, 4, 8, 32],
    "merge_alpha4_large": [0, 2, 4, 8, 32],
}


def current() -> dict:
    return {k: native.get_option(k) for k in SPACE}


def apply(table: dict) -> None:
    for k, v in table.items():
        if k in SPACE:
            native.set_option(k, int(v))


def signature(graph, schedules) -> str:
    h = hashlib.sha256()
    h.update(f"{graph.v_cnt}:{graph.e_cnt}:{graph.max_degree}".encode())
    for s in schedules:
        h.update(bytes(memoryview(s.tables)))
    return h.hexdigest()[:16]


def save(table: dict, path: str | Path, key: str) -> None:
    p = Path(path)
    data = json.loads(p.read_text()) if p.exists() else {}
    data[key] = table
    p.write_text(json.dumps(data, indent=1, sort_keys=True))


def load(path: str | Path, key: str) -> dict | None:
    p = Path(path)
    if not p.exists():
        return None
    return json.loads(p.read_text()).get(key)


class _Trial:
    """Times one batched launch over the sample stripes."""

    def __init__(self, graph, plans, stripes: int, sample: list[int]):
        self.n = len(plans)
        self.gh = (C.c_void_p * self.n)(*([graph.device()] * self.n))
        self.ph = (C.c_void_p * self.n)(*[p.handle for p in plans])
        self.stripes = stripes
        self.sample = sample

    def run(self) -> tuple[float, list[int]]:
        native.set_option("raw_sums", 1)
        native.set_option("stripes", self.stripes)
        ms, sums = 0.0, [0] * self.n
        try:
            for st in self.sample:
                native.set_option("stripe", st)
                outs = (U128 * self.n)()
                check(lib().gpm_batch_count(self.n, self.gh, self.ph, outs), "gpm_batch_count")
                ms += native.last_launch_stats()[0]
                sums = [a + o.value for a, o in zip(sums, outs)]
        finally:
            native.set_option("stripes", 1)
            native.set_option("stripe", 0)
            native.set_option("raw_sums", 0)
        return ms, sums


def autotune(graph, schedules, stripes: int = 1024, sample_stripes: int = 2, repeats: int = 2,
             budget_s: float = 90.0, space: dict | None = None, verbose: bool = False,
             sample: list[int] | None = None) -> dict:
    """Returns the fastest knob table found (and leaves it applied).  The
    sample is `sample` (stripe ids of `stripes`), else sample_stripes evenly
    spaced stripes."""
    from .api import Plan
    space = space or SPACE
    plans = [Plan(s) for s in schedules]
    if sample is None:
        step = max(1, stripes // max(1, sample_stripes))
        sample = [i * step + step // 2 for i in range(sample_stripes)]
    trial = _Trial(graph, plans, stripes, list(sample))
    t_start = time.time()
    best = current()
    apply(best)
    trial.run()  # warm caches / scratch
    base_sums = None

    def measure() -> float:
        nonlocal base_sums
        times = []
        for _ in range(repeats):
            ms, sums = trial.run()
            if base_sums is None:
                base_sums = sums
            elif sums != base_sums:
                raise AssertionError("autotune: counts changed with engine knobs")
            times.append(ms)
        return statistics.median(times)

    best_ms = measure()
    history = [(dict(best), best_ms)]
    try:
        for _sweep in range(2):
            improved = False
            for knob, values in space.items():
                for v in values:
                    if v == best[knob] or time.time() - t_start > budget_s:
                        continue
                    cand = dict(best)
                    cand[knob] = v
                    apply(cand)
                    try:
                        ms = measure()
                    except native.GpmError as e:  # a shape this device cannot launch
                        if verbose:
                            print(f"[autotune] {knob}={v}: skipped ({e})", flush=True)
                        continue
                    history.append((cand, ms))
                    if verbose:
                        print(f"[autotune] {knob}={v}: {ms:.2f} ms (best {best_ms:.2f})", flush=True)
                    if ms < best_ms * 0.98:
                        best, best_ms, improved = cand, ms, True
                apply(best)
            if not improved:
                break
    finally:
        apply(best)
        for p in plans:
            p.close()
    best = dict(best)
    best["_ms"] = best_ms
    best["_trials"] = len(history)
    best["_default_ms"] = history[0][1]
    return best


TUNED = Path(__file__).resolve().parent / "tuned" / "tables.json"


def apply_stored(graph, schedules, path: str | Path = TUNED) -> dict | None:
    """Installs the table tuned for this graph and pattern set, if one is
    stored; returns it (None when there is none)."""
    table = load(path, signature(graph, schedules))
    if table:
        apply({k: v for k, v in table.items() if not k.startswith("_")})
    return table


def main(argv: list[str] | None = None) -> dict:
    """Tunes the knobs for the 29 motifs (3-5 vertices) on an R-MAT graph and
    stores the table under its signature.

        python -m graphpi_gb300.autotune --scale 22 --out graphpi_gb300/tuned/tables.json
    """
    import argparse

    from . import workloads
    from .api import Schedule, motifs_3_to_5

    ap = argparse.ArgumentParser()
    ap.add_argument("--scale", type=int, default=22)
    ap.add_argument("--seed", type=int, default=3)
    ap.add_argument("--stripes", type=int, default=1 << 23, help="the sample is a few of this many stripes")
    ap.add_argument("--samples", type=int, default=8)
    ap.add_argument("--skip", type=int, default=48,
                    help="the sample is drawn from the seeded random stripe ids after the first SKIP (the "
                         "benchmark's timed and warm-up steps use the first ones)")
    ap.add_argument("--budget", type=float, default=120.0, help="seconds")
    ap.add_argument("--out", default=str(TUNED))
    a = ap.parse_args(argv)
    g = workloads.rmat_s22() if (a.scale, a.seed) == (22, 3) else workloads.rmat_scale(a.scale, a.seed)
    tri = g.triangle_counting_mt()
    scheds = [Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, tri) for p in motifs_3_to_5()]
    sample = workloads.random_stripes(a.stripes, a.skip + a.samples)[a.skip:]
    table = autotune(g, scheds, stripes=a.stripes, sample=sample, repeats=1, budget_s=a.budget, verbose=True)
    table["_graph"] = f"rmat s{a.scale} seed {a.seed}"
    table["_sample"] = f"random stripes {sample} of {a.stripes}"
    Path(a.out).parent.mkdir(parents=True, exist_ok=True)
    save(table, a.out, signature(g, scheds))
    print(json.dumps(table, indent=1, sort_keys=True))
    return table


if __name__ == "__main__":
    main()
