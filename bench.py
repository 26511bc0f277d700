"""Benchmark: batched counting of all 29 connected 3-5-vertex motifs on the
R-MAT scale-22 graph (4,194,304 vertices, edge factor 16,
a/b/c/d = .57/.19/.19/.05, seed 3), one persistent launch per step.

A step is one stripe of the job's first-level tasks (the directed edges
(v0, v1) of the degree-relabelled CSR, or root vertices for plans whose
inclusion-exclusion tail starts at depth 1): the tasks t with t mod S = s,
S = 2^23 stripes in all (about 15 tasks per motif per step), counted for all
29 motifs in one launch.  The stripe ids are drawn uniformly at random from
a seeded stream (workloads.random_stripes): the timed steps take ids[0..K),
the warm-up steps ids[K..K+W).  A uniformly random stripe is an unbiased
sample of the whole job, so embeddings/s over the steps estimates the whole
job's throughput.  The graph (0.5 GB of CSR, larger than the 129 MB L2)
stays resident in HBM.

Schedules: the engine's Schedule (perf=1, restricts=1, IEP on) for the
graph's v/e/tri counts; the bench checks that its tables equal the
reference's own, recorded with the undivided sums of the reference itself
over the first 48 stripe ids in tests/golden/bench_stripes.json.  Every
timed stripe's raw sums are compared with those recorded sums, bit for bit.

Reported on one JSON line (rank 0):
  value      embeddings/s over the timed steps, inputs resident in HBM
             (one CUDA-graph replay of the batched launch per step)
  e2e        the same through gpm_count_host with pinned host buffers: upload,
             device relabel, count, download, free inside every step
  plain      the same stripes counted one pattern per launch (29 launches)
  roofline   algorithmic bytes of the intersections per launch / kernel time
             against the measured HBM copy bandwidth; DRAM bytes per launch
             from a committed ncu capture beside it
  cpu_baseline  the CPU oracle (a restatement of the reference's OpenMP
             pattern_matching, split into the same first-level tasks) on the
             first timed stripes, all host cores, sums checked equal

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--config c3|c2]

--config c2: rectangle and house on R-MAT scale 20 (seed 2), one pattern
per launch, a step = one random stripe of 2^16.
--impl reference: the reference's CPU path (the oracle port, no GPU, without
the engine library in the process) on exactly the same stripes.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "embeddings/s, batched 5-motif R-MAT s22 vs per-pattern GPU; HBM % peak; p50"
HBM_FALLBACK_GBS = 6800.0
GOLDEN = ROOT / "tests" / "golden" / "bench_stripes.json"

CONFIGS = {
    "c3": dict(scale=22, seed=3, golden="rmat_s22", stripes=1 << 23, batched=True,
               workload="rmat_s22 x 29 motifs (3-5 vertices), batched persistent launch"),
    "c2": dict(scale=20, seed=2, golden="rmat_s20", stripes=1 << 16, batched=False,
               workload="rmat_s20 x {rectangle, house}, one pattern per launch"),
}


def _peak_hbm() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return HBM_FALLBACK_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows: list[list[str]] = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                for line in out.stdout.strip().splitlines():
                    self.rows.append([x.strip() for x in line.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=6)

    def summary(self) -> dict:
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i - 5] for r in self.rows for i in range(5, 9)
                          if len(r) > i and r[i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def _signed(v: int) -> int:
    return v - (1 << 128) if v >= (1 << 127) else v


def load_golden(cfg: dict, g0=None) -> dict | None:
    """The reference's recorded tables and stripe sums for this graph (None
    when absent or recorded for another graph)."""
    if not GOLDEN.exists():
        return None
    e = json.loads(GOLDEN.read_text()).get(cfg["golden"])
    if e is None:
        return None
    if g0 is not None:
        from tests.oracle_lib import csr_checksum
        if csr_checksum(g0) != e["checksum"]:
            raise AssertionError("the generated graph differs from the one the reference sums were recorded on")
    return e


def step_ids(args, S: int) -> tuple[list[int], list[int]]:
    from graphpi_gb300 import workloads
    ids = workloads.random_stripes(S, args.steps + args.warmup)
    return ids[:args.steps], ids[args.steps:]


def bench_config(args, cfg: dict, S: int) -> dict:
    """The workload description both arms print (identical by construction)."""
    return {
        "workload": cfg["workload"],
        "graph": f"R-MAT scale {cfg['scale']}, edge factor 16, (.57,.19,.19,.05), seed {cfg['seed']}, "
                 "symmetrised, deduplicated, relabelled by degree",
        "schedule": "perf=1, restricts=1, IEP on (tables equal to the reference's Schedule)",
        "stripes": S,
        "step": f"one seeded random stripe = 1/{S} of the first-level tasks "
                f"(workloads.random_stripes: timed ids[0..{args.steps}), warm-up ids[{args.steps}..{args.steps + args.warmup}))",
        "l2": "inputs larger than L2 (CSR of the graph vs 129 MB)",
    }


def check_against_golden(golden, ids: list[int], raws_by_step: list[list[int]]) -> int:
    """Compares raw stripe sums with the reference's recorded ones (mod 2^64,
    the reference's long long); returns how many stripes were checked."""
    if golden is None:
        return 0
    pos = {s: j for j, s in enumerate(golden["ids"])}
    checked = 0
    for s, raws in zip(ids, raws_by_step):
        j = pos.get(s)
        if j is None:
            continue
        for i, r in enumerate(raws):
            want = golden["raw"][i][j]
            if (r - want) % (1 << 64) != 0:
                raise AssertionError(f"stripe {s}, pattern {golden['names'][i]}: raw sum {r} != reference {want}")
        checked += 1
    return checked


def patterns_for(gp, cfg: dict):
    if cfg["batched"]:
        return gp.motifs_3_to_5()
    return [gp.Pattern(gp.PatternType.Rectangle), gp.Pattern(gp.PatternType.House)]


def run_ours(args, rank: int, world: int) -> dict | None:
    import torch
    import graphpi_gb300 as gp
    from graphpi_gb300 import native, workloads

    cfg = CONFIGS[args.config]
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    native.check(gp.lib().gpm_set_device(dev), "gpm_set_device")
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    free0 = torch.cuda.mem_get_info(dev)[0]
    t = time.time()
    g = workloads.rmat_scale(cfg["scale"], cfg["seed"])
    gen_s = time.time() - t
    golden = load_golden(cfg, g)
    t = time.time()
    g.device()
    upload_s = time.time() - t
    tri = g.triangle_counting_mt()
    pats = patterns_for(gp, cfg)
    scheds = [gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, tri) for p in pats]
    tables_equal = None
    if golden is not None:
        if tri != golden["tri_cnt"]:
            raise AssertionError(f"GPU triangle count {tri} != reference {golden['tri_cnt']}")
        tables_equal = all([int(x) for x in s.tables] == want for s, want in zip(scheds, golden["tables"]))
        if not tables_equal:
            raise AssertionError("engine schedule tables differ from the reference's")
    red = [s.get_in_exclusion_optimize_redundancy() for s in scheds]
    n = len(scheds)
    from graphpi_gb300 import autotune
    tuned = autotune.apply_stored(g, scheds) if not args.no_tuning else None
    forced = {}
    for kv in args.set:
        k, v = kv.split("=", 1)
        gp.set_option(k, int(v))
        forced[k] = int(v)
    S = args.stripes or cfg["stripes"]
    timed_ids, warm_ids = step_ids(args, S)
    # rank r takes every world-th step of the sequence
    timed_ids = timed_ids[rank::world]
    gp.set_option("raw_sums", 1)
    gp.set_option("stripes", S)
    gp.set_option("pair_log2", args.pair_log2)
    if args.leaf_batch is not None:
        gp.set_option("leaf_batch", args.leaf_batch)
    if args.pair_max_ops is not None:
        gp.set_option("pair_max_ops", args.pair_max_ops)
    plans = [gp.Plan(s) for s in scheds]
    gh = (C.c_void_p * n)(*([g.device()] * n))
    ph = (C.c_void_p * n)(*[p.handle for p in plans])

    exec_h = C.c_void_p()

    def batched(stripe: int) -> list[int]:
        gp.set_option("stripe", stripe)
        outs = (native.U128 * n)()
        native.check(gp.lib().gpm_batch_exec_run(C.byref(exec_h), n, gh, ph, outs), "gpm_batch_exec_run")
        return [_signed(o.value) for o in outs]

    def per_pattern(stripe: int) -> tuple[list[int], list[float]]:
        gp.set_option("stripe", stripe)
        raws, ms = [], []
        for p in plans:
            o = native.U128()
            native.check(gp.lib().gpm_count(g.device(), p.handle, C.byref(o)), "gpm_count")
            raws.append(_signed(o.value))
            ms.append(gp.last_launch_stats()[0])
        return raws, ms

    def embeddings(raws) -> float:
        return sum(r / d for r, d in zip(raws, red))

    step = batched if cfg["batched"] else (lambda s: per_pattern(s)[0])
    print(f"[bench] {cfg['workload']}: stripes={S}, timed ids {timed_ids[:4]}...", file=sys.stderr, flush=True)
    for s in warm_ids:
        step(s)
        print(f"[bench] warmup stripe {s}: {gp.last_launch_stats()[0]:.1f} ms", file=sys.stderr, flush=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    # device memory the engine holds for this workload (graph copies, plans,
    # launch scratch), from the free memory before and after the warm-up
    engine_bytes = free0 - torch.cuda.mem_get_info(dev)[0]
    kernel_ms, emb, raws_all = [], 0.0, []
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clocks:
        e0.record()
        for s in timed_ids:
            if cfg["batched"]:
                r = batched(s)
                kernel_ms.append(gp.last_launch_stats()[0])
            else:
                r, ms = per_pattern(s)
                kernel_ms.append(sum(ms))
            raws_all.append(r)
            emb += embeddings(r)
        e1.record()
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    elapsed_ms = e0.elapsed_time(e1)
    if dist:
        tt = torch.tensor([elapsed_ms, emb], device="cuda", dtype=torch.float64)
        mx = tt.clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        dist.all_reduce(tt, op=dist.ReduceOp.SUM)
        elapsed_ms, emb = float(mx[0]), float(tt[1])
    value = emb / (elapsed_ms / 1e3)
    print(f"[bench] timed: {elapsed_ms:.1f} ms for {len(timed_ids)} steps; kernel ms {kernel_ms}",
          file=sys.stderr, flush=True)
    checked = check_against_golden(golden, timed_ids, raws_all)
    # exact 128-bit reduction of the ranks' raw sums (one host-side sum, no
    # data-path collective); with every stripe recorded, it must equal the
    # reference's total over all K stripes
    from graphpi_gb300 import shard
    totals = shard.reduce_raw_sums([sum(r[i] for r in raws_all) for i in range(n)], dist)
    all_ids = step_ids(args, S)[0]
    exact_total_checked = False
    if golden is not None and golden["stripes"] == S and all(s in golden["ids"] for s in all_ids):
        pos = {s: j for j, s in enumerate(golden["ids"])}
        want = [sum(golden["raw"][i][pos[s]] for s in all_ids) for i in range(n)]
        if totals != want:
            raise AssertionError("rank-reduced raw totals differ from the reference's")
        exact_total_checked = True

    # ---- plain: one launch per pattern over the same stripes -------------
    plain_ms, by_pattern = [], [[] for _ in plans]
    if cfg["batched"]:
        for s, want in zip(timed_ids, raws_all):
            raws, ms = per_pattern(s)
            if raws != want:
                raise AssertionError(f"stripe {s}: plain and batched counts differ")
            plain_ms.append(sum(ms))
            for j, m in enumerate(ms):
                by_pattern[j].append(m)
        print(f"[bench] plain: {[round(x, 1) for x in plain_ms]}", file=sys.stderr, flush=True)

    # ---- per-schedule generated kernels, one launch pair per pattern -------
    gen_ms, gen_by_pattern, gen_compile_s = [], [[] for _ in plans], None
    if args.generated:
        from graphpi_gb300 import codegen
        t = time.time()
        gen = codegen.Generated(scheds)
        gen_compile_s = time.time() - t
        # the first few timed stripes only: the generated 5-cycle runs its
        # |A|·|B| loops (about 12 s a stripe), so all K would not fit the run
        for s, want in list(zip(timed_ids, raws_all))[:args.generated_steps]:
            tot = 0.0
            for j in range(n):
                r = gen.raw(g, j, stripes=S, stripe=s)
                if r != want[j]:
                    raise AssertionError(f"stripe {s}, pattern {j}: generated kernel and interpreter differ")
                tot += gen.last_ms
                gen_by_pattern[j].append(gen.last_ms)
            gen_ms.append(tot)
        print(f"[bench] generated: {[round(x, 1) for x in gen_ms]}", file=sys.stderr, flush=True)

    # ---- algorithmic bytes of one launch (separate counting run) ----------
    gp.set_option("count_bytes", 1)
    algo_bytes = 0
    if cfg["batched"]:
        gp.set_option("stripe", timed_ids[0])
        outs = (native.U128 * n)()
        native.check(gp.lib().gpm_batch_count(n, gh, ph, outs), "gpm_batch_count")
        algo_bytes = gp.last_launch_stats()[2]
    else:
        gp.set_option("stripe", timed_ids[0])
        for p in plans:
            o = native.U128()
            native.check(gp.lib().gpm_count(g.device(), p.handle, C.byref(o)), "gpm_count")
            algo_bytes += gp.last_launch_stats()[2]
    gp.set_option("count_bytes", 0)
    k0 = kernel_ms[0]
    achieved = algo_bytes / (k0 / 1e3) / 1e9
    peak, peak_kind = _peak_hbm()
    traffic, traffic_src, dram_frac = None, None, None
    cap = ROOT / "profiles" / f"dram_{args.config}.json"
    if cap.exists():
        c = json.loads(cap.read_text())
        if c.get("stripes") == S and c.get("stripe") == timed_ids[0]:
            traffic = c.get("dram_bytes_per_launch")
            traffic_src = c.get("source")
            dram_frac = traffic / (k0 / 1e3) / 1e9 / peak if traffic else None

    # ---- e2e through the host-buffer C ABI ---------------------------------
    vtx = torch.from_numpy(g.vertex.view(np.int32)).pin_memory()
    edg = torch.from_numpy(g.edge).pin_memory()
    tabs = [np.ascontiguousarray(s.tables, dtype=np.int64) for s in scheds]
    flat = np.ascontiguousarray(np.concatenate(tabs))
    nw = np.array([len(t) for t in tabs], dtype=np.int32)
    e2e_emb, e2e_ms = 0.0, 0.0
    h0, h1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for s, want in zip(timed_ids, raws_all):
        gp.set_option("stripe", s)
        outs = (native.U128 * n)()
        torch.cuda.synchronize()
        h0.record()
        native.check(gp.lib().gpm_count_host(g.v_cnt, vtx.data_ptr(), edg.data_ptr(), n, flat.ctypes.data,
                                             nw.ctypes.data, outs), "gpm_count_host")
        h1.record()
        torch.cuda.synchronize()
        e2e_ms += h0.elapsed_time(h1)
        got = [_signed(o.value) for o in outs]
        if got != want:
            raise AssertionError(f"stripe {s}: host-buffer path and resident path differ")
        e2e_emb += embeddings(got)
    gp.lib().gpm_batch_exec_destroy(exec_h)
    gp.set_option("stripes", 1)
    gp.set_option("stripe", 0)
    gp.set_option("raw_sums", 0)

    if rank != 0:
        return None
    cpu = cpu_baseline(g, scheds, red, S, timed_ids, raws_all, budget_s=args.cpu_budget) if args.cpu_budget > 0 else None
    launches = len(timed_ids) * (1 if cfg["batched"] else n)
    res = {
        "metric": METRIC,
        "value": value,
        "unit": "embeddings/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": elapsed_ms / len(timed_ids),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int32 CSR / int128 counts",
        "data": "synthetic (seeded R-MAT generator)",
        "config": bench_config(args, cfg, S),
        "tuning": ({k: v for k, v in tuned.items() if not k.startswith("_ms")} if tuned else "defaults"),
        "options_set": forced or None,
        "path": ("CUDA-graph replay of the batched launch (gpm_batch_exec_run)" if cfg["batched"]
                 else "one gpm_count launch per pattern"),
        "kernel_ms_per_step": statistics.median(kernel_ms),
        "kernel_ms_by_step": [round(x, 2) for x in kernel_ms],
        "embeddings_per_step": emb / len(timed_ids),
        "parity": {"schedule_tables_equal_reference": tables_equal, "tri_cnt_equal_reference": golden is not None,
                   "stripes_checked_against_reference_sums": checked, "of": len(timed_ids),
                   "rank_reduced_totals_equal_reference": exact_total_checked},
        "e2e": {"value": e2e_emb / (e2e_ms / 1e3), "unit": "embeddings/s",
                "h2d_bytes_per_step": int(g.vertex.nbytes + g.edge.nbytes + flat.nbytes),
                "d2h_bytes_per_step": 16 * n, "ms_per_step": e2e_ms / len(timed_ids)},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_src,
                     "dram_frac": dram_frac, "peak_kind": peak_kind, "algo_bytes_per_launch": algo_bytes,
                     "launch_stripe": timed_ids[0]},
        "clocks": clocks.summary(),
        "cpu_baseline": cpu,
        "setup_s": {"generate": round(gen_s, 2), "upload_relabel": round(upload_s, 3)},
        "device_memory_gb": round(engine_bytes / 1e9, 2),
    }
    if gen_ms:
        res["generated"] = {
            "what": "per-schedule generated kernels (graphpi_gb300/codegen.py), one pattern per launch, "
                    f"the first {len(gen_ms)} timed stripes",
            "ms_per_step": statistics.median(gen_ms), "ms_by_motif": [round(sum(m), 2) for m in gen_by_pattern],
            "interpreted_ms_by_motif_same_stripes": [round(sum(m[:len(gen_ms)]), 2) for m in by_pattern],
            "compile_s": round(gen_compile_s, 1),
            "vs_interpreted_one_pattern_per_launch": (statistics.median(plain_ms[:len(gen_ms)]) /
                                                      statistics.median(gen_ms) if plain_ms else None)}
    if cfg["batched"]:
        res["plain_per_pattern_ms_per_step"] = statistics.median(plain_ms)
        res["plain_ms_by_motif"] = [round(sum(m), 2) for m in by_pattern]
        res["batched_speedup_vs_plain"] = statistics.median(plain_ms) / statistics.median(kernel_ms)
        res["batched_speedup_vs_plain_total"] = sum(plain_ms) / sum(kernel_ms)
    return res


def _oracle_graph(g):
    """The degree-relabelled host CSR: the numbering the engine's tasks use."""
    from graphpi_gb300 import api
    return api.relabel_by_degree(g)


def cpu_baseline(g, scheds, red, S: int, ids: list[int], raws_all: list[list[int]], budget_s: float = 20.0) -> dict:
    """The oracle (port of the reference's OpenMP pattern_matching, split into
    the engine's first-level tasks) on the first timed stripes, one stripe at
    a time until about budget_s of host time; sums must equal the GPU's."""
    from tests import oracle_lib
    orc = oracle_lib.load()
    gr = _oracle_graph(g)
    threads = os.cpu_count() or 1
    tabs = [np.ascontiguousarray(s.tables, dtype=np.int64) for s in scheds]
    t0 = time.time()
    emb, used = 0.0, []
    for s, want in zip(ids, raws_all):
        got = [row[0] for row in orc.stripes_raw(gr, tabs, S, [s], threads)]
        if got != want:
            raise AssertionError(f"stripe {s}: CPU oracle and GPU raw sums differ")
        emb += sum(r / d for r, d in zip(got, red))
        used.append(s)
        if time.time() - t0 >= budget_s:
            break
    dt = time.time() - t0
    return {"value": emb / dt, "unit": "embeddings/s", "cores": threads, "kind": "port",
            "sample": f"stripes {used} of {S} (the first timed steps), {len(scheds)} patterns, {dt:.1f} s; "
                      "raw sums equal to the GPU's",
            "seconds": dt}


def run_reference(args, rank: int, world: int) -> dict | None:
    """The reference's CPU path on the host cores, on exactly the stripes the
    GPU arm times.  The reference library is compiled from its sources only
    where they exist, not on the GPU host, so its restatement in
    oracle/oracle.c (same algorithm and task split, 128-bit sums) runs; the
    graph comes from the generator library alone and the schedule tables are
    the reference's own, recorded in tests/golden/bench_stripes.json, so the
    engine library is never loaded in this process."""
    if rank != 0:
        return None
    from graphpi_gb300 import api, workloads
    from tests import oracle_lib

    cfg = CONFIGS[args.config]
    g0 = workloads.rmat_scale(cfg["scale"], cfg["seed"])
    golden = load_golden(cfg, g0)
    if golden is None:
        print(json.dumps({"impl": "reference", "unavailable": "tests/golden/bench_stripes.json has no "
                          f"{cfg['golden']} entry (the reference's schedule tables for this graph)"}))
        return None
    g = api.relabel_by_degree(g0)
    orc = oracle_lib.load()
    tabs = [np.ascontiguousarray(t, dtype=np.int64) for t in golden["tables"]]
    red = [int(t[-2]) for t in golden["tables"]]  # in_exclusion_optimize_redundancy
    S = args.stripes or cfg["stripes"]
    timed_ids, warm_ids = step_ids(args, S)
    threads = os.cpu_count() or 1
    # warm-up: the same code on a 1/256 part of each warm-up stripe
    for s in warm_ids:
        orc.stripes_raw(g, tabs, S * 256, [s], threads)
    t0 = time.time()
    emb, per_step = 0.0, []
    raws_all = []
    for s in timed_ids:
        ts = time.time()
        got = [row[0] for row in orc.stripes_raw(g, tabs, S, [s], threads)]
        per_step.append(time.time() - ts)
        raws_all.append(got)
        emb += sum(r / d for r, d in zip(got, red))
        print(f"[reference] stripe {s}: {per_step[-1]:.2f} s", file=sys.stderr, flush=True)
    dt = time.time() - t0
    checked = check_against_golden(golden if S == golden["stripes"] else None, timed_ids, raws_all)
    value = emb / dt
    return {
        "metric": METRIC, "value": value, "unit": "embeddings/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt * 1e3 / len(timed_ids), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32 CSR / int128 counts",
        "data": "synthetic (seeded R-MAT generator)",
        "config": bench_config(args, cfg, S),
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "embeddings/s", "cores": threads, "kind": "port",
                         "sample": f"the {len(timed_ids)} timed stripes of the GPU arm, every task counted "
                                   f"({dt:.1f} s); schedule tables and sums from the reference itself "
                                   f"(sums checked on {checked} stripes)"},
        "parity": {"stripes_checked_against_reference_sums": checked, "of": len(timed_ids)},
        "seconds_by_step": [round(x, 2) for x in per_step],
        "e2e": {"value": value, "unit": "embeddings/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c3", choices=sorted(CONFIGS))
    ap.add_argument("--stripes", type=int, default=0, help="stripes per full job (0: the config's)")
    ap.add_argument("--scale", type=int, default=0,
                    help="R-MAT scale instead of the config's (small cases for profiling; no recorded sums)")
    ap.add_argument("--no-tuning", action="store_true", help="ignore the stored autotuner table")
    ap.add_argument("--set", action="append", default=[], metavar="KEY=VALUE",
                    help="engine option for this run (gpm_set_option), after the stored table")
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--generated", type=int, default=1, choices=[0, 1],
                    help="also time the per-schedule generated kernels on the same stripes")
    ap.add_argument("--generated-steps", type=int, default=3, help="timed stripes the generated kernels run")
    ap.add_argument("--pair-max-ops", type=int, default=None,
                    help="longest pair sum one warp takes on (default: the engine's)")
    ap.add_argument("--leaf-batch", type=int, default=None, choices=[0, 1],
                    help="force the batched deepest level on or off (default: the engine's)")
    ap.add_argument("--pair-log2", type=int, default=0,
                    help="entries per warp of the pair-sum table as a power of two (0: sized to free memory)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
    if world != args.gpus and "WORLD_SIZE" not in os.environ:
        world = 1
    if args.warmup < 3:
        args.warmup = 3
    if args.scale:
        c = dict(CONFIGS[args.config])
        c.update(scale=args.scale, golden=f"none_s{args.scale}",
                 workload=c["workload"].replace(f"rmat_s{c['scale']}", f"rmat_s{args.scale}"))
        CONFIGS[args.config] = c
    if args.impl == "reference":
        res = run_reference(args, rank, world)
    else:
        import graphpi_gb300  # noqa: F401  (fails loudly when the engine is not built)
        res = run_ours(args, rank, world)
    if rank == 0 and res is not None:
        print(json.dumps(res))


if __name__ == "__main__":
    main()
