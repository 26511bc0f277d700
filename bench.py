"""Benchmark: batched counting of all 29 connected 3-5-vertex motifs on the
R-MAT scale-22 graph (4,194,304 vertices, edge factor 16,
a/b/c/d = .57/.19/.19/.05, seed 3), one persistent launch per step.

A step is one launch over one stripe of the first-level work: the
schedule-driven enumeration of all 29 motifs for the first-level tasks
(root, first neighbour) t with t mod S = s, S stripes in all (the same
interleaved partition that splits the job across GPUs).  S is fixed
(2^23: about 15 edge tasks per motif per step) so that runs compare: the
timed steps take stripes 0..K-1, the warm-up steps the next W.  The whole
job is far beyond a benchmark window, and embeddings/s is dominated by the
hub edges each stripe holds (the first tasks belong to the largest hub).
The graph (0.5 GB of CSR, larger than the 129 MB L2) stays resident in HBM.

Reported on one JSON line (rank 0):
  value      embeddings/s over the timed steps, inputs resident in HBM
  e2e        the same through gpm_count_host with pinned host buffers: upload,
             device relabel, count, download, free inside every step
  plain      the same stripes counted one pattern per launch (29 launches)
  roofline   algorithmic bytes of the intersections per launch / kernel time
             against the measured HBM copy bandwidth
  cpu_baseline  the CPU oracle (a restatement of the reference's OpenMP
             pattern_matching) on a bounded root sample, all host cores

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
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


def build_workload(gp, workloads, scale: int = 22):
    t = time.time()
    g = workloads.rmat_s22() if scale == 22 else workloads.rmat_scale(scale, 3)
    gen_s = time.time() - t
    return g, gen_s


def run_ours(args, rank: int, world: int) -> dict | None:
    import torch
    import graphpi_gb300 as gp
    from graphpi_gb300 import native, workloads

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    native.check(gp.lib().gpm_set_device(dev), "gpm_set_device")
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    g, gen_s = build_workload(gp, workloads, args.scale)
    t = time.time()
    g.device()
    upload_s = time.time() - t
    tri = g.triangle_counting_mt()
    pats = gp.motifs_3_to_5()
    scheds = [gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, tri) for p in pats]
    red = [s.get_in_exclusion_optimize_redundancy() for s in scheds]
    from graphpi_gb300 import autotune
    tuned = autotune.apply_stored(g, scheds) if not args.no_tuning else None
    plans = [gp.Plan(s) for s in scheds]
    n = len(plans)
    gh = (C.c_void_p * n)(*([g.device()] * n))
    ph = (C.c_void_p * n)(*[p.handle for p in plans])
    gp.set_option("raw_sums", 1)
    gp.set_option("pair_log2", args.pair_log2)
    if args.leaf_batch is not None:
        gp.set_option("leaf_batch", args.leaf_batch)
    if args.pair_max_ops is not None:
        gp.set_option("pair_max_ops", args.pair_max_ops)

    def batched(stripe: int) -> list[int]:
        gp.set_option("stripe", stripe)
        outs = (native.U128 * n)()
        native.check(gp.lib().gpm_batch_count(n, gh, ph, outs), "gpm_batch_count")
        return [_signed(o.value) for o in outs]

    def embeddings(raws) -> float:
        return sum(r / d for r, d in zip(raws, red))

    # stripes for this rank: step i takes stripe (i * world + rank) mod S
    def stripe_of(i: int) -> int:
        return (i * world + rank) % S

    if args.stripes == "auto":
        # calibrate from the thinnest stripe (about one task per motif):
        # double the work until a launch takes a quarter of --step-seconds,
        # then extrapolate to a step of about --step-seconds (power of two)
        want = args.step_seconds * 1e3
        S = 1 << 27
        while True:
            gp.set_option("stripes", S)
            batched(S - 1)
            t = max(gp.last_launch_stats()[0], 1e-3)
            print(f"[bench] calibrate: stripes={S} {t:.1f} ms", file=sys.stderr, flush=True)
            if t >= want / 4 or S == 1:
                break
            S //= 2
        while S > 1 and t * 2 <= want:
            S //= 2
            t *= 2
    else:
        S = int(args.stripes)
    gp.set_option("stripes", S)
    print(f"[bench] stripes={S}", file=sys.stderr, flush=True)
    for i in range(args.warmup):
        batched(stripe_of(args.steps + i))
        print(f"[bench] warmup {i}: {gp.last_launch_stats()[0]:.1f} ms", file=sys.stderr, flush=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    kernel_ms, emb, raws_all = [], 0.0, []
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clocks:
        e0.record()
        for i in range(args.steps):
            r = batched(stripe_of(i))
            kernel_ms.append(gp.last_launch_stats()[0])
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

    print(f"[bench] timed: {elapsed_ms:.1f} ms for {args.steps} steps", file=sys.stderr, flush=True)
    # ---- plain: one launch per pattern over the same stripes -------------
    plain_ms, by_motif = [], [[] for _ in plans]
    for i in range(args.steps):
        gp.set_option("stripe", stripe_of(i))
        tot = 0.0
        for j, p in enumerate(plans):
            o = native.U128()
            native.check(gp.lib().gpm_count(g.device(), p.handle, C.byref(o)), "gpm_count")
            ms = gp.last_launch_stats()[0]
            tot += ms
            by_motif[j].append(ms)
            if _signed(o.value) != raws_all[i][j]:
                raise AssertionError(f"plain and batched counts differ for motif {j}")
        plain_ms.append(tot)

    print(f"[bench] plain: {plain_ms}", file=sys.stderr, flush=True)
    # ---- algorithmic bytes of one batched launch (separate counting run) ---
    gp.set_option("count_bytes", 1)
    batched(stripe_of(0))
    _, _, algo_bytes = gp.last_launch_stats()
    gp.set_option("count_bytes", 0)
    k0 = kernel_ms[0]
    achieved = algo_bytes / (k0 / 1e3) / 1e9
    peak, peak_kind = _peak_hbm()
    # DRAM bytes of one batched launch from the committed one-pass ncu capture
    traffic, traffic_src = None, None
    cap = ROOT / "profiles" / "match_kernel_dram.json"
    if args.scale == 22 and cap.exists():
        c = json.loads(cap.read_text())
        traffic = c.get("dram_bytes_per_launch")
        traffic_src = f"ncu capture of stripe {c.get('stripe')} of {c.get('stripes')}, {c.get('knobs')}"


    # ---- e2e through the host-buffer C ABI ---------------------------------
    vtx = torch.from_numpy(g.vertex.view(np.int32)).pin_memory()
    edg = torch.from_numpy(g.edge).pin_memory()
    tabs = [np.ascontiguousarray(s.tables, dtype=np.int64) for s in scheds]
    flat = np.ascontiguousarray(np.concatenate(tabs))
    nw = np.array([len(t) for t in tabs], dtype=np.int32)
    e2e_emb, e2e_ms = 0.0, 0.0
    h0, h1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for i in range(args.steps):
        gp.set_option("stripe", stripe_of(i))
        outs = (native.U128 * n)()
        torch.cuda.synchronize()
        h0.record()
        native.check(gp.lib().gpm_count_host(g.v_cnt, vtx.data_ptr(), edg.data_ptr(), n, flat.ctypes.data,
                                             nw.ctypes.data, outs), "gpm_count_host")
        h1.record()
        torch.cuda.synchronize()
        e2e_ms += h0.elapsed_time(h1)
        e2e_emb += embeddings([_signed(o.value) for o in outs])
    gp.set_option("stripes", 1)
    gp.set_option("stripe", 0)
    gp.set_option("raw_sums", 0)

    if rank != 0:
        return None
    cpu = cpu_baseline(g, scheds, red, budget_s=args.cpu_budget) if args.cpu_budget > 0 else None
    return {
        "metric": METRIC,
        "value": value,
        "unit": "embeddings/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": elapsed_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int32 CSR / int128 counts",
        "data": "synthetic (seeded R-MAT generator)",
        "config": {
            "workload": f"rmat_s{args.scale} x 29 motifs (3-5 vertices), batched persistent launch",
            "graph": {"v_cnt": g.v_cnt, "e_cnt_directed": g.e_cnt,
                      "generator": f"R-MAT scale {args.scale}, ef 16, (.57,.19,.19,.05), seed 3"},
            "schedule": "perf=1, restricts=1, IEP on",
            "stripes": S,
            "tuning": ({k: v for k, v in tuned.items() if not k.startswith("_ms")} if tuned else "defaults"),
            "step": f"one stripe = 1/{S} of the first-level tasks, all 29 motifs",
            "l2": "inputs larger than L2 (0.5 GB CSR vs 129 MB)",
            "gen_s": round(gen_s, 2),
            "upload_relabel_s": round(upload_s, 3),
        },
        "kernel_ms_per_step": statistics.median(kernel_ms),
        "plain_per_pattern_ms_per_step": statistics.median(plain_ms),
        "plain_ms_by_motif": [round(sum(m), 2) for m in by_motif],
        "batched_speedup_vs_plain": statistics.median(plain_ms) / statistics.median(kernel_ms),
        "embeddings_per_step": emb / args.steps,
        "e2e": {"value": e2e_emb / (e2e_ms / 1e3), "unit": "embeddings/s",
                "h2d_bytes_per_step": int(g.vertex.nbytes + g.edge.nbytes + flat.nbytes),
                "d2h_bytes_per_step": 16 * n, "ms_per_step": e2e_ms / args.steps},
        "gpu_launches": args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_src,
                     "peak_kind": peak_kind, "algo_bytes_per_launch": algo_bytes},
        "clocks": clocks.summary(),
        "cpu_baseline": cpu,
    }


def cpu_baseline(g, scheds, red, budget_s: float = 20.0, offset: int = 1, stride: int = 4096) -> dict:
    """Oracle (port of the reference's OpenMP pattern_matching) on a bounded
    root sample: roots offset, offset+stride, ... for every motif."""
    from tests import oracle_lib
    orc = oracle_lib.load()
    roots = np.arange(offset, g.v_cnt, stride, dtype=np.int32)
    threads = os.cpu_count() or 1
    per_motif = budget_s / max(1, len(scheds))
    t0 = time.time()
    emb, done_roots = 0.0, 0
    for s, d in zip(scheds, red):
        raw, done = orc.raw_roots_timed(g, s, roots, per_motif, threads)
        emb += raw / d
        done_roots += done
    dt = time.time() - t0
    return {"value": emb / dt, "unit": "embeddings/s", "cores": threads, "kind": "port",
            "sample": f"roots {offset} mod {stride} ({len(roots)} roots, {done_roots} root-motif runs finished "
                      f"within {per_motif:.2f} s per motif), {len(scheds)} motifs, {dt:.1f} s",
            "seconds": dt}


def run_reference(args, rank: int, world: int) -> dict | None:
    """The reference's CPU path on the host cores.  The reference library is
    compiled from its sources only where they exist; elsewhere its
    restatement in oracle/oracle.c (same algorithm, 128-bit sums) runs."""
    if rank != 0:
        return None
    import graphpi_gb300 as gp
    from graphpi_gb300 import workloads
    g, _ = build_workload(gp, workloads, args.scale)
    from tests import oracle_lib
    orc = oracle_lib.load()
    tri = orc.triangles(g, os.cpu_count() or 1)
    scheds = [gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, tri) for p in gp.motifs_3_to_5()]
    red = [s.get_in_exclusion_optimize_redundancy() for s in scheds]
    per_step = max(2.0, args.cpu_budget / 2)
    for i in range(args.warmup):
        cpu_baseline(g, scheds, red, budget_s=per_step / 4, offset=1 + 7 * (args.steps + i), stride=16384)
    t0 = time.time()
    emb = 0.0
    samples = []
    for i in range(args.steps):
        r = cpu_baseline(g, scheds, red, budget_s=per_step, offset=1 + 7 * i, stride=4096)
        emb += r["value"] * r["seconds"]
        samples.append(r["sample"])
    dt = time.time() - t0
    value = emb / dt
    threads = os.cpu_count() or 1
    return {
        "metric": METRIC, "value": value, "unit": "embeddings/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int64/int128 counts", "data": "synthetic (seeded R-MAT generator)",
        "config": {"workload": f"rmat_s{args.scale} x 29 motifs (3-5 vertices)", "step": "bounded root sample per step"},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "embeddings/s", "cores": threads, "kind": "port",
                         "sample": samples[0]},
        "e2e": {"value": value, "unit": "embeddings/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--stripes", default=os.environ.get("GPM_BENCH_STRIPES", str(1 << 23)),
                    help="stripes per full job (a step is one stripe), or 'auto' to size a step to --step-seconds")
    ap.add_argument("--step-seconds", type=float, default=4.0)
    ap.add_argument("--scale", type=int, default=22, help="R-MAT scale (22 is the benchmark graph)")
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--no-tuning", action="store_true", help="ignore the stored autotuner table")
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
    import graphpi_gb300  # noqa: F401  (fails loudly when the engine is not built)
    res = run_reference(args, rank, world) if args.impl == "reference" else run_ours(args, rank, world)
    if rank == 0 and res is not None:
        print(json.dumps(res))


if __name__ == "__main__":
    main()
