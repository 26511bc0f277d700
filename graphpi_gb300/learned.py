"""Learned schedule choice.

GraphPi's Schedule picks a loop order and restriction set by minimising an
analytic cost (reference src/schedule.cpp:30-139, 1487-1574).  Here a small
MLP (gpm_mlp_*: hand-written forward/backward/Adam kernels) predicts the
log runtime of every candidate instead, trained on runtimes the GPU
enumerator itself measures; the analytic model remains the fallback (no
model, or a pattern size the model was not trained for) and measured
runtime the final arbiter.  Every candidate is an exact schedule, so counts
do not change with the choice.
"""
from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np

from . import native
from .api import Graph, Pattern, Plan, Schedule, schedule_candidates, schedule_from_order
from .native import U128, check, lib

N_FEATURES = 32


def graph_stats(g: Graph) -> dict:
    return {"v_cnt": g.v_cnt, "e_cnt": g.e_cnt, "tri_cnt": g.ensure_tri_cnt(), "max_degree": g.max_degree}


def schedule_features(s: Schedule, stats: dict, analytic_cost: float) -> np.ndarray:
    """Fixed-length description of a schedule on a graph."""
    n = s.size
    adj = s.adj_mat
    f = np.zeros(N_FEATURES, dtype=np.float32)
    for d in range(min(n, 8)):
        f[d] = float(adj[d, :d].sum())  # earlier neighbours of depth d (sets intersected)
    rcount = [0] * 8
    for d in range(n):
        i = s.restrict_last[d]
        while i != -1:
            rcount[d] += 1
            i = s.restrict_next[i]
    f[8:16] = rcount
    k = s.in_exclusion_optimize_num
    f[16] = n
    f[17] = k
    f[18] = (n - k) if k else (n - 1)
    f[19] = s.total_prefix_num
    f[20] = s.total_restrict_num
    f[21] = math.log2(max(1, s.in_exclusion_optimize_redundancy))
    f[22] = math.log2(max(2, stats["v_cnt"]))
    f[23] = math.log2(max(2, stats["e_cnt"]))
    f[24] = math.log2(max(2, stats["tri_cnt"] + 1))
    f[25] = math.log2(max(2, stats["max_degree"]))
    f[26] = math.log10(max(1e-30, analytic_cost))
    # restrictions that bind the deepest levels prune the most work
    f[27] = sum(rcount[max(0, n - 2):n])
    f[28] = sum(1 for d in range(1, n) if s.father_prefix_id[s.loop_set_prefix_id[d]] == -1)
    f[29] = float(s.label_sensitive())
    f[30] = f[26] * f[18]
    f[31] = 1.0
    return f


def _time_schedule(g: Graph, s: Schedule, max_launch_ms: float = 150.0, cap_ms: float = 3.0e6) -> float:
    """Estimated full-run kernel time (ms): one interleaved stripe, sized so
    the launch stays short, scaled up by the stripe count."""
    plan = Plan(s)
    gh = g.device()
    out = U128()

    def run(stripes: int) -> float:
        native.set_option("raw_sums", 1)
        native.set_option("stripes", stripes)
        native.set_option("stripe", stripes // 2)
        try:
            check(lib().gpm_count(gh, plan.handle, C.byref(out)), "gpm_count")
        finally:
            native.set_option("stripes", 1)
            native.set_option("stripe", 0)
            native.set_option("raw_sums", 0)
        return native.last_launch_stats()[0]

    try:
        S = 4096
        t = run(S)
        est = t * S
        if est > cap_ms:
            return est
        while S > 1 and est / (S // 2) <= max_launch_ms:
            S //= 2
        return run(S) * S
    finally:
        plan.close()


def _work_schedule(g: Graph, s: Schedule, stripes: int = 16) -> float:
    """Algorithmic bytes of one stripe of the schedule's job, counted exactly
    by the counting build of the kernel (the int32 elements the reference's
    merges would read).  Loop sharing is off while counting, so the figure
    does not depend on how warps happen to be scheduled: a deterministic
    measure of a candidate's work."""
    plan = Plan(s)
    out = U128()
    old = {k: native.get_option(k) for k in ("count_bytes", "split", "raw_sums", "stripes", "stripe")}
    try:
        native.set_option("count_bytes", 1)
        native.set_option("split", 0)
        native.set_option("raw_sums", 1)
        native.set_option("stripes", stripes)
        native.set_option("stripe", stripes // 2)
        check(lib().gpm_count(g.device(), plan.handle, C.byref(out)), "gpm_count")
        return float(native.last_launch_stats()[2])
    finally:
        for k, v in old.items():
            native.set_option(k, v)
        plan.close()


def relativize(feats: np.ndarray) -> np.ndarray:
    """Features of one pattern's candidates relative to each other: the
    analytic cost terms become differences to the cheapest candidate, so the
    model compares schedules of a pattern rather than graphs."""
    f = np.array(feats, dtype=np.float32, copy=True)
    f[:, 26] -= f[:, 26].min()
    f[:, 30] -= f[:, 30].min()
    return f


def collect(g: Graph, patterns: list[Pattern], max_candidates: int = 32, use_iep: bool = True,
            verbose: bool = False, label: str = "ms") -> list[dict]:
    """Measures candidate schedules of every pattern on g (GPU).  The label
    each row is fitted to ("y") is the estimated kernel time in ms
    (label="ms") or the exact algorithmic bytes of a fixed stripe of the job
    (label="work", deterministic)."""
    stats = graph_stats(g)
    rows = []
    for pi, p in enumerate(patterns):
        cands = schedule_candidates(p, 1, 1, stats["v_cnt"], stats["e_cnt"], stats["tri_cnt"])
        idx = list(range(len(cands)))
        if len(idx) > max_candidates:
            step = len(idx) / max_candidates
            idx = sorted({int(i * step) for i in range(max_candidates)})
            # always include the analytic choice
            best = min(range(len(cands)), key=lambda i: (cands[i]["cost"], i))
            if best not in idx:
                idx[-1] = best
        mine = []
        for i in idx:
            c = cands[i]
            s = schedule_from_order(p, c["order"], c["pairs"], use_iep, 1)
            y = _time_schedule(g, s) if label == "ms" else _work_schedule(g, s)
            mine.append({"pattern": pi, "cand": i, "features": schedule_features(s, stats, c["cost"]),
                         "ms": y if label == "ms" else None, "y": y, "cost": c["cost"], "order": c["order"],
                         "pairs": c["pairs"]})
        rel = relativize(np.stack([r["features"] for r in mine]))
        for r, f in zip(mine, rel):
            r["features"] = f
        rows += mine
        if verbose:
            print(f"[learned] pattern {pi}: {len(idx)} candidates", flush=True)
    return rows


class CostModel:
    """MLP over standardised features that corrects the analytic model.

    Targets are a candidate's measured log10 runtime (or work) relative to the
    other candidates of its pattern; the analytic model's relative log cost
    (feature 26 after `relativize`) is the prior, and the network learns the
    residual.  A prediction is prior + network output, so an untrained or
    strongly regularised network ranks candidates as the analytic model does,
    and what the network adds is the learned correction."""

    def __init__(self, hidden: int = 64, seed: int = 1):
        self.hidden = hidden
        h = C.c_void_p()
        check(lib().gpm_mlp_create(N_FEATURES, hidden, seed, C.byref(h)), "gpm_mlp_create")
        self.h = h
        self.mu = np.zeros(N_FEATURES, dtype=np.float32)
        self.sd = np.ones(N_FEATURES, dtype=np.float32)

    @property
    def n_params(self) -> int:
        return self.hidden * N_FEATURES + 2 * self.hidden + 1

    def _x(self, feats: np.ndarray) -> np.ndarray:
        return np.ascontiguousarray(((feats - self.mu) / self.sd).astype(np.float32))

    def fit(self, rows: list[dict], epochs: int = 3000, lr: float = 3e-3, weight_decay: float = 1e-4) -> float:
        """Targets are log10 runtimes relative to the mean over the same
        pattern's candidates: only the order within a pattern matters."""
        X = np.stack([r["features"] for r in rows]).astype(np.float32)
        logs = np.array([math.log10(max(r["y"], 1e-3)) for r in rows], dtype=np.float64)
        pats = np.array([r["pattern"] for r in rows])
        y = np.zeros(len(rows), dtype=np.float32)
        for p in np.unique(pats):
            m = pats == p
            y[m] = (logs[m] - logs[m].mean()).astype(np.float32)
        prior = X[:, 26].astype(np.float64)
        for p in np.unique(pats):
            m = pats == p
            y[m] -= (prior[m] - prior[m].mean()).astype(np.float32)
        self.mu = X.mean(axis=0)
        self.sd = X.std(axis=0) + 1e-3
        Xs = self._x(X)
        loss = C.c_float()
        check(lib().gpm_mlp_train(self.h, Xs.ctypes.data, y.ctypes.data, len(y), epochs, lr, weight_decay,
                                  C.byref(loss)), "gpm_mlp_train")
        return loss.value

    def predict(self, feats: np.ndarray) -> np.ndarray:
        """Relative log10 runtime (work) of candidates: the analytic prior
        plus the network's correction."""
        f = np.atleast_2d(feats)
        return f[:, 26].astype(np.float32) + self.correction(f)

    def correction(self, feats: np.ndarray) -> np.ndarray:
        """The network's output alone (the learned correction to the prior)."""
        Xs = self._x(np.atleast_2d(feats))
        y = np.zeros(len(Xs), dtype=np.float32)
        check(lib().gpm_mlp_forward(self.h, Xs.ctypes.data, len(Xs), y.ctypes.data), "gpm_mlp_forward")
        return y

    def params(self) -> np.ndarray:
        p = np.zeros(self.n_params, dtype=np.float32)
        check(lib().gpm_mlp_params(self.h, p.ctypes.data, len(p), 0), "gpm_mlp_params")
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        check(lib().gpm_mlp_params(self.h, p.ctypes.data, len(p), 1), "gpm_mlp_params")

    def close(self) -> None:
        if self.h:
            lib().gpm_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def choose(pattern: Pattern, g: Graph, model: CostModel | None, use_iep: bool = True,
           judge: int = 0, shortlist: int = 0) -> tuple[Schedule, dict]:
    """Learned schedule choice (analytic model when model is None).  With
    shortlist=s the model only re-ranks the s analytically cheapest
    candidates.  With judge=k the k candidates the model ranks fastest and
    the analytic choice are timed on a sample of the work and the fastest
    measured one wins."""
    stats = graph_stats(g)
    cands = schedule_candidates(pattern, 1, 1, stats["v_cnt"], stats["e_cnt"], stats["tri_cnt"])
    if model is None:
        i = min(range(len(cands)), key=lambda j: (cands[j]["cost"], j))
        c = cands[i]
        return schedule_from_order(pattern, c["order"], c["pairs"], use_iep, 1), {"index": i, "by": "analytic"}
    scheds = [schedule_from_order(pattern, c["order"], c["pairs"], use_iep, 1) for c in cands]
    feats = relativize(np.stack([schedule_features(s, stats, c["cost"]) for s, c in zip(scheds, cands)]))
    pred = model.predict(feats)
    if shortlist > 0:  # the model re-ranks the analytically cheapest candidates
        keep = sorted(range(len(cands)), key=lambda j: (cands[j]["cost"], j))[:shortlist]
        pred = np.array([pred[j] if j in keep else np.inf for j in range(len(cands))], dtype=np.float64)
    if judge <= 0:
        i = int(np.argmin(pred))
        return scheds[i], {"index": i, "by": "mlp", "pred_rel_log10_ms": float(pred[i])}
    # measured runtime judges the model's top candidates and the analytic choice
    a = min(range(len(cands)), key=lambda j: (cands[j]["cost"], j))
    shortlist = sorted(set([int(j) for j in np.argsort(pred)[:judge]] + [a]))
    timed = {j: _time_schedule(g, scheds[j]) for j in shortlist}
    i = min(timed, key=lambda j: (timed[j], j))
    return scheds[i], {"index": i, "by": "mlp+measured", "timed_ms": timed, "analytic_index": a}


def evaluate(rows: list[dict], model: CostModel, judge: int = 3, shortlist: int = 4) -> dict:
    """Per pattern: measured time of the MLP's pick over all candidates, of
    its pick among the `shortlist` analytically cheapest ("rerank"), of the
    judged pick (the fastest measured among the MLP's top `judge` and the
    analytic choice), of the analytic pick, and of the best candidate."""
    by_pat: dict[int, list[dict]] = {}
    for r in rows:
        by_pat.setdefault(r["pattern"], []).append(r)
    tot = {"mlp": 0.0, "rerank": 0.0, "judged": 0.0, "analytic": 0.0, "best": 0.0}
    per = []
    for pi, rs in sorted(by_pat.items()):
        pred = model.predict(np.stack([r["features"] for r in rs]))
        order = np.argsort(pred)
        m = rs[int(order[0])]["y"]
        by_cost = sorted(range(len(rs)), key=lambda i: (rs[i]["cost"], rs[i]["cand"]))
        a = rs[by_cost[0]]["y"]
        short = by_cost[:shortlist]
        rr = rs[min(short, key=lambda i: (pred[i], i))]["y"]
        j = min([rs[int(i)]["y"] for i in order[:judge]] + [a])
        b = min(r["y"] for r in rs)
        tot["mlp"] += m
        tot["rerank"] += rr
        tot["judged"] += j
        tot["analytic"] += a
        tot["best"] += b
        per.append({"pattern": pi, "mlp_ms": m, "rerank_ms": rr, "judged_ms": j, "analytic_ms": a, "best_ms": b})
    for k in ("mlp", "rerank", "judged", "analytic"):
        tot[f"{k}_over_best"] = tot[k] / max(tot["best"], 1e-9)
    tot["per_pattern"] = per
    return tot


def main(argv: list[str] | None = None) -> dict:
    """Trains the cost model on runtimes measured on one R-MAT graph and
    reports, for held-out patterns on another, the measured runtime of the
    MLP's choice, of the analytic model's choice and of the best candidate.

        python -m graphpi_gb300.learned --train-scale 14 --eval-scale 16
    """
    import argparse
    import json

    from . import workloads
    from .api import MotifGenerator

    ap = argparse.ArgumentParser()
    ap.add_argument("--train-scale", type=int, default=14)
    ap.add_argument("--eval-scale", type=int, default=16)
    ap.add_argument("--six-stride", type=int, default=8, help="every k-th of the 112 six-vertex motifs")
    ap.add_argument("--candidates", type=int, default=12)
    ap.add_argument("--epochs", type=int, default=3000)
    ap.add_argument("--label", default="ms", choices=["ms", "work"],
                    help="fit to measured kernel time or to exact algorithmic bytes of a fixed stripe")
    ap.add_argument("--out", default="")
    a = ap.parse_args(argv)
    t0 = time.time()
    pats = MotifGenerator(5).generate() + MotifGenerator(6).generate()[::a.six_stride]
    train, held = pats[::2], pats[1::2]
    g_tr = workloads.rmat_scale(a.train_scale, 2)
    rows_tr = collect(g_tr, train, max_candidates=a.candidates, label=a.label)
    g_ev = workloads.rmat_scale(a.eval_scale, 4)
    rows_ev = collect(g_ev, held, max_candidates=a.candidates, label=a.label)
    model = CostModel(hidden=64, seed=1)
    loss = model.fit(rows_tr, epochs=a.epochs)
    ev = evaluate(rows_ev, model)
    res = {"label": a.label, "train_graph": f"rmat s{a.train_scale}", "eval_graph": f"rmat s{a.eval_scale}",
           "train_rows": len(rows_tr), "eval_rows": len(rows_ev), "train_loss": loss,
           "mlp_over_best": ev["mlp_over_best"], "rerank_over_best": ev["rerank_over_best"],
           "judged_over_best": ev["judged_over_best"], "analytic_over_best": ev["analytic_over_best"],
           "mlp_ms": ev["mlp"], "rerank_ms": ev["rerank"], "judged_ms": ev["judged"], "analytic_ms": ev["analytic"],
           "best_ms": ev["best"],
           "per_pattern": ev["per_pattern"], "seconds": time.time() - t0}
    model.close()
    text = json.dumps(res, indent=1)
    if a.out:
        with open(a.out, "w") as f:
            f.write(text)
    print(text)
    return res


if __name__ == "__main__":
    main()
