"""Learned schedule cost model: the MLP kernels against a numpy restatement
(forward, mean-squared-error gradients), training, and the learned choice
of loop order (exact counts, runtime against the analytic model)."""
import ctypes as C

import numpy as np
import pytest

import graphpi_gb300 as gp
from graphpi_gb300 import learned
from graphpi_gb300.native import check, lib


def np_forward(p, X, H):
    D = X.shape[1]
    W1 = p[:H * D].reshape(H, D)
    b1 = p[H * D:H * D + H]
    W2 = p[H * D + H:H * D + 2 * H]
    b2 = p[-1]
    A = X @ W1.T + b1
    Hh = np.maximum(A, 0)
    return Hh @ W2 + b2, Hh, A


def np_grads(p, X, T, H):
    N, D = X.shape
    Y, Hh, A = np_forward(p, X, H)
    W2 = p[H * D + H:H * D + 2 * H]
    dy = 2 * (Y - T) / N
    gW2 = Hh.T @ dy
    gb2 = dy.sum()
    dH = np.outer(dy, W2) * (A > 0)
    gW1 = dH.T @ X
    gb1 = dH.sum(axis=0)
    return np.concatenate([gW1.reshape(-1), gb1, gW2, [gb2]]), np.mean((Y - T) ** 2)


def test_feature_vector_shape(engine):
    s = gp.Schedule(gp.Pattern(gp.PatternType.House), 1, 1, True, 1000, 8000, 500)
    f = learned.schedule_features(s, {"v_cnt": 1000, "e_cnt": 8000, "tri_cnt": 500, "max_degree": 40}, 1e6)
    assert f.shape == (learned.N_FEATURES,) and np.all(np.isfinite(f))


@pytest.mark.gpu
def test_mlp_forward_and_gradients_match_cpu(engine):
    rng = np.random.default_rng(0)
    m = learned.CostModel(hidden=64, seed=3)
    p = m.params().astype(np.float64)
    X = rng.normal(size=(300, learned.N_FEATURES)).astype(np.float32)
    T = rng.normal(size=300).astype(np.float32)
    y = np.zeros(300, dtype=np.float32)
    check(lib().gpm_mlp_forward(m.h, X.ctypes.data, 300, y.ctypes.data), "forward")
    want, _, _ = np_forward(p, X.astype(np.float64), 64)
    np.testing.assert_allclose(y, want, rtol=1e-4, atol=1e-4)
    g = np.zeros(m.n_params, dtype=np.float32)
    loss = C.c_float()
    check(lib().gpm_mlp_gradients(m.h, X.ctypes.data, T.ctypes.data, 300, g.ctypes.data, C.byref(loss)), "grad")
    gw, lw = np_grads(p, X.astype(np.float64), T.astype(np.float64), 64)
    np.testing.assert_allclose(g, gw, rtol=1e-3, atol=1e-5)
    assert abs(loss.value - lw) <= 1e-4 * max(1.0, lw)
    m.close()


@pytest.mark.gpu
def test_mlp_training_fits_a_smooth_target(engine):
    rng = np.random.default_rng(1)
    X = rng.normal(size=(800, learned.N_FEATURES)).astype(np.float32)
    T = (np.sin(X[:, 0]) + 0.5 * X[:, 1] * X[:, 2] + 0.1 * X[:, 3]).astype(np.float32)
    m = learned.CostModel(hidden=64, seed=5)
    loss0 = C.c_float()
    g = np.zeros(m.n_params, dtype=np.float32)
    check(lib().gpm_mlp_gradients(m.h, X.ctypes.data, T.ctypes.data, 800, g.ctypes.data, C.byref(loss0)), "grad")
    fl = C.c_float()
    check(lib().gpm_mlp_train(m.h, X.ctypes.data, T.ctypes.data, 800, 1500, 3e-3, 0.0, C.byref(fl)), "train")
    assert fl.value < 0.2 * loss0.value
    m.close()


@pytest.mark.gpu
def test_learned_choice_exact_and_reported(engine, oracle):
    g = gp.rmat(12, 8, 0.57, 0.19, 0.19, 6)
    pats = gp.MotifGenerator(5).generate()
    train, held = pats[::2], pats[1::2]
    rows = learned.collect(g, train, max_candidates=12)
    model = learned.CostModel(hidden=64, seed=2)
    model.fit(rows, epochs=2000)
    test_rows = learned.collect(g, held, max_candidates=12)
    ev = learned.evaluate(test_rows, model)
    print(f"learned vs best {ev['mlp_over_best']:.3f}, judged {ev['judged_over_best']:.3f}, "
          f"analytic vs best {ev['analytic_over_best']:.3f}")
    assert ev["mlp_over_best"] >= 1.0 and ev["analytic_over_best"] >= 1.0
    # measured runtime judges the model's shortlist, which holds the analytic choice
    assert ev["judged_over_best"] <= ev["analytic_over_best"] + 1e-9
    assert ev["rerank_over_best"] >= 1.0
    # whatever is chosen counts exactly
    tri = g.triangle_counting_mt()
    for p in held[:4]:
        s_mlp, _ = learned.choose(p, g, model)
        s_rr, _ = learned.choose(p, g, model, shortlist=4)
        assert g.pattern_matching(s_rr) == oracle.count(g, s_rr)
        s_jdg, info = learned.choose(p, g, model, judge=2)
        assert info["analytic_index"] in info["timed_ms"]
        s_ref = gp.Schedule(p, 1, 1, True, g.v_cnt, g.e_cnt, tri)
        want = oracle.count(g, s_ref)
        assert g.pattern_matching(s_mlp) == g.pattern_matching(s_jdg) == g.pattern_matching(s_ref) == want
    model.close()


@pytest.mark.gpu
def test_network_ranks_held_out_candidates(engine):
    """Trained on the exact work (algorithmic bytes, deterministic) of the
    candidates of half the 5- and 6-vertex motifs on one graph, the model
    (analytic prior + learned correction) ranks the candidates of the other
    half on another graph.  Its rank correlation with the measured work is
    compared with the analytic model's alone, and the work of its picks with
    the analytic picks' (both reported); the learned correction must not
    make the ranking worse than the prior by more than noise."""
    pats = gp.MotifGenerator(5).generate() + gp.MotifGenerator(6).generate()[::8]
    train, held = pats[::2], pats[1::2]
    g_tr = gp.rmat(11, 8, 0.57, 0.19, 0.19, 2)
    g_ev = gp.rmat(12, 8, 0.57, 0.19, 0.19, 4)
    rows_tr = learned.collect(g_tr, train, max_candidates=12, label="work")
    rows_ev = learned.collect(g_ev, held, max_candidates=12, label="work")
    model = learned.CostModel(hidden=64, seed=3)
    model.fit(rows_tr, epochs=2000, weight_decay=1e-3)

    def rank(x):
        return np.argsort(np.argsort(np.asarray(x, dtype=np.float64))).astype(float)

    rho_model, rho_prior = [], []
    for pi in sorted({r["pattern"] for r in rows_ev}):
        rs = [r for r in rows_ev if r["pattern"] == pi]
        if len(rs) < 3 or len({r["y"] for r in rs}) < 2 or len({r["cost"] for r in rs}) < 2:
            continue
        feats = np.stack([r["features"] for r in rs])
        y = rank([r["y"] for r in rs])
        rho_model.append(float(np.corrcoef(rank(model.predict(feats)), y)[0, 1]))
        rho_prior.append(float(np.corrcoef(rank(feats[:, 26]), y)[0, 1]))
    ev = learned.evaluate(rows_ev, model, judge=3, shortlist=4)
    print(f"held-out rank correlation: model {np.mean(rho_model):.3f}, analytic {np.mean(rho_prior):.3f} over "
          f"{len(rho_model)} patterns; work over best: model {ev['mlp_over_best']:.3f}, re-ranked shortlist "
          f"{ev['rerank_over_best']:.3f}, analytic {ev['analytic_over_best']:.3f}")
    # measured: model 0.27 against analytic 0.29; picks 1.33 against 1.04 x best
    assert rho_model and np.mean(rho_model) >= np.mean(rho_prior) - 0.1
    assert ev["mlp_over_best"] <= 1.5 * ev["analytic_over_best"]
    model.close()


@pytest.mark.gpu
def test_learned_rerank_beats_analytic_choice_on_runtime(engine):
    """Trained on runtimes the enumerator measures on R-MAT s15 (every other
    5-vertex and a sample of 6-vertex motifs), the network re-ranks the
    analytic model's four cheapest candidates of the held-out motifs on
    R-MAT s17: the picks' summed runtime is no worse than the analytic
    choices' (measured 1.20 and 1.52 against 1.70 and 1.68 x the best
    candidates' in two runs), and timing the network's three best plus the
    analytic choice comes close to the best (1.08, 1.09 x best)."""
    from graphpi_gb300 import workloads
    pats = gp.MotifGenerator(5).generate() + gp.MotifGenerator(6).generate()[::8]
    train, held = pats[::2], pats[1::2]
    rows_tr = learned.collect(workloads.rmat_scale(15, 2), train, max_candidates=8)
    rows_ev = learned.collect(workloads.rmat_scale(17, 4), held, max_candidates=8)
    model = learned.CostModel(hidden=64, seed=1)
    model.fit(rows_tr, epochs=3000)
    ev = learned.evaluate(rows_ev, model, judge=3, shortlist=4)
    print(f"runtime over best: re-ranked {ev['rerank_over_best']:.3f}, timed shortlist "
          f"{ev['judged_over_best']:.3f}, analytic {ev['analytic_over_best']:.3f}, network alone "
          f"{ev['mlp_over_best']:.3f}")
    assert ev["rerank_over_best"] <= ev["analytic_over_best"]
    assert ev["judged_over_best"] <= 1.15  # the 10 % target, with room for timing noise
    model.close()
