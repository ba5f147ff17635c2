"""Kernels of compact support and the spheroidal family on the tree backend: cub and sph run
near-field-only trees whose leaves are at least as wide as the support (the radius search of
src/fmm/direct_evaluator.hpp:41-68), and sp3-sp9 are split into a compact direct part and a
smooth fast part evaluated by the FMM (src/fmm/spheroidal_evaluator.hpp:8-62). Checked against
the oracle's exact sums, and through fits whose residual the oracle recomputes."""
import numpy as np
import pytest

import oracle
import polatory_gb300 as pg

pytestmark = pytest.mark.gpu

KINDS = {"cub": pg.CovCubic, "sph": pg.CovSpherical, "sp3": pg.CovSpheroidal3,
         "sp5": pg.CovSpheroidal5, "sp7": pg.CovSpheroidal7, "sp9": pg.CovSpheroidal9}


@pytest.mark.parametrize("precision", [pg.PLAIN, pg.MIXED], ids=["plain", "mixed"])
@pytest.mark.parametrize("name", list(KINDS))
def test_tree_backend_matches_exact_sums(name, precision):
    g = np.random.Generator(np.random.PCG64(71))
    src = g.random((40_000, 3))
    trg = g.random((12_000, 3))
    w = g.standard_normal(40_000)
    rbf = KINDS[name]([1.0, 0.15])
    rbf.anisotropy = np.array([[1.0, 0.1, 0.0], [0.0, 1.2, 0.0], [0.0, 0.0, 0.8]])
    ev = pg.FmmEvaluator(rbf, [0, 0, 0, 1, 1, 1], precision=precision)
    ev.configure(backend=2)
    ev.set_source_points(src)
    ev.set_target_points(trg)
    ev.set_weights(w)
    got = ev.evaluate()
    m = pg.Model(rbf, -1)._c()
    want = oracle.direct_evaluate(m, src, w, trg)
    scale = np.abs(w).sum() * 1e-3 + np.max(np.abs(want))
    compact = name in ("cub", "sph")
    # cub/sph: exact sums (FP64, or FP32 rounding). Spheroidal: the fast part's far field at the
    # default accuracy (order 6) is off by ~1e-5 of the scale at this range.
    if compact:
        bound = 1e-12 if precision == pg.PLAIN else 1e-5
    else:
        bound = 1e-4
    assert np.max(np.abs(got - want)) <= bound * scale, (np.max(np.abs(got - want)), scale)
    if not compact:
        # A finite accuracy: the estimator's order (or exact sums) meets it.
        acc = 1e-7 * scale
        ev2 = pg.FmmEvaluator(rbf, [0, 0, 0, 1, 1, 1], precision=precision)
        ev2.configure(backend=2)
        ev2.set_accuracy(acc)
        ev2.set_source_points(src)
        ev2.set_target_points(trg)
        ev2.set_weights(w)
        assert np.max(np.abs(ev2.evaluate() - want)) <= 2 * acc


@pytest.mark.parametrize("name,range_", [("cub", 0.2), ("sp3", 0.3)])
def test_compact_fit_200k(name, range_):
    # 200,000 points: the tree backend serves the operator, the preconditioner's residual
    # updates and the evaluation; the residual at sampled data points is recomputed exactly.
    g = np.random.Generator(np.random.PCG64(72))
    pts = g.random((200_000, 3))
    vals = np.sin(4 * pts[:, 0]) + pts[:, 1] * pts[:, 2]
    model = pg.Model(KINDS[name]([1.0, range_]), 0)
    model.nugget = 1e-3
    tol = 1e-4
    it = pg.Interpolant(model)
    it.fit(pts, vals, tol)
    w = it.weights
    idx = g.choice(pts.shape[0], 2000, replace=False)
    fit_vals = oracle.direct_evaluate(model, pts, w, pts[idx]) + model.nugget * w[idx]
    assert np.max(np.abs(fit_vals - vals[idx])) <= tol
    q = g.random((3000, 3))
    want = oracle.direct_evaluate(model, pts, w, q)
    assert np.max(np.abs(it.evaluate(q, accuracy=1e-7) - want)) <= 2e-7
