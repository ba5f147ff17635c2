"""GPU fits against the oracle: the fitted weights reproduce the data to the requested absolute
tolerance (interpolation/solver.hpp convergence test; test/interpolation/test_fitter.cpp), the
device evaluation agrees with the oracle's exact sums for the same weights, and the interpolant
agrees with the exact solution of the fit system at query points."""
import numpy as np
import pytest

import oracle
import polatory_gb300 as pg
from polatory_gb300 import workloads

pytestmark = pytest.mark.gpu


def check_fit(interp, model, pts, vals, tol, queries):
    w = interp.weights
    l = model.poly_basis_size
    assert w.shape == (pts.shape[0] + l,)
    # Residual at every data point with exact FP64 sums (oracle).
    fit_vals = oracle.direct_evaluate(model, pts, w, pts) + model.nugget * w[: pts.shape[0]]
    assert np.max(np.abs(fit_vals - vals)) <= tol
    # Device evaluation == oracle evaluation for the same weights.
    got = interp.evaluate(queries)
    want = oracle.direct_evaluate(model, pts, w, queries)
    return got, want


@pytest.mark.parametrize("precision", [pg.PLAIN, pg.MIXED], ids=["plain", "mixed"])
def test_fit_small_biharmonic(precision):
    # Fewer than 2048 points: one RAS level (the coarse solve alone).
    g = np.random.Generator(np.random.PCG64(21))
    pts = g.random((1500, 3))
    vals = workloads.f_c1(pts)
    model = pg.Model(pg.Biharmonic3D([1.0]), 1)
    interp = pg.Interpolant(model, precision)
    tol = 1e-5
    interp.fit(pts, vals, tol)
    q = g.random((700, 3))
    got, want = check_fit(interp, model, pts, vals, tol, q)
    # Below 2^30 source-target pairs the mixed request runs the FP64 path.
    assert np.max(np.abs(got - want)) <= 1e-10
    exact = oracle.fit_exact(model, pts, vals)
    ref = oracle.direct_evaluate(model, pts, exact, q)
    assert np.max(np.abs(got - ref)) <= 1e-3


@pytest.mark.parametrize("precision", [pg.PLAIN, pg.MIXED], ids=["plain", "mixed"])
def test_fit_c1_two_levels(precision):
    # The C1 workload: 10,000 points, biharmonic, degree 1, tol 1e-5 (two RAS levels).
    pts, vals, grid = workloads.c1()
    model = pg.Model(pg.Biharmonic3D([1.0]), 1)
    interp = pg.Interpolant(model, precision)
    tol = 1e-5
    interp.fit(pts, vals, tol)
    stats = interp.fit_stats
    assert stats["levels"] == 2
    assert stats["iterations"] <= 60
    q = grid[::97]
    got, want = check_fit(interp, model, pts, vals, tol, q)
    assert np.max(np.abs(got - want)) <= 1e-9


def test_small_mixed_request_keeps_fp64_sums():
    # Below 2^30 pairs a mixed fit keeps FP64 operator sums and residuals (only its
    # preconditioner is FP32), and its evaluation is FP64.
    pts, vals, grid = workloads.c1()
    model = pg.Model(pg.Biharmonic3D([1.0]), 1)
    b = pg.Interpolant(model, pg.MIXED)
    b.fit(pts, vals, 1e-5)
    w = b.weights
    fit_vals = oracle.direct_evaluate(model, pts, w, pts)
    assert np.max(np.abs(fit_vals - vals)) <= 1e-5
    q = grid[::50]
    assert np.max(np.abs(b.evaluate(q) - oracle.direct_evaluate(model, pts, w, q))) <= 1e-9


@pytest.mark.parametrize("kind", ["biharmonic", "cov_exponential"])
def test_fit_mixed_large(kind):
    # Above 2^30 pairs: FP32 operator and preconditioner, FP64 residuals (iterative refinement).
    g = np.random.Generator(np.random.PCG64(24))
    n = 60000
    pts = g.random((n, 3))
    if kind == "biharmonic":
        vals = workloads.f_c1(pts)
        model = pg.Model(pg.Biharmonic3D([1.0]), 1)
        tol = 1e-5
    else:
        vals = np.sin(4 * pts[:, 0]) + pts[:, 1]
        rbf = pg.CovExponential([1.0, 0.3])
        rbf.anisotropy = np.diag([1.0, 1.0, 2.0])
        model = pg.Model(rbf, 0)
        model.nugget = 1e-3
        tol = 1e-4
    mixed = pg.Interpolant(model, pg.MIXED)
    mixed.fit(pts, vals, tol)
    w = mixed.weights
    fit_vals = oracle.direct_evaluate(model, pts, w, pts) + model.nugget * w[:n]
    assert np.max(np.abs(fit_vals - vals)) <= tol
    q = g.random((40000, 3))  # 2.4e9 pairs: FP32 evaluation
    got = mixed.evaluate(q)
    want = oracle.direct_evaluate(model, pts, w, q)
    assert np.max(np.abs(got - want)) <= 1e-4
    plain = pg.Interpolant(model, pg.PLAIN)
    plain.fit(pts, vals, tol)
    assert np.max(np.abs(plain.evaluate(q) - got)) <= 1e-4


def test_fit_covariance_with_nugget():
    g = np.random.Generator(np.random.PCG64(22))
    pts = g.random((3000, 3))
    vals = np.sin(4 * pts[:, 0]) + pts[:, 1]
    rbf = pg.CovExponential([1.0, 0.5])
    rbf.anisotropy = np.diag([1.0, 1.0, 2.0])
    model = pg.Model(rbf, 0)
    model.nugget = 1e-3
    interp = pg.Interpolant(model)
    tol = 1e-4
    interp.fit(pts, vals, tol)
    q = g.random((500, 3))
    got, want = check_fit(interp, model, pts, vals, tol, q)
    assert np.max(np.abs(got - want)) <= 1e-10


def test_fit_argument_errors():
    model = pg.Model(pg.Biharmonic3D([1.0]), 1)
    interp = pg.Interpolant(model)
    pts = np.random.default_rng(0).random((10, 3))
    with pytest.raises(pg.PolatoryError, match="tolerance must be positive"):
        interp.fit(pts, np.zeros(10), 0.0)
    with pytest.raises(pg.PolatoryError, match="greater than or equal to 4"):
        interp.fit(pts[:3], np.zeros(3), 1e-3)
    with pytest.raises(pg.PolatoryError, match="has not been fitted"):
        interp.evaluate(pts)


def test_max_iter_reached():
    g = np.random.Generator(np.random.PCG64(23))
    pts = g.random((5000, 3))
    vals = workloads.f_c1(pts)
    interp = pg.Interpolant(pg.Model(pg.Biharmonic3D([1.0]), 1))
    with pytest.raises(pg.PolatoryError, match="reached the maximum number of iterations"):
        interp.fit(pts, vals, 1e-12, max_iter=2)


@pytest.mark.parametrize("kind", ["bh3", "exp"])
def test_fit_mixed_fmm_hybrid_residual(kind):
    # 120k points: the FP32 operator runs the FMM and residuals are checked with the hybrid
    # operator (FP32 far field; float-float near field for the polyharmonic kernel, FP64 for the
    # covariance). At tol 1e-5 the biharmonic fit needs the FP64 grade for its last residuals.
    # The exact residual at 4000 sampled data points (oracle) must be within the tolerance.
    g = np.random.Generator(np.random.PCG64(25))
    n = 120000
    pts = g.random((n, 3))
    vals = workloads.f_c1(pts)
    if kind == "bh3":
        model = pg.Model(pg.Biharmonic3D([1.0]), 1)
        tol = 1e-5
    else:
        model = pg.Model(pg.CovExponential([1.0, 0.2]), 0)
        model.nugget = 1e-3
        tol = 1e-4
    it = pg.Interpolant(model, pg.MIXED)
    it.fit(pts, vals, tol)
    w = it.weights
    idx = g.choice(n, 4000, replace=False)
    fit_vals = oracle.direct_evaluate(model, pts, w, pts[idx]) + model.nugget * w[idx]
    assert np.max(np.abs(fit_vals - vals[idx])) <= tol


def test_fit_incrementally():
    # interpolation/incremental_fitter.hpp:46-183: the centres are a subset of the points and
    # every point (centre or not) is within the tolerance, recomputed by the oracle.
    g = np.random.Generator(np.random.PCG64(26))
    pts = g.random((6000, 3))
    vals = 0.2 * workloads.f_c1(pts)
    model = pg.Model(pg.Biharmonic3D([1.0]), 1)
    it = pg.Interpolant(model)
    tol = 1e-3
    it.fit_incrementally(pts, vals, tol)
    c = it.centers
    assert 0 < c.shape[0] <= pts.shape[0]
    rows = {tuple(p) for p in pts}
    assert all(tuple(p) in rows for p in c)
    w = it.weights
    fit_vals = oracle.direct_evaluate(model, c, w, pts)
    assert np.max(np.abs(fit_vals - vals)) <= tol


def test_fit_inequality():
    # interpolation/inequality_fitter.hpp:43-187: equality points are interpolated, bounds hold
    # within the tolerance at every bounded point (recomputed by the oracle).
    g = np.random.Generator(np.random.PCG64(27))
    n = 3000
    pts = g.random((n, 3))
    f = 0.2 * workloads.f_c1(pts)
    nan = np.full(n, np.nan)
    values, lb, ub = nan.copy(), nan.copy(), nan.copy()
    eq = np.arange(0, n, 10)
    values[eq] = f[eq]
    low = np.arange(1, n, 3)
    lb[low] = f[low] - 0.02
    high = np.arange(2, n, 3)
    ub[high] = f[high] + 0.02
    model = pg.Model(pg.Biharmonic3D([1.0]), 1)
    it = pg.Interpolant(model)
    tol = 1e-4
    it.fit_inequality(pts, values, lb, ub, tol)
    c = it.centers
    w = it.weights
    fit = oracle.direct_evaluate(model, c, w, pts)
    assert np.max(np.abs(fit[eq] - values[eq])) <= tol
    assert np.all(fit[low] >= lb[low] - 2 * tol)
    assert np.all(fit[high] <= ub[high] + 2 * tol)


@pytest.mark.parametrize("kind", ["bh3_plain", "bh3_mixed", "cov_aniso"])
def test_device_division_equals_host_division(monkeypatch, kind):
    # The RAS levels divided on the device (domains, inner flags, coarse points) equal the host
    # restatement's, so the fits agree bit for bit. 60k points: three levels.
    g = np.random.Generator(np.random.PCG64(41))
    pts = g.random((60000, 3))
    vals = workloads.f_c1(pts)
    if kind == "cov_aniso":
        rbf = pg.CovExponential([1.0, 0.3])
        rbf.anisotropy = np.array([[1.0, 0.2, 0.0], [0.0, 1.0, 0.0], [0.1, 0.0, 0.5]])
        model = pg.Model(rbf, 0)
        model.nugget = 1e-3
    else:
        model = pg.Model(pg.Biharmonic3D([1.0]), 1)
    precision = pg.MIXED if kind == "bh3_mixed" else pg.PLAIN

    def fit():
        it = pg.Interpolant(model, precision)
        it.fit(pts, vals, 1e-4)
        return it.weights, it.fit_stats

    monkeypatch.delenv("PGPU_RAS_HOST_DIVIDE", raising=False)
    w_dev, s_dev = fit()
    w_again, _ = fit()
    monkeypatch.setenv("PGPU_RAS_HOST_DIVIDE", "1")
    w_host, s_host = fit()
    np.testing.assert_array_equal(w_dev, w_again)  # the fit itself is deterministic
    assert s_dev["levels"] == s_host["levels"] >= 3
    assert s_dev["n_domains"] == s_host["n_domains"]
    assert s_dev["iterations"] == s_host["iterations"]
    np.testing.assert_array_equal(w_dev, w_host)


def test_c3_kriging_tenth_scale_mixed_vs_plain():
    # The kriging configuration at a tenth of its size: 50,000 Gaussian-mixture points,
    # cov_exponential (range 0.2, anisotropy 1:1:0.5, nugget 1e-3), degree 0, tol 1e-4, 1M
    # uniform queries. At the default evaluation accuracy (infinity: order 6) the far field of
    # either arithmetic is off the exact sums by ~1e-3 for these weights, so the interpolants are
    # compared with evaluations at accuracy 1e-6 (the estimator's order, or exact sums): the
    # mixed interpolant is within 1e-4 of the plain FP64 one at every query, and the mixed
    # weights meet the tolerance at sampled data points, recomputed by the oracle.
    pts, vals, q, aniso = workloads.c3(n=50_000, n_eval=1_000_000)
    rbf = pg.CovExponential([1.0, 0.2])
    rbf.anisotropy = aniso
    model = pg.Model(rbf, 0)
    model.nugget = 1e-3
    tol = 1e-4
    mixed = pg.Interpolant(model, pg.MIXED)
    mixed.fit(pts, vals, tol)
    assert mixed.fit_stats["precision_used"] == pg.MIXED and mixed.fit_stats["fell_back"] == 0
    plain = pg.Interpolant(model, pg.PLAIN)
    plain.fit(pts, vals, tol)
    got = mixed.evaluate(q, accuracy=1e-6)
    want = plain.evaluate(q, accuracy=1e-6)
    assert np.max(np.abs(got - want)) <= 1e-4
    g = np.random.Generator(np.random.PCG64(51))
    idx = g.choice(pts.shape[0], 3000, replace=False)
    w = mixed.weights
    fit_vals = oracle.direct_evaluate(model, pts, w, pts[idx]) + model.nugget * w[idx]
    assert np.max(np.abs(fit_vals - vals[idx])) <= tol
    sub = q[g.choice(q.shape[0], 2000, replace=False)]
    exact = oracle.direct_evaluate(model, pts, w, sub)
    assert np.max(np.abs(mixed.evaluate(sub, accuracy=1e-6) - exact)) <= 1e-6


def test_evaluation_at_tight_accuracy_bh3():
    # A finite accuracy below what the far-field orders here reach falls back to exact sums
    # instead of failing (the reference reaches it with orders up to 20): accuracy 1e-8 on a
    # 30,000-point biharmonic interpolant at 400,000 queries, checked against the oracle.
    g = np.random.Generator(np.random.PCG64(52))
    pts = g.random((30_000, 3))
    vals = workloads.f_c1(pts)
    model = pg.Model(pg.Biharmonic3D([1.0]), 1)
    it = pg.Interpolant(model)
    it.fit(pts, vals, 1e-6)
    q = g.random((400_000, 3))
    got = it.evaluate(q, accuracy=1e-8)
    sub = g.choice(q.shape[0], 2000, replace=False)
    want = oracle.direct_evaluate(model, pts, it.weights, q[sub])
    assert np.max(np.abs(got[sub] - want)) <= 1e-8
    # The same at the default accuracy (order 6) is allowed a larger error.
    assert np.max(np.abs(it.evaluate(q[sub]) - want)) <= 1e-4


def test_c4_size_batched_fits_against_oracle():
    # 64 fits drawn like the batched configuration (N log-uniform in [200, 20000], triharmonic,
    # degree 1, tol 1e-5, 4,096 queries each): every residual at every data point and every
    # evaluation, recomputed by the oracle.
    fits = workloads.c4(n_fits=64)
    model = pg.Model(pg.Triharmonic3D([1.0]), 1)
    tol = 1e-5
    res = pg.fit_batch(model, fits, tol, precision=pg.MIXED)
    assert max(p.shape[0] for p, _, _ in fits) > 10_000
    for (p, v, q), r in zip(fits, res):
        assert r["status"] == 0
        w = r["weights"]
        assert np.max(np.abs(oracle.direct_evaluate(model, p, w, p) - v)) <= tol
        want = oracle.direct_evaluate(model, p, w, q)
        assert np.max(np.abs(r["values"] - want)) <= 1e-8 * max(1.0, np.max(np.abs(want)))
