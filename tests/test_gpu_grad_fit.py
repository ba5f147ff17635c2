"""Fits with gradient data (Hermite-Birkhoff interpolation): test/interpolation/test_fitter.cpp
restated. Points and gradient points, a triharmonic kernel with a random anisotropy, nugget
0.01, degree 1, tolerance 1e-3 for values and for gradients, accuracy tolerance / 100. The
residual of the GPU weights is recomputed by the oracle at every data point (values) and every
gradient point (the three derivatives), and small fits are compared with the oracle's exact
dense solution of the same system."""
import numpy as np
import pytest

import oracle
import polatory_gb300 as pg

pytestmark = pytest.mark.gpu


def random_anisotropy(g):
    # random_scaling() * random_rotation() of test/utility.hpp: a rotation from an
    # orthonormalised random matrix (determinant +1) and a scaling of determinant 1.
    q, _ = np.linalg.qr(g.uniform(-1, 1, (3, 3)))
    if np.linalg.det(q) < 0:
        q[:, 0] *= -1
    s = 10.0 ** (0.5 * g.uniform(-1, 1, 3))
    s *= np.prod(s) ** (-1.0 / 3)
    return np.diag(s) @ q


def sample(g, n, n_grad, aniso):
    # sample_data / sample_grad_data of test/utility.hpp: points in [-1, 1]^3, values
    # sum_j sin(pi (A p)_j) and their gradients A^T (pi cos(pi (A p)_j)).
    pts = g.uniform(-1, 1, (n, 3))
    vals = np.sin(np.pi * pts @ aniso.T).sum(axis=1)
    gpts = g.uniform(-1, 1, (n_grad, 3))
    grads = (np.pi * np.cos(np.pi * gpts @ aniso.T)) @ aniso
    return pts, gpts, np.concatenate([vals, grads.reshape(-1)])


def th3_model(aniso, nugget=0.01):
    rbf = pg.Triharmonic3D([1.0])
    rbf.anisotropy = aniso
    model = pg.Model(rbf, rbf.cpd_order - 1)
    model.nugget = nugget
    return model


def residuals(model, pts, gpts, w, rhs):
    mu = pts.shape[0]
    fit = oracle.direct_evaluate(model, pts, w, pts, gsrc=gpts, gtrg=gpts)
    fit[:mu] += model.nugget * w[:mu]
    return np.max(np.abs(fit[:mu] - rhs[:mu])), np.max(np.abs(fit[mu:] - rhs[mu:]), initial=0.0)


@pytest.mark.parametrize("n,n_grad", [(10000, 10000), (1, 10000)], ids=["values_and_grads", "special_case"])
@pytest.mark.parametrize("precision", [pg.PLAIN, pg.MIXED], ids=["plain", "mixed"])
def test_fitter(n, n_grad, precision):
    g = np.random.Generator(np.random.PCG64(101))
    aniso = random_anisotropy(g)
    pts, gpts, rhs = sample(g, n, n_grad, aniso)
    model = th3_model(aniso)
    tol = grad_tol = 1e-3
    it = pg.Interpolant(model, precision)
    it.fit(pts, rhs, tol, max_iter=100, accuracy=tol / 100, grad_points=gpts,
           grad_tolerance=grad_tol, grad_accuracy=grad_tol / 100)
    w = it.weights
    assert w.shape == (n + 3 * n_grad + model.poly_basis_size,)
    st = it.fit_stats
    assert st["precision_used"] == pg.PLAIN  # gradient data runs in FP64
    r, gr = residuals(model, pts, gpts, w, rhs)
    assert r < tol and gr < grad_tol, (r, gr, st)
    # The interpolant's values and gradients at new points equal the oracle's sums.
    q = g.uniform(-1, 1, (500, 3))
    got = it.evaluate(q, grad_points=q[:200])
    want = oracle.direct_evaluate(model, pts, w, q, gsrc=gpts, gtrg=q[:200])
    assert np.max(np.abs(got - want)) <= 1e-8 * max(1.0, np.max(np.abs(want)))


@pytest.mark.parametrize("kind", ["th3", "gau"])
def test_small_fit_equals_exact_solution(kind):
    # One RAS level (the coarse grid with value, gradient and Hessian blocks): the fit is the
    # oracle's exact dense solution of the same system, to the tolerance.
    g = np.random.Generator(np.random.PCG64(102))
    aniso = random_anisotropy(g)
    pts, gpts, rhs = sample(g, 300, 200, aniso)
    if kind == "th3":
        model = th3_model(aniso)
    else:
        rbf = pg.CovGaussian([1.0, 1.5])
        rbf.anisotropy = aniso
        model = pg.Model(rbf, 0)
        model.nugget = 1e-2
    it = pg.Interpolant(model)
    tol = 1e-8
    it.fit(pts, rhs, tol, grad_points=gpts, grad_tolerance=tol)
    w = it.weights
    r, gr = residuals(model, pts, gpts, w, rhs)
    assert r < tol and gr < tol
    exact = oracle.fit_exact(model, pts, rhs, gpts=gpts)
    q = g.uniform(-1, 1, (400, 3))
    got = it.evaluate(q)
    ref = oracle.direct_evaluate(model, pts, exact, q, gsrc=gpts)
    assert np.max(np.abs(got - ref)) <= 1e-5 * max(1.0, np.max(np.abs(ref)))


def test_warm_start_with_gradient_centres():
    # Interpolant::build_initial_weights with gradient centres: refitting the same data from the
    # previous interpolant converges at once (iteration 0).
    g = np.random.Generator(np.random.PCG64(103))
    aniso = random_anisotropy(g)
    pts, gpts, rhs = sample(g, 3000, 2000, aniso)
    model = th3_model(aniso)
    a = pg.Interpolant(model)
    a.fit(pts, rhs, 1e-4, grad_points=gpts, grad_tolerance=1e-4)
    b = pg.Interpolant(model)
    b.fit(pts, rhs, 1e-4, grad_points=gpts, grad_tolerance=1e-4, initial=a)
    assert b.fit_stats["iterations"] <= 1
    r, gr = residuals(model, pts, gpts, b.weights, rhs)
    assert r < 1e-4 and gr < 1e-4


def test_kernels_without_hessian_are_rejected():
    g = np.random.Generator(np.random.PCG64(104))
    pts = g.random((50, 3))
    gpts = g.random((20, 3))
    rhs = np.zeros(50 + 60)
    it = pg.Interpolant(pg.Model(pg.CovCubic([1.0, 0.5]), 0))
    with pytest.raises(pg.PolatoryError, match="cov_cubic::evaluate_hessian_isotropic is not implemented"):
        it.fit(pts, rhs, 1e-4, grad_points=gpts, grad_tolerance=1e-4)


def test_fitter_through_the_fmm():
    # 40,000 points and 40,000 gradient points (160,000 rows): the operator, the residual
    # check and the preconditioner's residual updates run the FMM's value, gradient, gradient-
    # transpose and Hessian blocks. The residual is recomputed by the oracle at 2,000 sampled
    # points and 2,000 sampled gradient points.
    g = np.random.Generator(np.random.PCG64(105))
    aniso = random_anisotropy(g)
    n = 40000
    pts, gpts, rhs = sample(g, n, n, aniso)
    model = th3_model(aniso)
    tol = 1e-3
    it = pg.Interpolant(model)
    it.fit(pts, rhs, tol, accuracy=tol / 100, grad_points=gpts, grad_tolerance=tol,
           grad_accuracy=tol / 100)
    st = it.fit_stats
    assert st["levels"] >= 3
    w = it.weights
    i = g.choice(n, 2000, replace=False)
    j = g.choice(n, 2000, replace=False)
    fit = oracle.direct_evaluate(model, pts, w, pts[i], gsrc=gpts, gtrg=gpts[j])
    fit[:2000] += model.nugget * w[i]
    want = np.concatenate([rhs[i], rhs[n:].reshape(-1, 3)[j].reshape(-1)])
    assert np.max(np.abs(fit[:2000] - want[:2000])) < tol, st
    assert np.max(np.abs(fit[2000:] - want[2000:])) < tol, st
