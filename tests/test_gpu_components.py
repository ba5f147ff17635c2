"""The reference's own unit tests of the solver components, restated against the device code
through the C ABI:

- test/krylov/test_krylov.cpp:21-137 (FGMRES): on a random symmetric 100 x 100 operator, the
  relative residual that FGMRES reports equals the true relative residual of its solution
  estimate to 1e-12 at every iteration, and it decreases strictly; with and without an initial
  solution and a right preconditioner (the operator's inverse plus a 0.1 diagonal perturbation).
- test/preconditioner/test_coarse_grid.cpp:35-122: the coarse grid over 1,000 points
  (triharmonic, degree 1, nugget 0.01) reproduces the data, the fit recomputed by the oracle in
  FP64, to a relative error of 1e-8.
- test/preconditioner/test_fine_grid.cpp:37-141: a fine-grid domain holding the same points, half
  of them inner, gives the coarse solution on its inner points to a relative error of 1e-8.

Inputs follow the reference tests: Eigen's Random() draws U(-1, 1), here from numpy PCG64; the
sample data are uniform points in [-1, 1]^3 with values sum_j sin(pi x_j) (test/utility.hpp).
The gradient-point cases of the grid tests (1 point + 300 gradient points) are not restated:
the device preconditioner takes value points only."""
import ctypes as C

import numpy as np
import pytest

import oracle
import polatory_gb300 as pg
from polatory_gb300 import _lib

pytestmark = pytest.mark.gpu


def _p(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def fgmres(op, rhs, iters, pc=None, x0=None):
    n = op.shape[0]
    sols = np.zeros((iters, n))
    res = np.zeros(iters)
    op = np.ascontiguousarray(op)
    pc = None if pc is None else np.ascontiguousarray(pc)
    _lib.check(_lib.lib.pgpu_krylov_fgmres_dense(n, _p(op), _p(pc), _p(rhs), _p(x0), iters,
                                                 _p(sols), _p(res)))
    return sols, res


@pytest.mark.parametrize("with_x0,with_pc", [(False, False), (False, True), (True, False),
                                             (True, True)],
                         ids=["plain", "right_pc", "x0", "x0_right_pc"])
def test_fgmres_reported_residual_is_true_and_decreasing(with_x0, with_pc):
    n = 100
    g = np.random.Generator(np.random.PCG64(31))
    m = (g.uniform(-1, 1, (n, n)) + 1.0) / 2.0
    m = np.triu(m) + np.triu(m, 1).T  # symmetric: the lower triangle mirrors the upper
    pc = np.linalg.inv(m) + np.diag(0.1 * g.uniform(-1, 1, n))
    solution = (g.uniform(-1, 1, n) + 1.0) / 2.0
    rhs = m @ solution
    x0 = g.uniform(-1, 1, n)
    sols, res = fgmres(m, rhs, n, pc if with_pc else None, x0 if with_x0 else None)
    rhs_norm = np.linalg.norm(rhs)
    last = 0.0
    for i in range(n):
        true = np.linalg.norm(rhs - m @ sols[i]) / rhs_norm
        assert abs(true - res[i]) <= 1e-12, (i, true, res[i])
        if i > 0:
            assert res[i] < last, (i, res[i], last)
        last = res[i]


def sample_data(g, n):
    pts = g.uniform(-1, 1, (n, 3))
    return pts, np.sin(np.pi * pts).sum(axis=1)


def domain_solve(model, pts, order, inner, rhs, coarse, use_inverse=False, precision=pg.PLAIN):
    n = pts.shape[0]
    l = model.poly_basis_size
    out = np.zeros(n + l)
    m = model._c()
    order = np.ascontiguousarray(order, dtype=np.int64)
    inner = np.ascontiguousarray(inner, dtype=np.uint8)
    _lib.check(_lib.lib.pgpu_ras_domain_solve(C.byref(m), _p(np.ascontiguousarray(pts)), n,
                                              C.c_void_p(order.ctypes.data),
                                              C.c_void_p(inner.ctypes.data), int(coarse),
                                              int(use_inverse), precision, _p(rhs), _p(out)))
    return out


def rel_err(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("use_inverse", [False, True], ids=["factor", "explicit_inverse"])
def test_coarse_grid_reproduces_data(use_inverse):
    g = np.random.Generator(np.random.PCG64(41))
    pts, vals = sample_data(g, 1000)
    model = pg.Model(pg.Triharmonic3D([1.0]), 1)
    model.nugget = 0.01
    order = g.permutation(pts.shape[0])
    sol = domain_solve(model, pts, order, np.ones(pts.shape[0]), vals, True, use_inverse)
    fit = oracle.direct_evaluate(model, pts, sol, pts) + model.nugget * sol[: pts.shape[0]]
    assert rel_err(fit, vals) < 1e-8


def test_fine_grid_equals_coarse_on_inner_points():
    g = np.random.Generator(np.random.PCG64(43))
    pts, vals = sample_data(g, 1000)
    n = pts.shape[0]
    model = pg.Model(pg.Triharmonic3D([1.0]), 1)
    l = model.poly_basis_size
    order = g.permutation(n)
    inner = np.ones(n, dtype=np.uint8)
    inner[n // 2:] = 0
    coarse = domain_solve(model, pts, order, np.ones(n), vals, True)
    fine = domain_solve(model, pts, order, inner, vals, False)
    want = coarse.copy()
    want[order[inner == 0]] = 0.0
    want[n:] = 0.0
    assert np.all(fine[order[inner == 0]] == 0.0)
    assert np.all(fine[n:] == 0.0)
    assert rel_err(fine, want) < 1e-8


def test_fine_grid_fp32_factors_biharmonic():
    # The mixed path's FP32 fine-grid factors serve kernels of cpd order 1 (biharmonic; the
    # triharmonic domain matrices keep FP64 factors): FP32-level agreement with the FP64 solve.
    g = np.random.Generator(np.random.PCG64(44))
    pts, vals = sample_data(g, 1000)
    n = pts.shape[0]
    model = pg.Model(pg.Biharmonic3D([1.0]), 0)
    order = g.permutation(n)
    inner = np.ones(n, dtype=np.uint8)
    inner[n // 2:] = 0
    fine64 = domain_solve(model, pts, order, inner, vals, False)
    fine32 = domain_solve(model, pts, order, inner, vals, False, precision=pg.MIXED)
    assert np.all(np.isfinite(fine32))
    assert rel_err(fine32, fine64) < 1e-2
