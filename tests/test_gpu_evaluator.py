"""GPU parity of the evaluator (fmm/fmm_evaluator.hpp interface) against the oracle's exact
direct sums (interpolation/direct_evaluator.hpp:38-88), for every kernel. Below the direct
threshold the device runs exact tiled sums, so FP64 results agree to rounding."""
import numpy as np
import pytest

import oracle
import polatory_gb300 as pg
from polatory_gb300 import _lib

pytestmark = pytest.mark.gpu

RBFS = [pg.Biharmonic2D, pg.Biharmonic3D, pg.CovCubic, pg.CovExponential, pg.CovGaussian,
        pg.CovGeneralizedCauchy3, pg.CovGeneralizedCauchy5, pg.CovGeneralizedCauchy7,
        pg.CovGeneralizedCauchy9, pg.CovSpherical, pg.CovSpheroidal3, pg.CovSpheroidal5,
        pg.CovSpheroidal7, pg.CovSpheroidal9, pg.Triharmonic2D, pg.Triharmonic3D]


def aniso(seed):
    g = np.random.Generator(np.random.PCG64(seed))
    q = np.linalg.qr(g.standard_normal((3, 3)))[0]
    if np.linalg.det(q) < 0:
        q[:, 0] *= -1
    s = np.diag(10 ** (0.5 * g.uniform(-1, 1, 3)))
    s /= np.prod(np.diag(s)) ** (1 / 3)
    return s @ q


@pytest.mark.parametrize("cls", RBFS, ids=lambda c: c.short_name)
@pytest.mark.parametrize("precision", [pg.PLAIN, pg.MIXED], ids=["plain", "mixed"])
def test_direct_evaluator_matches_oracle(cls, precision):
    g = np.random.Generator(np.random.PCG64(5))
    src = g.uniform(-1, 1, (1500, 3))
    trg = g.uniform(-1, 1, (1100, 3))
    w = g.standard_normal(1500)
    params = [1.0, 0.0] if cls._polyharmonic else [1.0, 0.6]
    rbf = cls(params)
    rbf.anisotropy = aniso(11)
    ev = pg.FmmEvaluator(rbf, [-1, -1, -1, 1, 1, 1], precision=precision)
    ev.set_source_points(src)
    ev.set_target_points(trg)
    ev.set_weights(w)
    got = ev.evaluate()
    model = pg.Model(rbf, -1 if cls.short_name not in ("bh2", "th2", "th3", "bh3") else rbf.cpd_order - 1)
    m = model._c()
    m.poly_degree = -1
    want = oracle.direct_evaluate(m, src, np.concatenate([w]), trg)
    scale = np.abs(w).sum() * max(1.0, np.abs(want).max())
    tol = 1e-12 if precision == pg.PLAIN else 2e-6
    assert np.max(np.abs(got - want)) <= tol * scale


def test_symmetric_evaluator_matches_oracle():
    g = np.random.Generator(np.random.PCG64(6))
    pts = g.uniform(0, 1, (2000, 3))
    w = g.standard_normal(2000)
    rbf = pg.Triharmonic3D([1.0])
    ev = pg.FmmEvaluator(rbf, [0, 0, 0, 1, 1, 1], symmetric=True)
    ev.set_points(pts)
    ev.set_weights(w)
    got = ev.evaluate()
    m = pg.Model(rbf, 1)._c()
    m.poly_degree = -1
    want = oracle.direct_evaluate(m, pts, w, pts)
    assert np.max(np.abs(got - want)) <= 1e-12 * np.abs(want).max()


@pytest.mark.parametrize("kind", [_lib.KERNEL_VALUE, _lib.KERNEL_GRADIENT,
                                  _lib.KERNEL_GRADIENT_TRANSPOSE, _lib.KERNEL_HESSIAN],
                         ids=["value", "grad", "grad_t", "hess"])
@pytest.mark.parametrize("precision", [pg.PLAIN, pg.MIXED], ids=["plain", "mixed"])
def test_evaluator_kernel_kinds(kind, precision):
    # The four FMM evaluator kinds of the reference's factories (make_fmm_evaluator,
    # make_fmm_gradient_evaluator, ..._transpose_..., make_fmm_hessian_evaluator): value or
    # gradient point sets on either side, km and kn in {1, 3}; against the oracle's blocks.
    g = np.random.Generator(np.random.PCG64(51))
    rbf = pg.Triharmonic3D([1.0])
    a = np.diag([1.1, 0.9, 1.0]) @ np.linalg.qr(g.standard_normal((3, 3)))[0]
    if np.linalg.det(a) < 0:
        a[:, 0] *= -1
    rbf.anisotropy = a
    src = g.uniform(-1, 1, (700, 3))
    trg = g.uniform(-1, 1, (500, 3))
    gs = kind in (_lib.KERNEL_GRADIENT, _lib.KERNEL_HESSIAN)
    gt = kind in (_lib.KERNEL_GRADIENT_TRANSPOSE, _lib.KERNEL_HESSIAN)
    w = g.standard_normal(src.shape[0] * (3 if gs else 1))
    ev = pg.FmmEvaluator(rbf, [-1, -1, -1, 1, 1, 1], kernel=kind, precision=precision)
    ev.set_source_points(src)
    ev.set_target_points(trg)
    ev.set_weights(w)
    got = ev.evaluate()
    m = pg.Model(rbf, rbf.cpd_order - 1)._c()
    m.poly_degree = -1
    e = np.zeros((0, 3))
    want = oracle.direct_evaluate(m, e if gs else src, w, e if gt else trg,
                                  gsrc=src if gs else None, gtrg=trg if gt else None)
    assert got.shape == want.shape
    scale = np.abs(w).sum()
    tol = 1e-12 if precision == pg.PLAIN else 2e-6
    assert np.max(np.abs(got - want)) <= tol * scale
