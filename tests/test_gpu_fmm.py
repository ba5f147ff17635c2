"""FMM parity against the oracle's exact sums, restating the reference's differential tests
(test/interpolation/test_evaluator.cpp:27-76: FMM evaluator vs DirectEvaluator within the
requested accuracy). The error is normalised by the conditioning of the sum,
s_i = sum_j |w_j phi(x_i - y_j)| (computed by the oracle), so the bound is independent of the
weights' scale."""
import numpy as np
import pytest

import oracle
import polatory_gb300 as pg
from polatory_gb300 import _lib

pytestmark = pytest.mark.gpu

# Relative-to-conditioning bounds per Chebyshev order (estimated from rho^-p with rho ~ 5.8 for
# the nearest well-separated cells, times a safety factor).
BOUND = {4: 2e-3, 6: 1e-4, 8: 5e-6}


def sample(n_src, n_trg, seed, clustered=False):
    g = np.random.Generator(np.random.PCG64(seed))
    if clustered:
        c = g.random((16, 3))
        src = c[g.integers(0, 16, n_src)] + 0.05 * g.standard_normal((n_src, 3))
    else:
        src = g.random((n_src, 3))
    trg = g.random((n_trg, 3))
    w = g.standard_normal(n_src)
    return src, trg, w


def check(rbf, order, precision, src, trg, w, symmetric=False, leaf_level=-1):
    lo = np.minimum(src.min(0), trg.min(0))
    hi = np.maximum(src.max(0), trg.max(0))
    ev = pg.FmmEvaluator(rbf, np.concatenate([lo, hi]), symmetric=symmetric, precision=precision)
    ev.configure(backend=2, order=order, leaf_level=leaf_level)
    if symmetric:
        ev.set_points(src)
    else:
        ev.set_source_points(src)
        ev.set_target_points(trg)
    ev.set_weights(w)
    got = ev.evaluate()
    m = pg.Model(rbf, rbf.cpd_order - 1)._c()
    m.poly_degree = -1
    tpts = src if symmetric else trg
    want = oracle.direct_evaluate(m, src, w, tpts)
    # |phi| sums: evaluate |phi| with |w| through the oracle on a subsample of targets.
    sub = np.arange(0, tpts.shape[0], max(1, tpts.shape[0] // 200))
    absum = np.zeros(sub.shape[0])
    for k, i in enumerate(sub):
        d = tpts[i] - src
        vals = np.array([oracle.rbf_evaluate(rbf._kind, rbf.parameters, rbf.anisotropy, dd)[0]
                         for dd in d[:: max(1, src.shape[0] // 2000)]])
        absum[k] = np.abs(vals).mean() * np.abs(w).sum()
    scale = absum.max()
    err = np.max(np.abs(got - want))
    return err, scale


@pytest.mark.parametrize("cls,params", [(pg.Biharmonic3D, [1.0]), (pg.Triharmonic3D, [1.0]),
                                        (pg.CovExponential, [1.0, 0.3]),
                                        (pg.CovGaussian, [1.0, 0.5])],
                         ids=["bh3", "th3", "exp", "gau"])
@pytest.mark.parametrize("order", [6, 8])
def test_fmm_plain_matches_direct(cls, params, order):
    src, trg, w = sample(20000, 3000, 31)
    err, scale = check(cls(params), order, pg.PLAIN, src, trg, w)
    print(f"order {order}: err {err:.3e} scale {scale:.3e} rel {err / scale:.3e}")
    assert err <= BOUND[order] * scale


@pytest.mark.parametrize("order", [6, 8])
def test_fmm_mixed_matches_direct(order):
    src, trg, w = sample(20000, 3000, 32)
    err, scale = check(pg.Biharmonic3D([1.0]), order, pg.MIXED, src, trg, w)
    print(f"mixed order {order}: err {err:.3e} scale {scale:.3e} rel {err / scale:.3e}")
    assert err <= max(BOUND[order], 2e-5) * scale


def test_fmm_clustered_symmetric_anisotropic():
    src, _, w = sample(15000, 0, 33, clustered=True)
    rbf = pg.Triharmonic3D([1.0])
    rbf.anisotropy = np.diag([1.0, 1.0, 2.0])
    err, scale = check(rbf, 6, pg.PLAIN, src, src, w, symmetric=True)
    print(f"clustered: err {err:.3e} scale {scale:.3e} rel {err / scale:.3e}")
    assert err <= BOUND[6] * scale


@pytest.mark.parametrize("leaf_level", [2, 3, 4])
def test_fmm_leaf_levels(leaf_level):
    src, trg, w = sample(12000, 2000, 34)
    err, scale = check(pg.Biharmonic3D([1.0]), 6, pg.PLAIN, src, trg, w, leaf_level=leaf_level)
    print(f"leaf level {leaf_level}: rel {err / scale:.3e}")
    assert err <= BOUND[6] * scale


def test_fmm_empty_and_tiny():
    rbf = pg.Biharmonic3D([1.0])
    ev = pg.FmmEvaluator(rbf, [0, 0, 0, 1, 1, 1])
    ev.configure(backend=2, order=6)
    ev.set_source_points(np.random.default_rng(0).random((5, 3)))
    ev.set_target_points(np.zeros((0, 3)))
    ev.set_weights(np.ones(5))
    assert ev.evaluate().shape == (0,)


@pytest.mark.parametrize("cls,params", [(pg.Biharmonic3D, [1.0]), (pg.Triharmonic3D, [1.0]),
                                        (pg.CovExponential, [1.0, 0.3])],
                         ids=["bh3", "th3", "exp"])
def test_fmm_mixed_tensor_core_m2l(cls, params):
    # 400k uniform sources at leaf level 5: every level runs the tensor-core M2L (TF32
    # head/tail split; the small levels split their offsets over several CTAs). Against the
    # FP64 FMM with the same order and tree, the difference is rounding only; against the exact
    # sums, the order-6 bound.
    src, trg, w = sample(400000, 4000, 33)
    rbf = cls(params)
    lo = np.minimum(src.min(0), trg.min(0))
    hi = np.maximum(src.max(0), trg.max(0))
    out = {}
    for prec in (pg.MIXED, pg.PLAIN):
        ev = pg.FmmEvaluator(rbf, np.concatenate([lo, hi]), precision=prec)
        ev.configure(backend=2, order=6, leaf_level=5)
        ev.set_source_points(src)
        ev.set_target_points(trg)
        ev.set_weights(w)
        out[prec] = ev.evaluate()
    m = pg.Model(rbf, rbf.cpd_order - 1)._c()
    m.poly_degree = -1
    want = oracle.direct_evaluate(m, src, w, trg)
    # Mean |phi| over the unit cube times sum |w| (from 2000 sampled pairs).
    g = np.random.Generator(np.random.PCG64(1))
    i, j = g.integers(0, src.shape[0], 2000), g.integers(0, trg.shape[0], 2000)
    phis = [oracle.rbf_evaluate(rbf._kind, rbf.parameters, rbf.anisotropy, d)[0]
            for d in trg[j] - src[i]]
    scale = np.abs(w).sum() * np.mean(np.abs(phis))
    assert np.all(np.isfinite(out[pg.MIXED]))
    d32 = np.max(np.abs(out[pg.MIXED] - out[pg.PLAIN]))
    e64 = np.max(np.abs(out[pg.PLAIN] - want))
    print(f"fp32 vs fp64 fmm {d32:.3e}, fp64 fmm vs exact {e64:.3e}, scale {scale:.3e}")
    assert d32 <= 1e-6 * scale
    assert np.max(np.abs(out[pg.MIXED] - want)) <= BOUND[6] * scale


@pytest.mark.parametrize("precision", [pg.PLAIN, pg.MIXED], ids=["plain", "mixed"])
def test_fmm_accuracy_estimate(precision):
    # A finite accuracy selects the order by comparing the FMM with exact sums at up to 10,000
    # sampled source points (fmm_accuracy_estimator.hpp:74-121); an accuracy no far-field order
    # here reaches falls back to exact sums (the reference's higher orders reach such accuracies).
    src, trg, w = sample(30000, 3000, 34)
    rbf = pg.Biharmonic3D([1.0])
    scale = np.abs(w).sum() * 0.66
    acc = (1e-6 if precision == pg.PLAIN else 3e-6) * scale
    lo = np.minimum(src.min(0), trg.min(0))
    hi = np.maximum(src.max(0), trg.max(0))
    ev = pg.FmmEvaluator(rbf, np.concatenate([lo, hi]), precision=precision)
    ev.configure(backend=2, order=0, leaf_level=-1)
    ev.set_accuracy(acc)
    ev.set_source_points(src)
    ev.set_target_points(trg)
    ev.set_weights(w)
    got = ev.evaluate()
    m = pg.Model(rbf, 0)._c()
    m.poly_degree = -1
    want = oracle.direct_evaluate(m, src, w, trg)
    assert np.max(np.abs(got - want)) <= 2.0 * acc
    bad = pg.FmmEvaluator(rbf, np.concatenate([lo, hi]), precision=precision)
    bad.configure(backend=2, order=0, leaf_level=-1)
    bad.set_accuracy(1e-13 * scale)
    bad.set_source_points(src)
    bad.set_target_points(trg)
    bad.set_weights(w)
    assert np.max(np.abs(bad.evaluate() - want)) <= 2e-13 * scale


@pytest.mark.parametrize("precision", [pg.PLAIN, pg.MIXED], ids=["plain", "mixed"])
@pytest.mark.parametrize("cls,params", [(pg.Biharmonic3D, [1.0]), (pg.CovExponential, [1.0, 0.3])],
                         ids=["bh3", "exp"])
def test_fmm_gradient_targets(cls, params, precision):
    # Value sources, gradient targets (fmm/gradient_transpose_kernel.hpp: grad_x of sum_j w_j
    # phi(A (x - y_j)) = A^T grad phi): L2P of the expansion's derivative and the gradient near
    # field, against the oracle's exact gradients (test/interpolation/test_evaluator.cpp:27-76
    # checks gradients of the FMM evaluator against the direct sums the same way).
    src, trg, w = sample(60000, 20000, 36)
    rbf = cls(params)
    rbf.anisotropy = np.array([[1.0, 0.2, 0.0], [0.0, 0.9, 0.1], [0.0, 0.0, 1.1]])
    ev = pg.FmmEvaluator(rbf, [0, 0, 0, 1, 1, 1], kernel=_lib.KERNEL_GRADIENT_TRANSPOSE,
                         precision=precision)
    ev.configure(backend=2)
    ev.set_source_points(src)
    ev.set_target_points(trg)
    ev.set_weights(w)
    got = ev.evaluate().reshape(-1, 3)
    m = pg.Model(rbf, 0)._c()
    m.poly_degree = -1
    want = oracle.direct_evaluate(m, src, w, np.zeros((0, 3)), gtrg=trg).reshape(-1, 3)
    scale = np.abs(w).sum() * max(1.0, np.max(np.abs(want)) / np.abs(w).sum())
    bound = 2e-5 if cls is pg.Biharmonic3D else 1e-4
    assert np.max(np.abs(got - want)) <= bound * scale, (np.max(np.abs(got - want)), scale)


def test_interpolant_gradients_through_the_fmm():
    # Interpolant::evaluate with gradient points (evaluate(points, grad_points)): values and
    # gradients of a 30,000-point biharmonic interpolant at 50,000 points.
    g = np.random.Generator(np.random.PCG64(37))
    pts = g.random((30000, 3))
    vals = np.sin(3 * pts[:, 0]) + pts[:, 1] * pts[:, 2]
    model = pg.Model(pg.Biharmonic3D([1.0]), 1)
    it = pg.Interpolant(model)
    it.fit(pts, vals, 1e-6)
    q = g.random((50000, 3))
    out = it.evaluate(q, grad_points=q)
    grads = out[q.shape[0]:].reshape(-1, 3)
    sub = g.choice(q.shape[0], 1000, replace=False)
    want = oracle.direct_evaluate(model, pts, it.weights, np.zeros((0, 3)), gtrg=q[sub]).reshape(-1, 3)
    assert np.max(np.abs(grads[sub] - want)) <= 1e-4 * max(1.0, np.max(np.abs(want)))


@pytest.mark.parametrize("precision", [pg.PLAIN, pg.MIXED], ids=["plain", "mixed"])
@pytest.mark.parametrize("kernel", [_lib.KERNEL_GRADIENT, _lib.KERNEL_HESSIAN], ids=["grad", "hess"])
@pytest.mark.parametrize("cls,params", [(pg.Biharmonic3D, [1.0]), (pg.CovGaussian, [1.0, 0.4])],
                         ids=["bh3", "gau"])
def test_fmm_gradient_sources(cls, params, kernel, precision):
    # Gradient sources (fmm/gradient_kernel.hpp, hessian_kernel.hpp): dipole P2M and near field,
    # value or gradient targets, against the oracle's exact sums (test_evaluator.cpp:27-76).
    g = np.random.Generator(np.random.PCG64(38))
    src = g.random((40000, 3))
    trg = g.random((15000, 3))
    w = g.standard_normal(3 * 40000)
    rbf = cls(params)
    rbf.anisotropy = np.array([[1.0, 0.1, 0.0], [0.0, 0.9, 0.0], [0.1, 0.0, 1.2]])
    ev = pg.FmmEvaluator(rbf, [0, 0, 0, 1, 1, 1], kernel=kernel, precision=precision)
    ev.configure(backend=2)
    ev.set_source_points(src)
    ev.set_target_points(trg)
    ev.set_weights(w)
    got = ev.evaluate()
    m = pg.Model(rbf, 0)._c()
    m.poly_degree = -1
    empty = np.zeros((0, 3))
    if kernel == _lib.KERNEL_GRADIENT:
        want = oracle.direct_evaluate(m, empty, w, trg, gsrc=src)
    else:
        want = oracle.direct_evaluate(m, empty, w, empty, gsrc=src, gtrg=trg)
    scale = np.abs(w).sum() / 3 * max(1.0, np.max(np.abs(want)) / (np.abs(w).sum() / 3))
    bound = 1e-4 if cls is pg.Biharmonic3D else 1e-3
    assert np.max(np.abs(got - want)) <= bound * scale, (np.max(np.abs(got - want)), scale)


def test_operator_cache_is_bounded():
    # Every bounding box gives the far field a new cell radius. The homogeneous kernels' operators
    # are stored at radius 1 and serve every box; the others' are kept within the byte limit,
    # least recently used first out, and results stay exact to the order's bound throughout.
    before = pg.operator_cache_stats()
    for s in (1.0, 0.37, 2.9, 11.0):
        src, trg, w = sample(60000, 3000, 91)
        err, scale = check(pg.Biharmonic3D([1.0]), 6, pg.MIXED, s * src, s * trg + 0.1, w,
                           leaf_level=4)
        assert err <= BOUND[6] * scale, (s, err, scale)
        if s == 1.0:
            first = pg.operator_cache_stats()
    assert pg.operator_cache_stats()["entries"] == first["entries"]
    assert first["entries"] - before["entries"] <= 3  # levels 2-4, once
    limit = before["limit"]
    try:
        pg.set_operator_cache_limit(300 << 20)
        assert pg.operator_cache_stats()["bytes"] <= 300 << 20
        for s in (1.0, 0.8, 1.3, 0.6, 1.7):
            src, trg, w = sample(60000, 3000, 92)
            err, scale = check(pg.CovExponential([1.0, 0.3]), 6, pg.MIXED, s * src, s * trg, w,
                               leaf_level=4)
            assert err <= BOUND[6] * scale, (s, err, scale)
            st = pg.operator_cache_stats()
            assert st["bytes"] <= st["limit"] or st["entries"] == 1, st
    finally:
        pg.set_operator_cache_limit(limit)
    assert pg.operator_cache_stats()["limit"] == limit
