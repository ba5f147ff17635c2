"""Batched fits (pgpu_fit_batch): every problem of an uneven batch meets its tolerance at its
data points (recomputed by the oracle), its evaluation equals the oracle's for the returned
weights, and each result equals the same fit run alone through Interpolant (same kernels, same
order of operations)."""
import numpy as np
import pytest

import oracle
import polatory_gb300 as pg
from polatory_gb300 import workloads

pytestmark = pytest.mark.gpu


def make_batch(n_fits, seed, n_min=200, n_max=5000, n_eval=300):
    g = np.random.Generator(np.random.PCG64(seed))
    sizes = np.round(np.exp(g.uniform(np.log(n_min), np.log(n_max), n_fits))).astype(int)
    probs = []
    for n in sizes:
        p = g.random((n, 3))
        v = workloads.f_c1(p) + g.normal(0.0, 1e-4, n)
        probs.append((p, v, g.random((n_eval, 3))))
    return probs


@pytest.mark.parametrize("precision", [pg.PLAIN, pg.MIXED], ids=["plain", "mixed"])
def test_batch_uneven_fits(precision):
    model = pg.Model(pg.Triharmonic3D([1.0]), 1)
    probs = make_batch(24, 41)
    tol = 1e-5
    res = pg.fit_batch(model, probs, tol, precision=precision, n_workers=8)
    for (p, v, q), r in zip(probs, res):
        assert r["status"] == 0
        w = r["weights"]
        fit_vals = oracle.direct_evaluate(model, p, w, p)
        assert np.max(np.abs(fit_vals - v)) <= tol
        want = oracle.direct_evaluate(model, p, w, q)
        # Below 2^30 pairs the sums are FP64 (plain) or float-float, FP64-class (mixed).
        assert np.max(np.abs(r["values"] - want)) <= (1e-9 if precision == pg.PLAIN else 1e-8)


def test_batch_result_equals_single_fit():
    model = pg.Model(pg.Triharmonic3D([1.0]), 1)
    probs = make_batch(6, 42, n_min=300, n_max=3000)
    res = pg.fit_batch(model, probs, 1e-5, n_workers=4)
    for (p, v, q), r in zip(probs, res):
        it = pg.Interpolant(model)
        it.fit(p, v, 1e-5)
        np.testing.assert_array_equal(it.weights, r["weights"])
        np.testing.assert_array_equal(it.evaluate(q), r["values"])


def test_batch_reports_failing_problem():
    model = pg.Model(pg.Triharmonic3D([1.0]), 1)
    probs = make_batch(3, 43, n_min=2500, n_max=4000)
    with pytest.raises(pg.PolatoryError):
        pg.fit_batch(model, probs, 1e-13, max_iter=1)
