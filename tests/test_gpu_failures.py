"""Failure detection without a GPU fault: failures are made on the host (an injected allocation
failure, non-finite inputs) or by a bounded device wait that is made to run out (the tensor-core
M2L leaves one operator copy unissued and polls its mbarrier a few times only), and each must
surface as the documented status while the library stays usable for the next call."""
import numpy as np
import pytest

import polatory_gb300 as pg
from polatory_gb300 import _lib, workloads

pytestmark = pytest.mark.gpu


def inject(what, after):
    _lib.check(_lib.lib.pgpu_debug_inject(what, after))


def small_fit(precision=pg.PLAIN, n=3000, seed=5):
    g = np.random.Generator(np.random.PCG64(seed))
    pts = g.random((n, 3))
    vals = workloads.f_c1(pts)
    interp = pg.Interpolant(pg.Model(pg.Biharmonic3D([1.0]), 1), precision)
    interp.fit(pts, vals, 1e-5)
    return interp


@pytest.mark.parametrize("after", [1, 7, 40])
def test_injected_allocation_failure_is_out_of_memory(after):
    inject(_lib.INJECT_ALLOC, after)
    try:
        with pytest.raises(_lib.PolatoryError) as e:
            small_fit()
    finally:
        inject(_lib.INJECT_ALLOC, 0)
    assert e.value.code == _lib.PGPU_OUT_OF_MEMORY
    assert "out of device memory" in str(e.value)
    # The next call succeeds.
    assert small_fit().fit_stats["iterations"] >= 1


def test_non_finite_inputs_are_rejected():
    g = np.random.Generator(np.random.PCG64(6))
    pts = g.random((500, 3))
    vals = workloads.f_c1(pts)
    model = pg.Model(pg.Biharmonic3D([1.0]), 1)
    for bad_pts, bad_vals in [(pts.copy(), vals), (pts, vals.copy())]:
        if bad_pts is not pts:
            bad_pts[17, 1] = np.nan
        else:
            bad_vals[3] = np.inf
        with pytest.raises(_lib.PolatoryError) as e:
            pg.Interpolant(model).fit(bad_pts, bad_vals, 1e-5)
        assert e.value.code == _lib.PGPU_INVALID_ARGUMENT
        assert "must be finite" in str(e.value)
    interp = pg.Interpolant(model)
    interp.fit(pts, vals, 1e-5)
    q = g.random((50, 3))
    q[7, 2] = np.nan
    with pytest.raises(_lib.PolatoryError) as e:
        interp.evaluate(q)
    assert e.value.code == _lib.PGPU_INVALID_ARGUMENT
    ev = pg.FmmEvaluator(model.rbfs[0], [0, 0, 0, 1, 1, 1])
    with pytest.raises(_lib.PolatoryError) as e:
        ev.set_source_points(q)
    assert e.value.code == _lib.PGPU_INVALID_ARGUMENT
    # Finite queries still evaluate.
    assert np.all(np.isfinite(interp.evaluate(np.nan_to_num(q, nan=0.5))))


def test_m2l_bounded_wait_runs_out_with_timeout_status():
    # An FP32 FMM evaluation large enough for the tensor-core M2L (order 6).
    g = np.random.Generator(np.random.PCG64(7))
    src = g.random((200_000, 3))
    w = g.standard_normal(200_000)
    trg = g.random((100_000, 3))
    rbf = pg.Biharmonic3D([1.0])
    ev = pg.FmmEvaluator(rbf, [0, 0, 0, 1, 1, 1], precision=pg.MIXED)
    ev.configure(backend=2, order=6)
    ev.set_source_points(src)
    ev.set_target_points(trg)
    ev.set_weights(w)
    want = ev.evaluate()
    inject(_lib.INJECT_M2L_STALL, 64)
    try:
        with pytest.raises(_lib.PolatoryError) as e:
            ev.evaluate()
    finally:
        inject(_lib.INJECT_M2L_STALL, 0)
    assert e.value.code == _lib.PGPU_TIMEOUT
    assert "bounded wait" in str(e.value)
    # The context is intact: the same evaluation runs again and gives the same result.
    again = ev.evaluate()
    assert np.array_equal(again, want)
