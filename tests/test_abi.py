"""CPU checks of the C ABI: the library loads, exports every function include/polatory_gpu.h
declares, and its host-side entry points (kernel formulas, model validation) agree with the
oracle. No GPU compute is called here."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import oracle
import polatory_gb300 as pg
from polatory_gb300 import _lib

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(pgpu_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(str(_lib.LIB_PATH))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert len(declared_functions()) >= 30


def test_version():
    assert _lib.lib.pgpu_version() >= 100


RBFS = [pg.Biharmonic2D, pg.Biharmonic3D, pg.CovCubic, pg.CovExponential, pg.CovGaussian,
        pg.CovGeneralizedCauchy3, pg.CovGeneralizedCauchy5, pg.CovGeneralizedCauchy7,
        pg.CovGeneralizedCauchy9, pg.CovSpherical, pg.CovSpheroidal3, pg.CovSpheroidal5,
        pg.CovSpheroidal7, pg.CovSpheroidal9, pg.Triharmonic2D, pg.Triharmonic3D]


@pytest.mark.parametrize("cls", RBFS, ids=lambda c: c.short_name)
def test_kernel_formulas_match_oracle(cls):
    g = np.random.Generator(np.random.PCG64(123))
    params = [1.3, 0.2] if cls._polyharmonic else [1.3, 0.8]
    rbf = cls(params)
    a = np.diag([1.2, 0.9, 1 / 1.08]) @ np.linalg.qr(g.standard_normal((3, 3)))[0]
    if np.linalg.det(a) < 0:
        a[:, 0] *= -1
    rbf.anisotropy = a
    diffs = g.uniform(-1.5, 1.5, (200, 3))
    vals = rbf.evaluate(diffs)
    grads = rbf.evaluate_gradient(diffs)
    has_h = cls.short_name not in ("cub", "sph")
    if has_h:
        hess = rbf.evaluate_hessian(diffs)
    else:
        with pytest.raises(pg.PolatoryError):
            rbf.evaluate_hessian(diffs)
    for i, d in enumerate(diffs):
        v, gr, h = oracle.rbf_evaluate(rbf._kind, params, a, d)
        assert vals[i] == pytest.approx(v, rel=1e-13, abs=1e-14)
        np.testing.assert_allclose(grads[i], gr, rtol=1e-12, atol=1e-13)
        if has_h:
            np.testing.assert_allclose(hess[i], h, rtol=1e-11, atol=1e-12)


def test_model_validation_errors():
    with pytest.raises(pg.PolatoryError, match="poly_degree must be within 0 to 2"):
        pg.Model(pg.Biharmonic3D([1.0]), -1)
    with pytest.raises(pg.PolatoryError, match="poly_degree must be within 2 to 2"):
        pg.Model(pg.Triharmonic2D([1.0]), 1)
    m = pg.Model(pg.Biharmonic3D([1.0]))
    assert m.poly_degree == 0 and m.poly_basis_size == 1
    m = pg.Model(pg.CovExponential([1.0, 0.2]))
    assert m.poly_degree == -1 and m.poly_basis_size == 0
    with pytest.raises(ValueError):
        m.nugget = -1.0
    with pytest.raises(ValueError, match="positive determinant"):
        pg.Biharmonic3D([1.0]).anisotropy = np.diag([1.0, 1.0, -1.0])
    with pytest.raises(RuntimeError, match="unknown RBF name"):
        pg.make_rbf("xyz", [])


def test_cpd_orders_and_support():
    assert pg.Biharmonic3D([1.0]).cpd_order == 1
    assert pg.Triharmonic3D([1.0]).cpd_order == 2
    assert pg.Biharmonic2D([1.0]).cpd_order == 2
    assert pg.Triharmonic2D([1.0]).cpd_order == 3
    assert pg.CovExponential([1.0, 0.5]).cpd_order == 0
    assert pg.CovCubic([1.0, 0.5]).support_radius_isotropic() == 0.5
    assert pg.CovSpherical([1.0, 0.7]).support_radius_isotropic() == 0.7
    assert np.isinf(pg.CovExponential([1.0, 0.5]).support_radius_isotropic())


def test_server_estimate_and_argument_checks():
    fit_small = pg.Server.estimate_bytes(_lib.REQUEST_FIT, 1000)
    fit_big = pg.Server.estimate_bytes(_lib.REQUEST_FIT, 1000000)
    fit_mixed = pg.Server.estimate_bytes(_lib.REQUEST_FIT, 1000000, pg.MIXED)
    ev = pg.Server.estimate_bytes(_lib.REQUEST_EVALUATE, 1000000)
    assert 0 < fit_small < fit_big
    assert fit_mixed < fit_big
    assert ev < fit_big
    assert _lib.lib.pgpu_server_estimate_bytes(None) == -1
    h = C.c_void_p()
    assert _lib.lib.pgpu_server_create(-1, 0, C.byref(h)) == _lib.PGPU_INVALID_ARGUMENT
    assert _lib.lib.pgpu_server_create(2, -5, C.byref(h)) == _lib.PGPU_INVALID_ARGUMENT
    assert _lib.lib.pgpu_server_destroy(None) == _lib.PGPU_OK


def test_operator_cache_controls_on_the_host():
    # The far-field operator cache's statistics and limit are host state: an empty cache, the
    # default 8 GiB limit (PGPU_M2L_CACHE_MB unset), a limit that can be set and restored, and
    # a negative limit refused.
    import os

    st = pg.operator_cache_stats()
    assert st["bytes"] >= 0 and st["entries"] >= 0
    if "PGPU_M2L_CACHE_MB" not in os.environ:
        assert st["limit"] == 8192 << 20
    pg.set_operator_cache_limit(123 << 20)
    assert pg.operator_cache_stats()["limit"] == 123 << 20
    pg.set_operator_cache_limit(st["limit"])
    assert pg.operator_cache_stats()["limit"] == st["limit"]
    with pytest.raises(pg.PolatoryError, match="limit must be >= 0"):
        pg.set_operator_cache_limit(-1)


def test_gradient_fit_argument_errors_on_the_host():
    # Interpolant::fit with gradient points (interpolant.hpp:82-113): the value count must be
    # mu + 3 sigma (checked before the library is called).
    it = pg.Interpolant(pg.Model(pg.Triharmonic3D([1.0]), 1))
    pts = np.random.default_rng(1).random((10, 3))
    gpts = np.random.default_rng(2).random((4, 3))
    with pytest.raises(pg.PolatoryError, match="values.rows\\(\\) must be equal to 22"):
        it.fit(pts, np.zeros(10), 1e-4, grad_points=gpts, grad_tolerance=1e-4)
