"""The oracle's kernel formulas against the reference's own invariant tests
(test/rbf/test_rbf.cpp:126-174: central-difference gradients and Hessians with h = 1e-8 and
tolerance 1e-4 on 100 random points in [h, 2]^3; the anisotropy identity) and against known
answers derived by hand from the reference formulas (sign conventions: Biharmonic3D is -r,
Triharmonic3D is +r^3, polyharmonic_odd.hpp:21)."""
import math

import numpy as np
import pytest

import oracle

KINDS = {"bh2": 0, "bh3": 1, "cub": 2, "exp": 3, "gau": 4, "gc3": 5, "gc5": 6, "gc7": 7,
         "gc9": 8, "sph": 9, "sp3": 10, "sp5": 11, "sp7": 12, "sp9": 13, "th2": 14, "th3": 15}
POLYHARMONIC = {"bh2", "bh3", "th2", "th3"}
NO_HESSIAN = {"cub", "sph"}


def params_for(name):
    # test_rbf.cpp:146-173: {1.1, 0.1} for polyharmonic kernels, {1.1, 0.9} for covariances.
    return [1.1, 0.1] if name in POLYHARMONIC else [1.1, 0.9]


def grad_approx(kind, p, v, h):
    out = np.zeros(3)
    for k in range(3):
        e = np.zeros(3)
        e[k] = h
        out[k] = (oracle.rbf_isotropic(kind, p, v + e)[0] - oracle.rbf_isotropic(kind, p, v - e)[0]) / (2 * h)
    return out


def hess_approx(kind, p, v, h):
    m = np.zeros((3, 3))
    for k in range(3):
        e = np.zeros(3)
        e[k] = h
        m[k] = (oracle.rbf_isotropic(kind, p, v + e)[1] - oracle.rbf_isotropic(kind, p, v - e)[1]) / (2 * h)
    return m


@pytest.mark.parametrize("name", sorted(KINDS))
def test_gradient_central_difference(name):
    kind, p = KINDS[name], params_for(name)
    h, tol = 1e-8, 1e-4
    g = np.random.Generator(np.random.PCG64(10 + kind))
    for _ in range(100):
        v = g.uniform(h, 2.0, 3)
        grad = oracle.rbf_isotropic(kind, p, v)[1]
        assert np.linalg.norm(grad_approx(kind, p, v, h) - grad) <= tol


@pytest.mark.parametrize("name", sorted(set(KINDS) - NO_HESSIAN))
def test_hessian_central_difference(name):
    kind, p = KINDS[name], params_for(name)
    h, tol = 1e-8, 1e-4
    g = np.random.Generator(np.random.PCG64(40 + kind))
    for _ in range(100):
        v = g.uniform(h, 2.0, 3)
        hess = oracle.rbf_isotropic(kind, p, v)[2]
        assert np.linalg.norm(hess_approx(kind, p, v, h) - hess) <= tol


@pytest.mark.parametrize("name", sorted(NO_HESSIAN))
def test_no_hessian(name):
    assert oracle.rbf_isotropic(KINDS[name], params_for(name), [0.1, 0.2, 0.3])[2] is None


def test_anisotropy_identity():
    # test_rbf.cpp:126-135: evaluate(A v) of the isotropic kernel == anisotropic evaluate(v).
    g = np.random.Generator(np.random.PCG64(7))
    rot, _ = np.linalg.qr(g.standard_normal((3, 3)))
    if np.linalg.det(rot) < 0:
        rot[:, 0] *= -1
    scale = np.diag(10 ** (0.5 * g.uniform(-1, 1, 3)))
    scale /= np.prod(np.diag(scale)) ** (1 / 3)
    a = scale @ rot
    v = np.ones(3)
    iso = oracle.rbf_evaluate(1, [1.0, 0.0], np.eye(3), a @ v)[0]
    ani = oracle.rbf_evaluate(1, [1.0, 0.0], a, v)[0]
    assert iso == pytest.approx(ani, rel=1e-14)


def test_known_answers():
    d = [3.0, 4.0, 0.0]  # |d| = 5
    assert oracle.rbf_isotropic(KINDS["bh3"], [1.0, 0.0], d)[0] == -5.0
    assert oracle.rbf_isotropic(KINDS["th3"], [1.0, 0.0], d)[0] == 125.0
    assert oracle.rbf_isotropic(KINDS["bh2"], [1.0, 0.0], d)[0] == pytest.approx(25 * math.log(5))
    assert oracle.rbf_isotropic(KINDS["th2"], [1.0, 0.0], d)[0] == pytest.approx(-625 * math.log(5))
    assert oracle.rbf_isotropic(KINDS["exp"], [2.0, 5.0], d)[0] == pytest.approx(2 * math.exp(-3))
    assert oracle.rbf_isotropic(KINDS["gau"], [2.0, 5.0], d)[0] == pytest.approx(2 * math.exp(-3))
    assert oracle.rbf_isotropic(KINDS["sph"], [1.0, 5.0], d)[0] == 0.0
    assert oracle.rbf_isotropic(KINDS["cub"], [1.0, 10.0], d)[0] == pytest.approx(
        1 + 0.25 * (-7 + 0.5 * (8.75 + 0.25 * (-3.5 + 0.75 * 0.25))))
    # Covariances are psill at 0; polyharmonic kernels vanish at 0 (c = 0).
    for name in KINDS:
        val = oracle.rbf_isotropic(KINDS[name], [1.0, 1.0] if name not in POLYHARMONIC else [1.0, 0.0],
                                   [0.0, 0.0, 0.0])[0]
        assert val == (0.0 if name in POLYHARMONIC else 1.0)
    # Biharmonic3D gradient at 0 is zero (polyharmonic_odd.hpp:47-49).
    assert np.all(oracle.rbf_isotropic(KINDS["bh3"], [1.0, 0.0], [0.0, 0.0, 0.0])[1] == 0.0)
