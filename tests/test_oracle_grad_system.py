"""CPU pinning of the oracle's gradient-data system (the checker of the gradient-fit GPU tests):
the fit system of interpolation/solver.hpp with gradient points, assembled here in numpy from the
oracle's pointwise kernel (itself pinned by central differences in test_oracle_rbf.py) by the
block rules of preconditioner/mat_a.hpp:10-61 and polynomial/monomial_basis.hpp, against the
oracle's exact solve (orc_fit_exact) and its direct operator and evaluator."""
import numpy as np
import pytest

import oracle


def random_anisotropy(g):
    q, _ = np.linalg.qr(g.uniform(-1, 1, (3, 3)))
    s = 10.0 ** (0.5 * g.uniform(-1, 1, 3))
    return np.diag(s / np.prod(s) ** (1.0 / 3)) @ q


def monomials(degree, p):
    x, y, z = p
    return np.array([1.0, x, y, z, x * x, x * y, x * z, y * y, y * z, z * z])[:(degree + 1) * (degree + 2) * (degree + 3) // 6]


def monomial_derivatives(degree, p):
    x, y, z = p
    d = np.array([[0, 1, 0, 0, 2 * x, y, z, 0, 0, 0],
                  [0, 0, 1, 0, 0, x, 0, 2 * y, z, 0],
                  [0, 0, 0, 1, 0, 0, x, 0, y, 2 * z]], dtype=np.float64)
    return d[:, :(degree + 1) * (degree + 2) * (degree + 3) // 6]


def system(kind, params, aniso, degree, nugget, pts, gpts):
    """[[A, P], [P^T, 0]] with A's blocks phi(x_i - x_j) (+ nugget), -grad phi(x_i - y_j),
    -H(y_i - y_j) and P's value and derivative rows."""
    k = oracle.RBF_KINDS.index(kind)
    mu, sigma = pts.shape[0], gpts.shape[0]
    m = mu + 3 * sigma
    l = (degree + 1) * (degree + 2) * (degree + 3) // 6 if degree >= 0 else 0
    a = np.zeros((m + l, m + l))
    for i in range(mu):
        for j in range(mu):
            a[i, j] = oracle.rbf_evaluate(k, params, aniso, pts[i] - pts[j])[0]
        a[i, i] += nugget
        for j in range(sigma):
            g = oracle.rbf_evaluate(k, params, aniso, pts[i] - gpts[j])[1]
            a[i, mu + 3 * j: mu + 3 * j + 3] = -g
            a[mu + 3 * j: mu + 3 * j + 3, i] = -g
    for i in range(sigma):
        for j in range(sigma):
            h = oracle.rbf_evaluate(k, params, aniso, gpts[i] - gpts[j])[2]
            a[mu + 3 * i: mu + 3 * i + 3, mu + 3 * j: mu + 3 * j + 3] = -h
    if l:
        p = np.zeros((m, l))
        for i in range(mu):
            p[i] = monomials(degree, pts[i])
        for j in range(sigma):
            p[mu + 3 * j: mu + 3 * j + 3] = monomial_derivatives(degree, gpts[j])
        a[:m, m:] = p
        a[m:, :m] = p.T
    return a


@pytest.mark.parametrize("kind,params,degree,nugget", [("th3", [1.0], 1, 0.01),
                                                       ("gau", [1.0, 1.2], 0, 0.01),
                                                       ("bh3", [1.0], 1, 0.0)])
def test_gradient_system_matches_the_block_rules(kind, params, degree, nugget):
    g = np.random.Generator(np.random.PCG64(7))
    aniso = random_anisotropy(g)
    pts = g.uniform(-1, 1, (24, 3))
    gpts = g.uniform(-1, 1, (9, 3))
    if kind == "bh3":
        gpts = gpts[:0]  # bh3 (-r) has no Hessian at coincident points: values only
    m = oracle.model(kind, params, degree, nugget, aniso)
    a = system(kind, params, aniso, degree, nugget, pts, gpts)
    n = pts.shape[0] + 3 * gpts.shape[0]
    rhs = g.standard_normal(n)
    want = np.linalg.solve(a, np.concatenate([rhs, np.zeros(a.shape[0] - n)]))
    got = oracle.fit_exact(m, pts, rhs, gpts=gpts)
    assert np.max(np.abs(got - want)) <= 1e-8 * max(1.0, np.max(np.abs(want)))
    # The oracle's operator applies the same matrix (values and derivative rows, then P^T w).
    w = g.standard_normal(a.shape[0])
    assert np.allclose(oracle.direct_operator(m, pts, w, gpts=gpts), a @ w, rtol=1e-10, atol=1e-10)
    # Its evaluator at the data points and gradient points gives the first n rows of A w without
    # the nugget.
    ev = oracle.direct_evaluate(m, pts, w, pts, gsrc=gpts, gtrg=gpts)
    aw = a[:n] @ w
    aw[:pts.shape[0]] -= nugget * w[:pts.shape[0]]
    assert np.allclose(ev, aw, rtol=1e-10, atol=1e-10)
