"""Seeded synthetic workloads (numpy PCG64) for the benchmark configurations.

No public dataset exists for these configurations; every input is generated here from a seed.
  c1: uniform cube fit, biharmonic, 64^3 evaluation grid
  c2: ellipsoid surface + off-surface SDF points, uniform evaluation points in the bbox
  c3: Gaussian-mixture points with a random-Fourier-feature exponential-covariance field
  c4: many independent uneven-size fits
"""
from __future__ import annotations

import numpy as np


def rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def f_c1(p: np.ndarray) -> np.ndarray:
    """f = sin(2 pi x) cos(2 pi y) + z^2."""
    return np.sin(2 * np.pi * p[:, 0]) * np.cos(2 * np.pi * p[:, 1]) + p[:, 2] ** 2


def c1(n: int = 10_000, grid: int = 64, seed: int = 1):
    g = rng(seed)
    pts = g.random((n, 3))
    vals = f_c1(pts)
    t = np.arange(grid) / (grid - 1)
    gx, gy, gz = np.meshgrid(t, t, t, indexing="ij")
    q = np.stack([gx.ravel(), gy.ravel(), gz.ravel()], axis=1)
    return np.ascontiguousarray(pts), vals, np.ascontiguousarray(q)


def ellipsoid_surface(n: int, axes=(1.0, 0.7, 0.5), seed: int = 2):
    """Points uniform by area on an ellipsoid (rejection on the area element of the scaled
    sphere) with outward unit normals."""
    a = np.asarray(axes, dtype=np.float64)
    g = rng(seed)
    out = []
    nrm = []
    gmax = 1.0 / a.min()
    have = 0
    while have < n:
        m = int((n - have) * 1.6) + 1024
        u = g.standard_normal((m, 3))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        w = np.sqrt(((u / a) ** 2).sum(axis=1))  # area element / (abc)
        keep = g.random(m) * gmax < w
        p = u[keep] * a
        nn = p / a**2
        nn /= np.linalg.norm(nn, axis=1, keepdims=True)
        out.append(p)
        nrm.append(nn)
        have += p.shape[0]
    return np.concatenate(out)[:n], np.concatenate(nrm)[:n]


def c2(n_surface: int = 1_000_000, offset: float = 0.01, n_eval: int = 2_000_000, seed: int = 2):
    axes = (1.0, 0.7, 0.5)
    s, nn = ellipsoid_surface(n_surface, axes, seed)
    pts = np.concatenate([s, s + offset * nn, s - offset * nn])
    vals = np.concatenate([np.zeros(n_surface), np.full(n_surface, offset),
                           np.full(n_surface, -offset)])
    g = rng(seed + 1000)
    lo = -np.asarray(axes)
    q = lo + g.random((n_eval, 3)) * (2 * np.asarray(axes))
    return np.ascontiguousarray(pts), vals, np.ascontiguousarray(q)


def c3(n: int = 500_000, n_eval: int = 10_000_000, n_comp: int = 32, sigma: float = 0.03,
       n_features: int = 256, range_: float = 0.2, seed: int = 3):
    """Gaussian-mixture points; values = random Fourier features of exp(-3 |A d| / range) with
    A = diag(1, 1, 2) (multivariate Cauchy frequencies scaled by 3 / range in the A frame)."""
    g = rng(seed)
    centres = g.random((n_comp, 3))
    comp = g.integers(0, n_comp, n)
    pts = centres[comp] + sigma * g.standard_normal((n, 3))
    aniso = np.diag([1.0, 1.0, 2.0])
    # Student-t (nu = 1) frequencies: normal / sqrt(chi2_1)
    z = g.standard_normal((n_features, 3))
    chi = np.sqrt(g.chisquare(1.0, n_features))[:, None]
    omega = (3.0 / range_) * z / chi
    phase = g.random(n_features) * 2 * np.pi
    amp = np.sqrt(2.0 / n_features)

    def field(p):
        ap = p @ aniso.T
        return amp * np.cos(ap @ omega.T + phase).sum(axis=1)

    vals = field(pts)
    q = g.random((n_eval, 3))
    return np.ascontiguousarray(pts), vals, np.ascontiguousarray(q), aniso


def c4(n_fits: int = 4096, n_min: int = 200, n_max: int = 20_000, n_eval: int = 4096,
       seed: int = 4):
    g = rng(seed)
    sizes = np.round(np.exp(g.uniform(np.log(n_min), np.log(n_max), n_fits))).astype(np.int64)
    fits = []
    for n in sizes:
        p = g.random((int(n), 3))
        v = f_c1(p) + g.normal(0.0, 1e-4, int(n))
        q = g.random((n_eval, 3))
        fits.append((p, v, q))
    return fits
