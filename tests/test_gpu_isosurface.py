"""The isosurface field function on the device (isosurface/rbf_field_function.hpp:21-27): the
values at lattice nodes of the reference's body-centred cubic lattice
(isosurface/rmt/primitive_lattice.hpp:19-43, positions (lc_origin + lc) * resolution * basis)
minus the isovalue, formed from the integer lattice coordinates on the device, equal the
interpolant's evaluate_impl at the same positions, and the oracle's exact sums within the
evaluation accuracy."""
import numpy as np
import pytest

import oracle
import polatory_gb300 as pg

pytestmark = pytest.mark.gpu

# Rows: the lattice vectors of the body-centred cubic lattice (primitive_lattice.hpp:19-26).
BCC = np.array([[1 / np.sqrt(3), np.sqrt(2 / 3), 0.0],
                [-1 / np.sqrt(3), 0.0, np.sqrt(2 / 3)],
                [1 / np.sqrt(3), -np.sqrt(2 / 3), 0.0]])


def sphere_sdf(n, seed):
    g = np.random.Generator(np.random.PCG64(seed))
    u = g.standard_normal((n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    pts = np.concatenate([0.5 * u, 0.52 * u, 0.48 * u])
    vals = np.concatenate([np.zeros(n), np.full(n, 0.02), np.full(n, -0.02)])
    return pts, vals


@pytest.mark.parametrize("precision", [pg.PLAIN, pg.MIXED], ids=["plain", "mixed"])
def test_lattice_field_values(precision):
    pts, vals = sphere_sdf(4000, 61)
    model = pg.Model(pg.Biharmonic3D([1.0]), 1)
    it = pg.Interpolant(model, precision)
    it.fit(pts, vals, 1e-5)
    resolution = 0.04
    basis = resolution * BCC
    lc_origin = np.array([0.25, -0.5, 0.125])
    r = np.arange(-20, 21)
    lcs = np.stack(np.meshgrid(r, r, r, indexing="ij"), axis=-1).reshape(-1, 3).astype(np.int32)
    pos = (lc_origin + lcs) @ basis
    isovalue = 0.01
    it.set_evaluation_bbox(pos.min(0), pos.max(0), accuracy=1e-9)
    got = it.evaluate_lattice(lc_origin, basis, lcs, isovalue)
    want = it.evaluate_impl(pos) - isovalue
    assert got.shape == (lcs.shape[0],)
    assert np.max(np.abs(got - want)) <= 1e-12
    g = np.random.Generator(np.random.PCG64(62))
    sub = g.choice(lcs.shape[0], 1500, replace=False)
    exact = oracle.direct_evaluate(model, pts, it.weights, pos[sub]) - isovalue
    assert np.max(np.abs(got[sub] - exact)) <= 1e-8
    # Lattice coordinates already on the device are taken as they are.
    import torch

    d = torch.from_numpy(lcs).to("cuda")
    out = np.empty(lcs.shape[0])
    from polatory_gb300 import _lib
    import ctypes as C

    _lib.check(_lib.lib.pgpu_interpolant_evaluate_lattice(
        it._h, _lib.ptr(np.ascontiguousarray(lc_origin)), _lib.ptr(np.ascontiguousarray(basis.reshape(9))),
        C.c_void_p(d.data_ptr()), lcs.shape[0], isovalue, _lib.ptr(out)))
    assert np.array_equal(out, got)
