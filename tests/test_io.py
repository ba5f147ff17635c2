"""Interpolant save/load in the reference's binary format (common/io.hpp:31-187 with
Write<Interpolant> at interpolant.hpp:345-367, Write<Model> at model.hpp:304-320, rbf/rbf_io.hpp,
geometry/bbox3d.hpp:82-96). The expected bytes are restated here field by field."""
import struct

import numpy as np
import pytest

import polatory_gb300 as pg


def expected_bytes(names, params, anisos, poly_degree, nugget, fitted, centers, bbox, weights):
    b = struct.pack("<Q", len(names))
    for name, p, a in zip(names, params, anisos):
        b += struct.pack("<Q", len(name)) + name.encode()
        b += struct.pack("<Q", len(p)) + struct.pack(f"<{len(p)}d", *p)
        b += struct.pack("<9d", *np.asarray(a, dtype=np.float64).reshape(9))  # row-major Mat3
    b += struct.pack("<i", poly_degree) + struct.pack("<d", nugget)
    b += struct.pack("<?", fitted)
    c = np.asarray(centers, dtype=np.float64).reshape(-1, 3)
    b += struct.pack("<q", c.shape[0]) + c.tobytes()          # centers (row-major Points)
    b += struct.pack("<q", 0)                                 # grad_centers
    b += struct.pack("<3d", *bbox[:3]) + struct.pack("<3d", *bbox[3:])
    w = np.asarray(weights, dtype=np.float64)
    b += struct.pack("<q", w.shape[0]) + w.tobytes()
    return b


def test_unfitted_interpolant_bytes(tmp_path):
    rbf = pg.CovExponential([1.5, 0.3])
    a = np.array([[1.2, 0.1, 0.0], [0.0, 0.9, 0.2], [0.0, 0.0, 1.1]])
    rbf.anisotropy = a
    model = pg.Model([rbf, pg.Biharmonic3D([2.0])], 1)
    model.nugget = 0.25
    it = pg.Interpolant(model)
    f = tmp_path / "unfitted.bin"
    it.save(f)
    inf = float("inf")
    want = expected_bytes(["exp", "bh3"], [[1.5, 0.3], [2.0, 0.0]], [a, np.eye(3)], 1, 0.25,
                          False, np.zeros((0, 3)), [inf, inf, inf, -inf, -inf, -inf], [])
    assert f.read_bytes() == want


def test_load_rejects_bad_files(tmp_path):
    with pytest.raises(pg.PolatoryError, match="cannot open file"):
        pg.Interpolant.load(tmp_path / "missing.bin")
    bad = tmp_path / "bad.bin"
    bad.write_bytes(struct.pack("<Q", 1) + struct.pack("<Q", 3) + b"xyz")
    with pytest.raises(pg.PolatoryError, match="unknown RBF"):
        pg.Interpolant.load(bad)
    short = tmp_path / "short.bin"
    short.write_bytes(struct.pack("<Q", 1))
    with pytest.raises(pg.PolatoryError, match="unexpected end"):
        pg.Interpolant.load(short)


@pytest.mark.gpu
def test_fitted_round_trip(tmp_path):
    g = np.random.Generator(np.random.PCG64(61))
    pts = g.random((2000, 3))
    vals = np.sin(3 * pts[:, 0]) + pts[:, 1] * pts[:, 2]
    model = pg.Model(pg.Biharmonic3D([1.0]), 1)
    it = pg.Interpolant(model)
    it.fit(pts, vals, 1e-6)
    f = tmp_path / "fitted.bin"
    it.save(f)
    lo, hi = pts.min(0), pts.max(0)
    want = expected_bytes(["bh3"], [[1.0, 0.0]], [np.eye(3)], 1, 0.0, True, pts,
                          list(lo) + list(hi), it.weights)
    assert f.read_bytes() == want
    back = pg.Interpolant.load(f)
    q = g.random((500, 3))
    np.testing.assert_array_equal(back.weights, it.weights)
    np.testing.assert_array_equal(back.evaluate(q), it.evaluate(q))
