"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of oracle/_build/liboracle.so, the FP64 C restatement
of the reference's exact arithmetic (see oracle.c for the followed files and the parity status).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, as the checker.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .build import OUT, build

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not OUT.exists():
            build()
        l = C.CDLL(str(OUT))
        P, I64 = C.c_void_p, C.c_int64
        l.orc_rbf_evaluate.argtypes = [C.c_int, P, P, P, P, P, P]
        l.orc_rbf_evaluate.restype = C.c_int
        l.orc_rbf_isotropic.argtypes = [C.c_int, P, P, P, P, P]
        l.orc_rbf_isotropic.restype = C.c_int
        l.orc_direct_evaluate.argtypes = [P, P, I64, P, I64, P, P, I64, P, I64, P]
        l.orc_direct_evaluate.restype = C.c_int
        l.orc_direct_operator.argtypes = [P, P, I64, P, I64, P, P]
        l.orc_direct_operator.restype = C.c_int
        l.orc_fit_exact.argtypes = [P, P, I64, P, I64, P, P]
        l.orc_fit_exact.restype = C.c_int
        l.orc_monomial_basis.argtypes = [C.c_int, P, I64, P, I64, P]
        l.orc_monomial_basis.restype = None
        l.orc_poly_basis_size.argtypes = [C.c_int]
        l.orc_poly_basis_size.restype = C.c_int
        l.orc_num_threads.restype = C.c_int
        _lib = l
    return _lib


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return C.c_void_p(a.ctypes.data)


def _arr(a, shape_last=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    if shape_last is not None:
        a = a.reshape(-1, shape_last)
    return a


def rbf_evaluate(kind: int, params, aniso, diff):
    """(value, gradient, hessian-or-None) of the anisotropic kernel at one difference vector."""
    pr = _arr(params)
    a = _arr(aniso).reshape(9)
    d = _arr(diff).reshape(3)
    v = np.zeros(1)
    g = np.zeros(3)
    h = np.zeros(9)
    rc = lib().orc_rbf_evaluate(kind, _p(pr), _p(a), _p(d), _p(v), _p(g), _p(h))
    return float(v[0]), g, (h.reshape(3, 3) if rc == 0 else None)


def rbf_isotropic(kind: int, params, diff):
    pr = _arr(params)
    d = _arr(diff).reshape(3)
    v = np.zeros(1)
    g = np.zeros(3)
    h = np.zeros(9)
    rc = lib().orc_rbf_isotropic(kind, _p(pr), _p(d), _p(v), _p(g), _p(h))
    return float(v[0]), g, (h.reshape(3, 3) if rc == 0 else None)


RBF_KINDS = ["bh2", "bh3", "cub", "exp", "gau", "gc3", "gc5", "gc7", "gc9", "sph", "sp3", "sp5",
             "sp7", "sp9", "th2", "th3"]


class Rbf(C.Structure):
    """pgpu_rbf of include/polatory_gpu.h (declared here so that the oracle needs no product
    library)."""
    _fields_ = [("kind", C.c_int32), ("reserved", C.c_int32), ("params", C.c_double * 2),
                ("aniso", C.c_double * 9)]


class Model(C.Structure):
    """pgpu_model of include/polatory_gpu.h."""
    _fields_ = [("n_rbfs", C.c_int32), ("poly_degree", C.c_int32), ("nugget", C.c_double),
                ("rbfs", Rbf * 4)]


def model(kind: str, params, poly_degree: int, nugget: float = 0.0, aniso=None) -> Model:
    """A one-RBF model struct: kind is the reference's short name ("bh3", "exp", ...), params
    the RBF's parameters (scale, or psill and range), aniso the 3x3 anisotropy (identity)."""
    m = Model()
    m.n_rbfs = 1
    m.poly_degree = poly_degree
    m.nugget = nugget
    r = m.rbfs[0]
    r.kind = RBF_KINDS.index(kind)
    p = list(params) + [0.0] * (2 - len(params))
    r.params[0], r.params[1] = p[0], p[1]
    a = np.eye(3) if aniso is None else np.asarray(aniso, dtype=np.float64).reshape(3, 3)
    for k in range(9):
        r.aniso[k] = a.reshape(9)[k]
    return m


def _model(model):
    """Accepts a polatory_gb300.Model (uses its C struct) or a ready ctypes struct."""
    return model._c() if hasattr(model, "_c") else model


def direct_evaluate(model, src, weights, trg, gsrc=None, gtrg=None):
    m = _model(model)
    src = _arr(src, 3)
    trg = _arr(trg, 3)
    gsrc = _arr(np.zeros((0, 3)) if gsrc is None else gsrc, 3)
    gtrg = _arr(np.zeros((0, 3)) if gtrg is None else gtrg, 3)
    w = _arr(weights).reshape(-1)
    out = np.zeros(trg.shape[0] + 3 * gtrg.shape[0])
    rc = lib().orc_direct_evaluate(C.byref(m), _p(src), src.shape[0], _p(gsrc), gsrc.shape[0],
                                   _p(w), _p(trg), trg.shape[0], _p(gtrg), gtrg.shape[0], _p(out))
    if rc:
        raise RuntimeError("oracle direct evaluation failed")
    return out


def direct_operator(model, pts, w, gpts=None):
    m = _model(model)
    pts = _arr(pts, 3)
    gpts = _arr(np.zeros((0, 3)) if gpts is None else gpts, 3)
    w = _arr(w).reshape(-1)
    out = np.zeros_like(w)
    rc = lib().orc_direct_operator(C.byref(m), _p(pts), pts.shape[0], _p(gpts), gpts.shape[0],
                                   _p(w), _p(out))
    if rc:
        raise RuntimeError("oracle operator failed")
    return out


def fit_exact(model, pts, values, gpts=None):
    m = _model(model)
    pts = _arr(pts, 3)
    gpts = _arr(np.zeros((0, 3)) if gpts is None else gpts, 3)
    vals = _arr(values).reshape(-1)
    l = lib().orc_poly_basis_size(m.poly_degree)
    out = np.zeros(vals.shape[0] + l)
    rc = lib().orc_fit_exact(C.byref(m), _p(pts), pts.shape[0], _p(gpts), gpts.shape[0], _p(vals),
                             _p(out))
    if rc:
        raise RuntimeError("oracle exact fit failed")
    return out


def monomial_basis(degree: int, pts, gpts=None):
    pts = _arr(pts, 3)
    gpts = _arr(np.zeros((0, 3)) if gpts is None else gpts, 3)
    l = lib().orc_poly_basis_size(degree)
    out = np.zeros((pts.shape[0] + 3 * gpts.shape[0], l))
    lib().orc_monomial_basis(degree, _p(pts), pts.shape[0], _p(gpts), gpts.shape[0], _p(out))
    return out


def num_threads() -> int:
    return lib().orc_num_threads()
