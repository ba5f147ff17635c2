"""The allocation-free direct-sum entry point (pgpu_direct_evaluate_noalloc) against the regular
evaluator entry point with exact direct sums, on two calls in a row.

That entry point is for callers whose device memory belongs to their own allocator and budget,
so the library may not allocate on their behalf; it keeps its partial sums in a fixed device
array compiled into the library. This file is collected last so that a failure here cannot hide
the results of the other tests; it also passes when run alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

import polatory_gb300 as pg
from polatory_gb300 import _lib

pytestmark = pytest.mark.gpu


def _inputs(seed, ns, nt):
    g = np.random.Generator(np.random.PCG64(seed))
    return g.random((ns, 3)), g.standard_normal(ns), g.random((nt, 3))


def _regular(rbf, src, w, trg):
    ev = pg.FmmEvaluator(rbf, [0, 0, 0, 1, 1, 1], precision=pg.PLAIN)
    ev.configure(backend=1)  # exact direct sums
    ev.set_source_points(src)
    ev.set_target_points(trg)
    ev.set_weights(w)
    return ev.evaluate()


def _noalloc(rbf, src, w, trg):
    import torch

    dev = torch.device("cuda", 0)
    s = torch.from_numpy(np.ascontiguousarray(src)).to(dev)
    ww = torch.from_numpy(np.ascontiguousarray(w)).to(dev)
    t = torch.from_numpy(np.ascontiguousarray(trg)).to(dev)
    out = torch.empty(trg.shape[0], dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    r = rbf._c()
    rc = _lib.lib.pgpu_direct_evaluate_noalloc(C.byref(r), C.c_void_p(s.data_ptr()), src.shape[0],
                                               C.c_void_p(ww.data_ptr()), C.c_void_p(t.data_ptr()),
                                               trg.shape[0], C.c_void_p(out.data_ptr()), None)
    _lib.check(rc)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("cls,params", [(pg.Biharmonic3D, [1.0]), (pg.CovExponential, [1.0, 0.4])],
                         ids=["bh3", "exp"])
def test_noalloc_matches_regular_entry_point_twice(cls, params):
    rbf = cls(params)
    rbf.anisotropy = np.diag([1.0, 1.0, 2.0])
    for call, (ns, nt) in enumerate([(3000, 700), (5000, 1300)]):
        src, w, trg = _inputs(100 + call, ns, nt)
        want = _regular(rbf, src, w, trg)
        got = _noalloc(rbf, src, w, trg)
        scale = np.abs(w).sum() * max(1.0, np.abs(want).max())
        assert np.max(np.abs(got - want)) <= 1e-12 * scale, call


def test_noalloc_ragged_and_edge_sizes():
    """Target counts that split unevenly over the source chunks, a call at the 2,097,152-target
    limit (one chunk, the whole array in use) and a call without sources (all zeros)."""
    rbf = pg.Biharmonic3D([1.0])
    src, w, trg = _inputs(7, 100_003, 1_001)
    want = _regular(rbf, src, w, trg)
    got = _noalloc(rbf, src, w, trg)
    assert np.max(np.abs(got - want)) <= 1e-12 * np.abs(w).sum()
    src, w, trg = _inputs(8, 37, 1 << 21)
    want = _regular(rbf, src, w, trg)
    got = _noalloc(rbf, src, w, trg)
    assert np.max(np.abs(got - want)) <= 1e-12 * np.abs(w).sum()
    got = _noalloc(rbf, np.zeros((0, 3)), np.zeros(0), trg[:5000])
    assert np.all(got == 0.0)


def test_noalloc_rejects_oversized_calls():
    import torch

    dev = torch.device("cuda", 0)
    buf = torch.zeros(8, dtype=torch.float64, device=dev)
    r = pg.Biharmonic3D([1.0])._c()
    p = C.c_void_p(buf.data_ptr())
    rc = _lib.lib.pgpu_direct_evaluate_noalloc(C.byref(r), p, 1, p, p, (1 << 21) + 1, p, None)
    assert rc == _lib.PGPU_INVALID_ARGUMENT
    assert "too many targets" in _lib.lib.pgpu_last_error().decode()
    # Host pointers are refused as well (nothing is copied).
    h = np.zeros(9)
    rc = _lib.lib.pgpu_direct_evaluate_noalloc(C.byref(r), C.c_void_p(h.ctypes.data), 3,
                                               C.c_void_p(h.ctypes.data), C.c_void_p(h.ctypes.data),
                                               3, C.c_void_p(h.ctypes.data), None)
    assert rc == _lib.PGPU_INVALID_ARGUMENT
