"""Python host API of the GB300 RBF fit/evaluate library.

Mirrors the reference's Python binding (python/python_binding.cpp:33-137): rbf classes taking a
parameter list, Model(rbf, poly_degree), Interpolant(model).fit/evaluate. Every call goes through
the C ABI of libpolatory_gpu.so (include/polatory_gpu.h); there is no CPU code path.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from ._lib import PolatoryError, as_points, check, lib, ptr

__all__ = [
    "Rbf", "Biharmonic2D", "Biharmonic3D", "CovCubic", "CovExponential", "CovGaussian",
    "CovGeneralizedCauchy3", "CovGeneralizedCauchy5", "CovGeneralizedCauchy7",
    "CovGeneralizedCauchy9", "CovSpherical", "CovSpheroidal3", "CovSpheroidal5",
    "CovSpheroidal7", "CovSpheroidal9", "Triharmonic2D", "Triharmonic3D", "Model", "Interpolant",
    "FmmEvaluator", "PolatoryError", "make_rbf", "PLAIN", "MIXED", "fit_batch", "Server",
]

PLAIN = _lib.PRECISION_PLAIN
MIXED = _lib.PRECISION_MIXED
INF = math.inf


class Rbf:
    """rbf::Rbf<3> (include/polatory/rbf/rbf.hpp:11-118)."""

    short_name = ""
    _kind = -1
    _polyharmonic = False

    def __init__(self, params=()):
        params = [float(p) for p in params]
        if self._polyharmonic:
            # PolyharmonicOdd/Even::set_parameters: {} -> {1, 0}; {s} -> {s, 0}.
            if len(params) == 0:
                params = [1.0, 0.0]
            elif len(params) == 1:
                params = [params[0], 0.0]
        if len(params) != 2:
            raise ValueError("params.size() must be 2")
        self._params = params
        self._aniso = np.eye(3)

    @property
    def parameters(self):
        return list(self._params)

    @parameters.setter
    def parameters(self, p):
        self.__init__(p)

    @property
    def anisotropy(self):
        return self._aniso.copy()

    @anisotropy.setter
    def anisotropy(self, a):
        a = np.asarray(a, dtype=np.float64).reshape(3, 3)
        if not np.linalg.det(a) > 0.0:
            raise ValueError("aniso must have a positive determinant")
        self._aniso = a.copy()

    @property
    def num_parameters(self):
        return 2

    def _c(self) -> _lib.PgpuRbf:
        r = _lib.PgpuRbf()
        r.kind = self._kind
        r.params[0], r.params[1] = self._params
        for i, v in enumerate(self._aniso.reshape(-1)):
            r.aniso[i] = float(v)
        return r

    @property
    def cpd_order(self) -> int:
        out = C.c_int()
        check(lib.pgpu_rbf_cpd_order(C.byref(self._c()), C.byref(out)))
        return out.value

    @property
    def is_covariance_function(self) -> bool:
        return self.cpd_order == 0

    def support_radius_isotropic(self) -> float:
        out = C.c_double()
        check(lib.pgpu_rbf_support_radius_isotropic(C.byref(self._c()), C.byref(out)))
        return out.value

    def _eval(self, diff, want):
        d = np.ascontiguousarray(np.asarray(diff, dtype=np.float64).reshape(-1, 3))
        n = d.shape[0]
        v = np.empty(n) if want == "v" else None
        g = np.empty((n, 3)) if want == "g" else None
        h = np.empty((n, 3, 3)) if want == "h" else None
        check(lib.pgpu_rbf_evaluate(C.byref(self._c()), ptr(d), n, ptr(v), ptr(g), ptr(h)))
        return {"v": v, "g": g, "h": h}[want]

    def evaluate(self, diff):
        out = self._eval(diff, "v")
        return float(out[0]) if np.asarray(diff).ndim == 1 else out

    def evaluate_gradient(self, diff):
        out = self._eval(diff, "g")
        return out[0] if np.asarray(diff).ndim == 1 else out

    def evaluate_hessian(self, diff):
        out = self._eval(diff, "h")
        return out[0] if np.asarray(diff).ndim == 1 else out


def _make(name, kind, polyharmonic):
    return type(name, (Rbf,), {"short_name": _lib.RBF_KINDS[kind], "_kind": kind,
                               "_polyharmonic": polyharmonic})


Biharmonic2D = _make("Biharmonic2D", 0, True)
Biharmonic3D = _make("Biharmonic3D", 1, True)
CovCubic = _make("CovCubic", 2, False)
CovExponential = _make("CovExponential", 3, False)
CovGaussian = _make("CovGaussian", 4, False)
CovGeneralizedCauchy3 = _make("CovGeneralizedCauchy3", 5, False)
CovGeneralizedCauchy5 = _make("CovGeneralizedCauchy5", 6, False)
CovGeneralizedCauchy7 = _make("CovGeneralizedCauchy7", 7, False)
CovGeneralizedCauchy9 = _make("CovGeneralizedCauchy9", 8, False)
CovSpherical = _make("CovSpherical", 9, False)
CovSpheroidal3 = _make("CovSpheroidal3", 10, False)
CovSpheroidal5 = _make("CovSpheroidal5", 11, False)
CovSpheroidal7 = _make("CovSpheroidal7", 12, False)
CovSpheroidal9 = _make("CovSpheroidal9", 13, False)
Triharmonic2D = _make("Triharmonic2D", 14, True)
Triharmonic3D = _make("Triharmonic3D", 15, True)

_BY_NAME = {c.short_name: c for c in [
    Biharmonic2D, Biharmonic3D, CovCubic, CovExponential, CovGaussian, CovGeneralizedCauchy3,
    CovGeneralizedCauchy5, CovGeneralizedCauchy7, CovGeneralizedCauchy9, CovSpherical,
    CovSpheroidal3, CovSpheroidal5, CovSpheroidal7, CovSpheroidal9, Triharmonic2D,
    Triharmonic3D]}


def make_rbf(name: str, params) -> Rbf:
    """rbf::make_rbf (include/polatory/rbf/make_rbf.hpp:24-50)."""
    if name not in _BY_NAME:
        raise RuntimeError(f"unknown RBF name: '{name}'")
    return _BY_NAME[name](params)


class Model:
    """Model<3> (include/polatory/model.hpp:23-183)."""

    MIN_REQUIRED_POLY_DEGREE = -2

    def __init__(self, rbf, poly_degree: int = MIN_REQUIRED_POLY_DEGREE):
        rbfs = list(rbf) if isinstance(rbf, (list, tuple)) else [rbf]
        if not rbfs:
            raise ValueError("rbfs must not be empty")
        self.rbfs = rbfs
        self._nugget = 0.0
        m = self._c(poly_degree)
        check(lib.pgpu_model_validate(C.byref(m)))
        min_deg = self.cpd_order - 1
        self.poly_degree = min_deg if poly_degree == self.MIN_REQUIRED_POLY_DEGREE else poly_degree

    @property
    def cpd_order(self) -> int:
        return max(r.cpd_order for r in self.rbfs)

    @property
    def nugget(self) -> float:
        return self._nugget

    @nugget.setter
    def nugget(self, v: float):
        if not v >= 0.0:
            raise ValueError("nugget must be non-negative")
        self._nugget = float(v)

    def set_nugget(self, v: float):
        self.nugget = v

    @property
    def poly_basis_size(self) -> int:
        d = self.poly_degree
        return 0 if d < 0 else (d + 1) * (d + 2) * (d + 3) // 6

    def _c(self, poly_degree=None) -> _lib.PgpuModel:
        m = _lib.PgpuModel()
        m.n_rbfs = len(self.rbfs)
        m.poly_degree = self.poly_degree if poly_degree is None else poly_degree
        m.nugget = self._nugget
        for i, r in enumerate(self.rbfs):
            m.rbfs[i] = r._c()
        return m


class Interpolant:
    """Interpolant<3> (include/polatory/interpolant.hpp:54-218) on the GPU library."""

    def __init__(self, model: Model, precision: int = PLAIN):
        self.model = model
        self._h = C.c_void_p()
        check(lib.pgpu_interpolant_create(C.byref(model._c()), C.byref(self._h)))
        check(lib.pgpu_interpolant_set_precision(self._h, precision))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.pgpu_interpolant_destroy(h)
            self._h = None

    def set_precision(self, precision: int):
        check(lib.pgpu_interpolant_set_precision(self._h, precision))

    def fit_incrementally(self, points, values, tolerance, max_iter=100, accuracy=INF):
        """Interpolant::fit_incrementally: the centres become the subset of the points the
        incremental fitter needed (incremental_fitter.hpp:46-183)."""
        pts = as_points(points)
        vals = np.ascontiguousarray(np.asarray(values, dtype=np.float64).reshape(-1))
        check(lib.pgpu_interpolant_fit_incrementally(
            self._h, ptr(pts), pts.shape[0], None, 0, ptr(vals), float(tolerance), INF,
            int(max_iter), float(accuracy), INF))

    def fit_inequality(self, points, values, values_lb, values_ub, tolerance, max_iter=100,
                       accuracy=INF):
        """Interpolant::fit_inequality: NaN marks an absent value or bound
        (inequality_fitter.hpp:43-187)."""
        pts = as_points(points)
        arrs = [np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1))
                for a in (values, values_lb, values_ub)]
        check(lib.pgpu_interpolant_fit_inequality(
            self._h, ptr(pts), pts.shape[0], ptr(arrs[0]), ptr(arrs[1]), ptr(arrs[2]),
            float(tolerance), int(max_iter), float(accuracy)))

    def save(self, filename: str) -> None:
        """Interpolant::save: the reference's binary format."""
        check(lib.pgpu_interpolant_save(self._h, str(filename).encode()))

    @classmethod
    def load(cls, filename: str, precision: int = PLAIN) -> "Interpolant":
        """Interpolant::load: reads the reference's binary format (model, centers, weights)."""
        obj = cls.__new__(cls)
        obj.model = None
        obj._h = C.c_void_p()
        check(lib.pgpu_interpolant_load(str(filename).encode(), C.byref(obj._h)))
        check(lib.pgpu_interpolant_set_precision(obj._h, precision))
        return obj

    def fit(self, points, values, tolerance, max_iter=100, accuracy=INF, initial=None, *,
            grad_points=None, grad_tolerance=INF, grad_accuracy=INF):
        pts = as_points(points)
        gpts = as_points(np.zeros((0, 3)) if grad_points is None else grad_points)
        vals = np.ascontiguousarray(np.asarray(values, dtype=np.float64).reshape(-1))
        n_rhs = pts.shape[0] + 3 * gpts.shape[0]
        if vals.shape[0] != n_rhs:
            # interpolant.hpp:88-91 (the C ABI takes a pointer and cannot check the length).
            raise PolatoryError(_lib.PGPU_INVALID_ARGUMENT, f"values.rows() must be equal to {n_rhs}")
        check(lib.pgpu_interpolant_fit(
            self._h, ptr(pts), pts.shape[0], ptr(gpts) if gpts.shape[0] else None, gpts.shape[0],
            ptr(vals), float(tolerance), float(grad_tolerance), int(max_iter), float(accuracy),
            float(grad_accuracy), initial._h if initial is not None else None))

    def evaluate(self, points, accuracy=INF, *, grad_points=None, grad_accuracy=INF):
        pts = as_points(points)
        gpts = as_points(np.zeros((0, 3)) if grad_points is None else grad_points)
        out = np.empty(pts.shape[0] + 3 * gpts.shape[0])
        check(lib.pgpu_interpolant_evaluate(
            self._h, ptr(pts), pts.shape[0], ptr(gpts) if gpts.shape[0] else None, gpts.shape[0],
            float(accuracy), float(grad_accuracy), ptr(out)))
        return out

    def fit_device(self, points, values, tolerance, max_iter=100, accuracy=INF):
        """fit() with device-resident inputs (torch CUDA float64 tensors, (n, 3) and (n,))."""
        n = int(points.shape[0])
        check(lib.pgpu_interpolant_fit(self._h, ptr(points), n, None, 0, ptr(values),
                                       float(tolerance), INF, int(max_iter), float(accuracy), INF,
                                       None))

    def evaluate_device(self, points, out, accuracy=INF):
        """evaluate() from device-resident points into a device-resident output tensor."""
        m = int(points.shape[0])
        check(lib.pgpu_interpolant_evaluate(self._h, ptr(points), m, None, 0, float(accuracy),
                                            INF, ptr(out)))

    def evaluate_impl(self, points, grad_points=None):
        pts = as_points(points)
        gpts = as_points(np.zeros((0, 3)) if grad_points is None else grad_points)
        out = np.empty(pts.shape[0] + 3 * gpts.shape[0])
        check(lib.pgpu_interpolant_evaluate_impl(
            self._h, ptr(pts), pts.shape[0], ptr(gpts) if gpts.shape[0] else None, gpts.shape[0],
            ptr(out)))
        return out

    def evaluate_lattice(self, lc_origin, basis, lattice_coordinates, isovalue=0.0):
        """isosurface::RbfFieldFunction over lattice nodes: value - isovalue at the positions
        (lc_origin + lc) @ basis of the integer lattice coordinates (n x 3), formed on the device
        (isosurface/rmt/primitive_lattice.hpp:41-43); uses the evaluation bbox of the last
        set_evaluation_bbox / evaluate, like evaluate_impl."""
        o = np.ascontiguousarray(np.asarray(lc_origin, dtype=np.float64).reshape(3))
        b = np.ascontiguousarray(np.asarray(basis, dtype=np.float64).reshape(9))
        lcs = np.ascontiguousarray(np.asarray(lattice_coordinates, dtype=np.int32).reshape(-1, 3))
        out = np.empty(lcs.shape[0])
        check(lib.pgpu_interpolant_evaluate_lattice(self._h, ptr(o), ptr(b),
                                                    C.c_void_p(lcs.ctypes.data), lcs.shape[0],
                                                    float(isovalue), ptr(out)))
        return out

    def set_evaluation_bbox(self, bbox_min, bbox_max, accuracy=INF, grad_accuracy=INF):
        """Interpolant::set_evaluation_bbox_impl (interpolant.hpp:201-210)."""
        b = np.ascontiguousarray(np.concatenate([np.asarray(bbox_min, dtype=np.float64).reshape(3),
                                                 np.asarray(bbox_max, dtype=np.float64).reshape(3)]))
        check(lib.pgpu_interpolant_set_evaluation_bbox(self._h, ptr(b), accuracy, grad_accuracy))

    @property
    def weights(self) -> np.ndarray:
        n = C.c_int64()
        check(lib.pgpu_interpolant_num_weights(self._h, C.byref(n)))
        out = np.empty(n.value)
        check(lib.pgpu_interpolant_weights(self._h, ptr(out), n.value))
        return out

    @property
    def centers(self) -> np.ndarray:
        mu, sg = C.c_int64(), C.c_int64()
        check(lib.pgpu_interpolant_num_centers(self._h, C.byref(mu), C.byref(sg)))
        c = np.empty((mu.value, 3))
        check(lib.pgpu_interpolant_centers(self._h, ptr(c), None))
        return c

    @property
    def bbox(self):
        b = np.empty(6)
        check(lib.pgpu_interpolant_bbox(self._h, ptr(b)))
        return b[:3].copy(), b[3:].copy()

    @property
    def fit_stats(self) -> dict:
        s = _lib.PgpuFitStats()
        check(lib.pgpu_interpolant_fit_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in s._fields_}


def fit_batch(model: Model, problems, tolerance, max_iter=100, precision=PLAIN, n_workers=0,
              return_weights=True):
    """Fits many independent problems with one model (pgpu_fit_batch).

    problems: list of (points, values) or (points, values, eval_points). Returns a list of dicts
    with 'weights', 'iterations', 'residual', 'status' and 'values' (the evaluation, if asked).
    """
    keep = []
    arr = (_lib.PgpuFitProblem * len(problems))()
    l = model.poly_basis_size
    for i, prob in enumerate(problems):
        pts = as_points(prob[0])
        vals = np.ascontiguousarray(np.asarray(prob[1], dtype=np.float64).reshape(-1))
        q = as_points(prob[2]) if len(prob) > 2 and prob[2] is not None else None
        w = np.empty(pts.shape[0] + l) if return_weights else None
        out = np.empty(q.shape[0]) if q is not None else None
        keep.append((pts, vals, q, w, out))
        p = arr[i]
        p.points = pts.ctypes.data
        p.n = pts.shape[0]
        p.values = vals.ctypes.data
        p.tolerance = float(tolerance)
        p.max_iter = int(max_iter)
        p.eval_points = q.ctypes.data if q is not None else None
        p.m = q.shape[0] if q is not None else 0
        p.eval_out = out.ctypes.data if out is not None else None
        p.weights_out = w.ctypes.data if w is not None else None
    rc = lib.pgpu_fit_batch(C.byref(model._c()), precision, arr, len(problems), n_workers)
    res = []
    for i, (pts, vals, q, w, out) in enumerate(keep):
        res.append({"weights": w, "iterations": arr[i].iterations, "residual": arr[i].residual,
                    "status": arr[i].status, "values": out})
    if rc != 0:
        msg = lib.pgpu_last_error().decode()
        err = PolatoryError(rc, msg)
        err.results = res
        raise err
    return res


class Server:
    """Serving loop (pgpu_server_*): fit and evaluate requests admitted under a device-memory
    budget, run concurrently on worker streams; fitted models stay resident in numbered slots.

    submit_fit / submit_evaluate return a ticket; wait(ticket) and poll(ticket) (None while
    running) return (status, latency_seconds, result, message) where result is the evaluation
    (None for a fit) and message the error text of a failed request.
    """

    def __init__(self, n_workers: int = 8, hbm_budget_bytes: int = 0):
        h = C.c_void_p()
        check(lib.pgpu_server_create(int(n_workers), int(hbm_budget_bytes), C.byref(h)))
        self._h = h
        self._keep = {}

    def close(self):
        if self._h:
            check(lib.pgpu_server_destroy(self._h))
            self._h = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _submit(self, req, keep):
        t = C.c_int64()
        check(lib.pgpu_server_submit(self._h, C.byref(req), C.byref(t)))
        self._keep[t.value] = keep
        return t.value

    @staticmethod
    def estimate_bytes(kind: int, n: int, precision: int = PLAIN) -> int:
        r = _lib.PgpuRequest()
        r.kind, r.n, r.precision = kind, n, precision
        return lib.pgpu_server_estimate_bytes(C.byref(r))

    def submit_fit(self, slot: int, model: Model, points, values, tolerance, max_iter=100,
                   precision=PLAIN) -> int:
        pts = as_points(points)
        vals = np.ascontiguousarray(np.asarray(values, dtype=np.float64).reshape(-1))
        m = model._c()
        r = _lib.PgpuRequest()
        r.kind, r.slot, r.model = _lib.REQUEST_FIT, slot, C.addressof(m)
        r.points, r.n, r.values = pts.ctypes.data, pts.shape[0], vals.ctypes.data
        r.tolerance, r.max_iter, r.precision = float(tolerance), int(max_iter), precision
        return self._submit(r, (pts, vals, None))

    def submit_evaluate(self, slot: int, points, precision=PLAIN) -> int:
        pts = as_points(points)
        out = np.empty(pts.shape[0])
        r = _lib.PgpuRequest()
        r.kind, r.slot = _lib.REQUEST_EVALUATE, slot
        r.points, r.n, r.out, r.precision = pts.ctypes.data, pts.shape[0], out.ctypes.data, precision
        return self._submit(r, (pts, None, out))

    def poll(self, ticket: int):
        done, st, lat = C.c_int(), C.c_int(), C.c_double()
        check(lib.pgpu_server_poll(self._h, ticket, C.byref(done), C.byref(st), C.byref(lat)))
        if not done.value:
            return None
        return self._result(ticket, st.value, lat.value)

    def wait(self, ticket: int):
        st, lat = C.c_int(), C.c_double()
        check(lib.pgpu_server_wait(self._h, ticket, C.byref(st), C.byref(lat)))
        return self._result(ticket, st.value, lat.value)

    def _result(self, ticket, status, latency):
        keep = self._keep.pop(ticket)
        msg = lib.pgpu_last_error().decode() if status != 0 else ""
        return status, latency, keep[2], msg

    def stats(self) -> dict:
        o = _lib.PgpuServerStats()
        check(lib.pgpu_server_stats_get(self._h, C.byref(o)))
        return {k: getattr(o, k) for k, _ in o._fields_}


def profile_enable(on: bool = True) -> None:
    check(lib.pgpu_profile_enable(int(on)))


def profile_reset() -> None:
    check(lib.pgpu_profile_reset())


def profile_report() -> dict:
    import json

    buf = C.create_string_buffer(1 << 16)
    check(lib.pgpu_profile_report(buf, len(buf)))
    return json.loads(buf.value.decode())


def launch_count() -> int:
    out = C.c_int64()
    check(lib.pgpu_launch_count(C.byref(out)))
    return out.value


def synchronize() -> None:
    check(lib.pgpu_synchronize())


def operator_cache_stats() -> dict:
    """Bytes and entries of the process-wide far-field operator cache, and its byte limit."""
    b, e, lim = C.c_int64(), C.c_int64(), C.c_int64()
    check(lib.pgpu_operator_cache_stats(C.byref(b), C.byref(e), C.byref(lim)))
    return {"bytes": b.value, "entries": e.value, "limit": lim.value}


def set_operator_cache_limit(nbytes: int) -> None:
    """Sets the far-field operator cache's byte limit and evicts down to it."""
    check(lib.pgpu_operator_cache_limit(int(nbytes)))


def stream_handle() -> int:
    """The library's cudaStream_t of this thread, as an integer handle."""
    out = C.c_void_p()
    check(lib.pgpu_stream(C.byref(out)))
    return int(out.value or 0)


class FmmEvaluator:
    """fmm::FmmGenericEvaluatorBase<3> (include/polatory/fmm/fmm_evaluator.hpp:17-41)."""

    def __init__(self, rbf: Rbf, bbox, kernel=_lib.KERNEL_VALUE, symmetric=False, precision=PLAIN):
        b = np.ascontiguousarray(np.asarray(bbox, dtype=np.float64).reshape(6))
        self._h = C.c_void_p()
        self._rbf = rbf._c()
        check(lib.pgpu_evaluator_create(C.byref(self._rbf), kernel, int(symmetric), ptr(b),
                                        precision, C.byref(self._h)))
        self._n_trg = 0
        # Outputs per target: 3 for the gradient-transpose and Hessian kernels.
        self._kn = 3 if kernel in (_lib.KERNEL_GRADIENT_TRANSPOSE, _lib.KERNEL_HESSIAN) else 1

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.pgpu_evaluator_destroy(h)
            self._h = None

    def configure(self, backend: int = 0, order: int = 0, leaf_level: int = -1):
        """backend 0 auto, 1 direct, 2 FMM; order 4/6/8 (0 = from accuracy); leaf_level -1 auto."""
        check(lib.pgpu_evaluator_configure(self._h, backend, order, leaf_level))

    def set_accuracy(self, acc: float):
        check(lib.pgpu_evaluator_set_accuracy(self._h, float(acc)))

    def set_source_points(self, pts):
        p = as_points(pts)
        check(lib.pgpu_evaluator_set_source_points(self._h, ptr(p), p.shape[0]))

    def set_target_points(self, pts):
        p = as_points(pts)
        self._n_trg = p.shape[0]
        check(lib.pgpu_evaluator_set_target_points(self._h, ptr(p), p.shape[0]))

    def set_points(self, pts):
        p = as_points(pts)
        self._n_trg = p.shape[0]
        check(lib.pgpu_evaluator_set_points(self._h, ptr(p), p.shape[0]))

    def set_weights(self, w):
        w = np.ascontiguousarray(np.asarray(w, dtype=np.float64).reshape(-1))
        check(lib.pgpu_evaluator_set_weights(self._h, ptr(w), w.shape[0]))

    def evaluate(self) -> np.ndarray:
        n = self._kn * self._n_trg
        out = np.empty(n)
        check(lib.pgpu_evaluator_evaluate(self._h, ptr(out), n))
        return out
