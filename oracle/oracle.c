/*
 * oracle.c — TEST INFRASTRUCTURE ONLY. A plain-C, FP64 restatement of the reference's exact
 * (non-FMM) arithmetic on the fit/evaluate path, used by tests/, __graft_entry__.smoke() and
 * bench.py's CPU baseline as the checker. Nothing in the product links or calls it.
 *
 * Parity status: the reference (polatory/polatory) cannot be built here (Eigen, ScalFMM3 and its
 * other dependencies are absent) and ships no golden vectors for this path, so this restatement
 * is pinned only against the reference's own invariant tests (test/rbf/test_rbf.cpp:
 * central-difference gradients/Hessians, the anisotropy identity; test/interpolation/
 * test_fitter.cpp: the residual criterion). Outputs of the reference itself: parity unpinned.
 *
 * Followed files (paths inside polatory/polatory):
 *   kernels        include/polatory/rbf/{polyharmonic_odd,polyharmonic_even,cov_*}.hpp
 *   anisotropy     include/polatory/rbf/rbf_base.hpp:40-53
 *   direct sums    include/polatory/interpolation/direct_evaluator.hpp:38-88
 *   operator       include/polatory/interpolation/direct_operator.hpp:31-85
 *   monomials      include/polatory/polynomial/monomial_basis.hpp:171-247
 *   saddle system  the linear system whose solution FGMRES approaches
 *                  (interpolation/solver.hpp:94-141 with operator.hpp:56-82)
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "polatory_gpu.h"

#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- isotropic kernels (value, gradient vector, Hessian matrix) ------------------------ */

static double ipow(double x, int n) {
  double r = 1.0;
  for (int i = 0; i < n; ++i) r *= x;
  return r;
}

/* x^(n/2) for odd n (rbf_base.hpp:125-147). */
static double sqrt_pow(double x, int n) { return ipow(x, n / 2) * sqrt(x); }

static double norm3(const double* v) { return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }

static void outer_hess(double coeff, double f, const double* d, double* h) {
  /* coeff * (I + f * d^T d) */
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) h[3 * i + j] = coeff * ((i == j ? 1.0 : 0.0) + f * d[i] * d[j]);
}

typedef struct {
  double rho0, a, b, c, d, e;
  int n; /* imq exponent: value 1/(1+c rho^2)^(n/2) */
} spheroidal_t;

static spheroidal_t spheroidal(int kind) {
  spheroidal_t s;
  switch (kind) {
    case PGPU_RBF_SP3:
      s = (spheroidal_t){0.18657871684006438, 2.009875543958482, 0.8734640537108553,
                         7.181510581693163, 18.81837403335934, 0.1392464703107397, 3};
      break;
    case PGPU_RBF_SP5:
      s = (spheroidal_t){0.2580127411803573, 1.6149073288415876, 0.8575980168032007,
                         2.5036086535164204, 10.735449080535068, 0.39942344766841226, 5};
      break;
    case PGPU_RBF_SP7:
      s = (spheroidal_t){0.2944149476843637, 1.4859979204216045, 0.8494862533016855,
                         1.44208314742683, 8.57520866899984, 0.6934412913598931, 7};
      break;
    default:
      s = (spheroidal_t){0.31622776601683794, 1.4230249470757708, 0.8445585690332554, 1.0,
                         7.601027121299299, 1.0, 9};
      break;
  }
  return s;
}

static void cauchy(int kind, double* ka, int* n) {
  switch (kind) {
    case PGPU_RBF_GC3: *ka = 7.0; *n = 3; break;
    case PGPU_RBF_GC5: *ka = 2.4822022531844965; *n = 5; break;
    case PGPU_RBF_GC7: *ka = 1.438027308408951; *n = 7; break;
    default: *ka = 1.0; *n = 9; break;
  }
}

/* Returns -1 when the Hessian is requested for a kernel without one (cub, sph). */
int orc_rbf_isotropic(int kind, const double* p, const double* d, double* val, double* grad,
                      double* hess) {
  const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  double coeff = 0.0; /* gradient = coeff * d */
  double hf = 0.0;    /* Hessian = coeff * (I + hf * d d^T) unless set otherwise */
  int has_hess = 1;
  if (kind == PGPU_RBF_BH3 || kind == PGPU_RBF_TH3) {
    /* PolyharmonicOdd<K> (polyharmonic_odd.hpp:21-67), kSign = -1 for K=1, +1 for K=3 */
    const int K = kind == PGPU_RBF_BH3 ? 1 : 3;
    const double sign = (((K + 1) / 2) % 2 == 0) ? 1.0 : -1.0;
    const double slope = p[0], c = p[1];
    const double rho2 = r2 + c * c, rho = sqrt(rho2);
    if (val) *val = sign * slope * ipow(rho, K);
    if (rho == 0.0) {
      coeff = 0.0;
      hf = 0.0;
    } else {
      coeff = sign * K * slope * (K == 1 ? 1.0 / rho : rho);
      hf = (K - 2) / rho2;
    }
  } else if (kind == PGPU_RBF_BH2 || kind == PGPU_RBF_TH2) {
    /* PolyharmonicEven<K> (polyharmonic_even.hpp:22-73), kSign = +1 for K=2, -1 for K=4 */
    const int K = kind == PGPU_RBF_BH2 ? 2 : 4;
    const double sign = ((K / 2 + 1) % 2 == 0) ? 1.0 : -1.0;
    const double slope = p[0], c = p[1];
    const double rho2 = r2 + c * c, rho = sqrt(rho2);
    if (rho == 0.0) {
      if (val) *val = 0.0;
      coeff = 0.0;
      hf = 0.0;
    } else {
      if (val) *val = sign * slope * ipow(rho, K) * log(rho);
      coeff = sign * slope * ipow(rho, K - 2) * (1.0 + K * log(rho));
      hf = (K - 2.0 + K / (1.0 + K * log(rho))) / rho2;
    }
  } else {
    const double psill = p[0], range = p[1];
    const double r = sqrt(r2), rho = r / range;
    switch (kind) {
      case PGPU_RBF_CUB: { /* cov_cubic.hpp:33-53 */
        const double rho2 = rho * rho;
        if (val)
          *val = r < range ? psill * (1.0 + rho2 * (-7.0 + rho * (8.75 + rho2 * (-3.5 + 0.75 * rho2))))
                           : 0.0;
        coeff = r < range ? psill * (-14.0 + rho * (26.25 + rho2 * (-17.5 + 5.25 * rho2))) / (range * range)
                          : 0.0;
        has_hess = 0;
        break;
      }
      case PGPU_RBF_EXP: /* cov_exponential.hpp:33-61 */
        if (val) *val = psill * exp(-3.0 * rho);
        coeff = -3.0 * psill * exp(-3.0 * rho) / (range * r);
        hf = -(1.0 / (r * r) + 3.0 / (range * r));
        break;
      case PGPU_RBF_GAU: /* cov_gaussian.hpp:33-61 */
        if (val) *val = psill * exp(-3.0 * rho * rho);
        coeff = -6.0 * psill * exp(-3.0 * rho * rho) / (range * range);
        hf = -6.0 / (range * range);
        break;
      case PGPU_RBF_GC3:
      case PGPU_RBF_GC5:
      case PGPU_RBF_GC7:
      case PGPU_RBF_GC9: { /* cov_generalized_cauchy*.hpp */
        double ka;
        int n;
        cauchy(kind, &ka, &n);
        const double q = 1.0 + ka * rho * rho;
        if (val) *val = psill / sqrt_pow(q, n);
        coeff = -ka * n * psill / (sqrt_pow(q, n + 2) * range * range);
        hf = -ka * (n + 2) / (ka * r * r + range * range);
        break;
      }
      case PGPU_RBF_SPH: /* cov_spherical.hpp:33-53 */
        if (val) *val = r < range ? psill * (1.0 + rho * (-1.5 + 0.5 * rho * rho)) : 0.0;
        coeff = r < range ? psill * (-1.5 / rho + 1.5 * rho) / (range * range) : 0.0;
        has_hess = 0;
        break;
      default: { /* cov_spheroidal*.hpp, full kind */
        spheroidal_t s = spheroidal(kind);
        if (rho < s.rho0) {
          if (val) *val = psill * (1.0 - s.a * rho);
          coeff = -psill * s.a / (r * range);
          hf = -1.0 / (r * r);
        } else {
          const double q = 1.0 + s.c * rho * rho;
          if (val) *val = psill * s.b / sqrt_pow(q, s.n);
          coeff = -psill * s.d / (sqrt_pow(q, s.n + 2) * range * range);
          hf = -(double)(s.n + 2) / (r * r + s.e * range * range);
        }
        break;
      }
    }
  }
  if (grad)
    for (int k = 0; k < 3; ++k) grad[k] = coeff * d[k];
  if (hess) {
    if (!has_hess) return -1;
    outer_hess(coeff, hf, d, hess);
  }
  return 0;
}

/* Anisotropic evaluation (rbf_base.hpp:40-53): value phi(A d), gradient grad(A d) A,
 * Hessian A^T H(A d) A. */
int orc_rbf_evaluate(int kind, const double* params, const double* a, const double* diff,
                     double* val, double* grad, double* hess) {
  double t[3];
  for (int r = 0; r < 3; ++r) t[r] = a[3 * r] * diff[0] + a[3 * r + 1] * diff[1] + a[3 * r + 2] * diff[2];
  double g[3], h[9];
  int rc = orc_rbf_isotropic(kind, params, t, val, grad ? g : NULL, hess ? h : NULL);
  if (grad)
    for (int k = 0; k < 3; ++k) grad[k] = g[0] * a[k] + g[1] * a[3 + k] + g[2] * a[6 + k];
  if (rc) return rc; /* no Hessian for this kernel */
  if (hess)
    for (int p = 0; p < 3; ++p)
      for (int q = 0; q < 3; ++q) {
        double s = 0;
        for (int u = 0; u < 3; ++u)
          for (int v = 0; v < 3; ++v) s += a[3 * u + p] * h[3 * u + v] * a[3 * v + q];
        hess[3 * p + q] = s;
      }
  return 0;
}

/* ---- polynomial --------------------------------------------------------------------- */

int orc_poly_basis_size(int degree) {
  if (degree < 0) return 0;
  int k = degree + 1;
  return k * (k + 1) * (k + 2) / 6;
}

/* Monomial basis rows: value rows for points, then 3 rows (d/dx, d/dy, d/dz) per grad point.
 * out is row-major (mu + 3 sigma) x l. */
void orc_monomial_basis(int degree, const double* pts, int64_t mu, const double* gpts,
                        int64_t sigma, double* out) {
  const int l = orc_poly_basis_size(degree);
  for (int64_t i = 0; i < mu; ++i) {
    const double* p = pts + 3 * i;
    double m[10] = {1.0, p[0], p[1], p[2], p[0] * p[0], p[0] * p[1], p[0] * p[2], p[1] * p[1],
                    p[1] * p[2], p[2] * p[2]};
    for (int k = 0; k < l; ++k) out[i * l + k] = m[k];
  }
  for (int64_t i = 0; i < sigma; ++i) {
    const double* p = gpts + 3 * i;
    double gx[10] = {0, 1, 0, 0, 2 * p[0], p[1], p[2], 0, 0, 0};
    double gy[10] = {0, 0, 1, 0, 0, p[0], 0, 2 * p[1], p[2], 0};
    double gz[10] = {0, 0, 0, 1, 0, 0, p[0], 0, p[1], 2 * p[2]};
    for (int k = 0; k < l; ++k) {
      out[(mu + 3 * i) * l + k] = gx[k];
      out[(mu + 3 * i + 1) * l + k] = gy[k];
      out[(mu + 3 * i + 2) * l + k] = gz[k];
    }
  }
}

/* ---- direct evaluator (direct_evaluator.hpp:38-88) ----------------------------------- */

/* out[trg_mu + 3 trg_sigma] = sum over RBFs of the four blocks + polynomial. */
int orc_direct_evaluate(const pgpu_model* model, const double* src, int64_t mu, const double* gsrc,
                        int64_t sigma, const double* weights, const double* trg, int64_t tm,
                        const double* gtrg, int64_t tmg, double* out) {
  const int l = orc_poly_basis_size(model->poly_degree);
  const int64_t nout = tm + 3 * tmg;
  memset(out, 0, sizeof(double) * nout);
  for (int r = 0; r < model->n_rbfs; ++r) {
    const pgpu_rbf* rb = &model->rbfs[r];
    int err = 0;
#pragma omp parallel for schedule(static) reduction(| : err)
    for (int64_t i = 0; i < tm; ++i) {
      double s = 0.0;
      for (int64_t j = 0; j < mu; ++j) {
        double d[3] = {trg[3 * i] - src[3 * j], trg[3 * i + 1] - src[3 * j + 1],
                       trg[3 * i + 2] - src[3 * j + 2]};
        double v;
        orc_rbf_evaluate(rb->kind, rb->params, rb->aniso, d, &v, NULL, NULL);
        s += weights[j] * v;
      }
      for (int64_t j = 0; j < sigma; ++j) {
        double d[3] = {trg[3 * i] - gsrc[3 * j], trg[3 * i + 1] - gsrc[3 * j + 1],
                       trg[3 * i + 2] - gsrc[3 * j + 2]};
        double g[3];
        orc_rbf_evaluate(rb->kind, rb->params, rb->aniso, d, NULL, g, NULL);
        const double* gw = weights + mu + 3 * j;
        s += -(gw[0] * g[0] + gw[1] * g[1] + gw[2] * g[2]);
      }
      out[i] += s;
    }
#pragma omp parallel for schedule(static) reduction(| : err)
    for (int64_t i = 0; i < tmg; ++i) {
      double s[3] = {0, 0, 0};
      for (int64_t j = 0; j < mu; ++j) {
        double d[3] = {gtrg[3 * i] - src[3 * j], gtrg[3 * i + 1] - src[3 * j + 1],
                       gtrg[3 * i + 2] - src[3 * j + 2]};
        double g[3];
        orc_rbf_evaluate(rb->kind, rb->params, rb->aniso, d, NULL, g, NULL);
        for (int k = 0; k < 3; ++k) s[k] += weights[j] * g[k];
      }
      for (int64_t j = 0; j < sigma; ++j) {
        double d[3] = {gtrg[3 * i] - gsrc[3 * j], gtrg[3 * i + 1] - gsrc[3 * j + 1],
                       gtrg[3 * i + 2] - gsrc[3 * j + 2]};
        double h[9];
        if (orc_rbf_evaluate(rb->kind, rb->params, rb->aniso, d, NULL, NULL, h)) err |= 1;
        const double* gw = weights + mu + 3 * j;
        /* (grad_w * -H)^T */
        for (int k = 0; k < 3; ++k) s[k] += -(gw[0] * h[k] + gw[1] * h[3 + k] + gw[2] * h[6 + k]);
      }
      for (int k = 0; k < 3; ++k) out[tm + 3 * i + k] += s[k];
    }
    if (err) return -1;
  }
  if (l > 0) {
    const double* c = weights + mu + 3 * sigma;
    double* p = (double*)malloc(sizeof(double) * (nout > 0 ? nout : 1) * l);
    orc_monomial_basis(model->poly_degree, trg, tm, gtrg, tmg, p);
    for (int64_t i = 0; i < nout; ++i) {
      double s = 0;
      for (int k = 0; k < l; ++k) s += p[i * l + k] * c[k];
      out[i] += s;
    }
    free(p);
  }
  return 0;
}

/* ---- direct operator (direct_operator.hpp:31-85) --------------------------------------- */

int orc_direct_operator(const pgpu_model* model, const double* pts, int64_t mu,
                        const double* gpts, int64_t sigma, const double* w, double* y) {
  const int l = orc_poly_basis_size(model->poly_degree);
  const int64_t n = mu + 3 * sigma;
  /* kernel blocks without polynomial: evaluate with zero polynomial weights */
  double* wz = (double*)malloc(sizeof(double) * (n + l + 1));
  memcpy(wz, w, sizeof(double) * n);
  for (int k = 0; k < l; ++k) wz[n + k] = 0.0;
  pgpu_model m0 = *model;
  m0.poly_degree = -1;
  int rc = orc_direct_evaluate(&m0, pts, mu, gpts, sigma, wz, pts, mu, gpts, sigma, y);
  free(wz);
  if (rc) return rc;
  for (int64_t i = 0; i < mu; ++i) y[i] += model->nugget * w[i];
  if (l > 0) {
    double* p = (double*)malloc(sizeof(double) * (n > 0 ? n : 1) * l);
    orc_monomial_basis(model->poly_degree, pts, mu, gpts, sigma, p);
    for (int64_t i = 0; i < n; ++i) {
      double s = 0;
      for (int k = 0; k < l; ++k) s += p[i * l + k] * w[n + k];
      y[i] += s;
    }
    for (int k = 0; k < l; ++k) {
      double s = 0;
      for (int64_t i = 0; i < n; ++i) s += p[i * l + k] * w[i];
      y[n + k] = s;
    }
    free(p);
  }
  return 0;
}

/* ---- exact fit: the saddle-point system [A + nugget I, P; P^T, 0] --------------------- */

/* LU with partial pivoting, in place on an n x n row-major matrix; solves for b. Right-looking
 * and blocked (panels of LU_NB columns): the panel is factored column by column with row
 * swaps across the whole matrix, the block row of U is solved with the panel's unit lower
 * triangle, and the trailing matrix takes one rank-LU_NB update, register-tiled 4 rows x 8
 * columns and spread over the host threads by row blocks. The arithmetic is the textbook
 * algorithm (Golub & Van Loan, Alg. 3.4.2 with the block update of section 3.2.10). */
#define LU_NB 64
static int lu_solve(double* a, int64_t n, double* b) {
  for (int64_t k0 = 0; k0 < n; k0 += LU_NB) {
    const int64_t kb = n - k0 < LU_NB ? n - k0 : LU_NB;
    const int64_t k1 = k0 + kb;
    for (int64_t k = k0; k < k1; ++k) {
      int64_t p = k;
      double best = fabs(a[k * n + k]);
      for (int64_t i = k + 1; i < n; ++i)
        if (fabs(a[i * n + k]) > best) {
          best = fabs(a[i * n + k]);
          p = i;
        }
      if (best == 0.0) return -1;
      if (p != k) {
        double* rk = a + k * n;
        double* rp = a + p * n;
        for (int64_t j = 0; j < n; ++j) {
          double t = rk[j];
          rk[j] = rp[j];
          rp[j] = t;
        }
        double t = b[k];
        b[k] = b[p];
        b[p] = t;
      }
      const double inv = 1.0 / a[k * n + k];
      /* Column k below the pivot, and the rest of the panel (columns k+1 .. k1-1). */
#pragma omp parallel for schedule(static) if (n - k > 4096)
      for (int64_t i = k + 1; i < n; ++i) {
        double* ri = a + i * n;
        const double f = ri[k] * inv;
        ri[k] = f;
        if (f != 0.0)
          for (int64_t j = k + 1; j < k1; ++j) ri[j] -= f * a[k * n + j];
      }
    }
    if (k1 >= n) break;
    /* U12 = L11^{-1} A12 (unit lower L11), by column chunks. */
#pragma omp parallel for schedule(static)
    for (int64_t j0 = k1; j0 < n; j0 += 256) {
      const int64_t j1 = j0 + 256 < n ? j0 + 256 : n;
      for (int64_t k = k0; k < k1; ++k)
        for (int64_t i = k + 1; i < k1; ++i) {
          const double f = a[i * n + k];
          if (f != 0.0)
            for (int64_t j = j0; j < j1; ++j) a[i * n + j] -= f * a[k * n + j];
        }
    }
    /* A22 -= L21 U12 over 4-row blocks; 8-column register tiles. */
    const int64_t nrb = (n - k1 + 3) / 4;
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t rb = 0; rb < nrb; ++rb) {
      const int64_t i0 = k1 + 4 * rb;
      const int64_t ni = n - i0 < 4 ? n - i0 : 4;
      double lrow[4][LU_NB];
      for (int r = 0; r < 4; ++r)
        for (int64_t k = 0; k < kb; ++k) lrow[r][k] = r < ni ? a[(i0 + r) * n + k0 + k] : 0.0;
      int64_t j = k1;
      for (; j + 8 <= n; j += 8) {
        double acc[4][8];
        for (int r = 0; r < 4; ++r)
          for (int c = 0; c < 8; ++c) acc[r][c] = r < ni ? a[(i0 + r) * n + j + c] : 0.0;
        for (int64_t k = 0; k < kb; ++k) {
          const double* u = a + (k0 + k) * n + j;
          for (int r = 0; r < 4; ++r) {
            const double f = lrow[r][k];
            for (int c = 0; c < 8; ++c) acc[r][c] -= f * u[c];
          }
        }
        for (int r = 0; r < ni; ++r)
          for (int c = 0; c < 8; ++c) a[(i0 + r) * n + j + c] = acc[r][c];
      }
      for (; j < n; ++j)
        for (int r = 0; r < ni; ++r) {
          double s = a[(i0 + r) * n + j];
          for (int64_t k = 0; k < kb; ++k) s -= lrow[r][k] * a[(k0 + k) * n + j];
          a[(i0 + r) * n + j] = s;
        }
    }
  }
  /* Forward (unit L) and backward (U) substitution. */
  for (int64_t i = 1; i < n; ++i) {
    double s = b[i];
    for (int64_t j = 0; j < i; ++j) s -= a[i * n + j] * b[j];
    b[i] = s;
  }
  for (int64_t i = n - 1; i >= 0; --i) {
    double s = b[i];
    for (int64_t j = i + 1; j < n; ++j) s -= a[i * n + j] * b[j];
    b[i] = s / a[i * n + i];
  }
  return 0;
}

/* weights_out (mu + 3 sigma + l): the exact solution of the fit system. */
int orc_fit_exact(const pgpu_model* model, const double* pts, int64_t mu, const double* gpts,
                  int64_t sigma, const double* values, double* weights_out) {
  const int l = orc_poly_basis_size(model->poly_degree);
  const int64_t n = mu + 3 * sigma, m = n + l;
  double* a = (double*)calloc(m * m, sizeof(double));
  if (!a) return -2;
  /* Kernel blocks as mat_a (preconditioner/mat_a.hpp:10-61): A (value-value, nugget on the
   * diagonal), -grad (value-gradient), -Hessian (gradient-gradient), mirrored. */
  int err = 0;
  for (int r = 0; r < model->n_rbfs; ++r) {
    const pgpu_rbf* rb = &model->rbfs[r];
#pragma omp parallel for schedule(dynamic, 16) reduction(| : err)
    for (int64_t i = 0; i < n; ++i) {
      const int gi = i >= mu;
      const int64_t pi = gi ? (i - mu) / 3 : i;
      const int ci = gi ? (int)((i - mu) % 3) : 0;
      const double* xi = gi ? gpts + 3 * pi : pts + 3 * pi;
      for (int64_t j = 0; j < n; ++j) {
        const int gj = j >= mu;
        const int64_t pj = gj ? (j - mu) / 3 : j;
        const int cj = gj ? (int)((j - mu) % 3) : 0;
        const double* xj = gj ? gpts + 3 * pj : pts + 3 * pj;
        double d[3] = {xi[0] - xj[0], xi[1] - xj[1], xi[2] - xj[2]};
        double v = 0, g[3], h[9];
        if (!gi && !gj) {
          orc_rbf_evaluate(rb->kind, rb->params, rb->aniso, d, &v, NULL, NULL);
        } else if (!gi && gj) {
          orc_rbf_evaluate(rb->kind, rb->params, rb->aniso, d, NULL, g, NULL);
          v = -g[cj];
        } else if (gi && !gj) {
          orc_rbf_evaluate(rb->kind, rb->params, rb->aniso, d, NULL, g, NULL);
          v = g[ci];
        } else {
          if (orc_rbf_evaluate(rb->kind, rb->params, rb->aniso, d, NULL, NULL, h)) err |= 1;
          v = -h[3 * ci + cj];
        }
        a[i * m + j] += v;
      }
    }
  }
  if (err) {
    free(a);
    return -1;
  }
  for (int64_t i = 0; i < mu; ++i) a[i * m + i] += model->nugget;
  if (l > 0) {
    double* p = (double*)malloc(sizeof(double) * (n > 0 ? n : 1) * l);
    orc_monomial_basis(model->poly_degree, pts, mu, gpts, sigma, p);
    for (int64_t i = 0; i < n; ++i)
      for (int k = 0; k < l; ++k) {
        a[i * m + n + k] = p[i * l + k];
        a[(n + k) * m + i] = p[i * l + k];
      }
    free(p);
  }
  for (int64_t i = 0; i < n; ++i) weights_out[i] = values[i];
  for (int64_t k = 0; k < l; ++k) weights_out[n + k] = 0.0;
  int rc = lu_solve(a, m, weights_out);
  free(a);
  return rc;
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
