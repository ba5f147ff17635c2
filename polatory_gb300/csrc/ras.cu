// Device part of the RAS preconditioner: batched assembly of Q^T A Q, batched blocked
// Cholesky (right-looking, 32x32 blocks, one launch per step for all domains of a level),
// batched fine/coarse solves with the inner-point scatter, and the multilevel sweep.
//
// Q^T A Q entries are formed without materialising A: with L_i the Lagrange-basis row of
// point i, u_i[k] = A(p_k, x_i) and v_i = A11 L_i (p_k the polynomial points),
//   (Q^T A Q)_ij = A(x_i, x_j) - u_i.L_j - L_i.u_j + L_i.v_j,
// which equals the four-block product of fine_grid.hpp:80-84 with q_top = -L^T.
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <mutex>
#include <thread>
#include <type_traits>

#include "kernels.cuh"
#include "linalg.hpp"
#include "profile.hpp"
#include "ras.hpp"
#include "ras_divide.hpp"
#include "tcgen05.cuh"

namespace pgpu {

namespace {

constexpr int NB = 32;
constexpr int kMaxL = 10;  // polynomial basis size at degree 2

template <class T>
__device__ __forceinline__ T rbf_value_rt(int kind, T r2, const KParams<T>& kp) {
  return dispatch_kind(kind, [&]<int K>() { return rbf_value<K>(r2, kp); });
}

struct RbfSet {
  int n;
  int kind[PGPU_MAX_RBFS];
  double p0[PGPU_MAX_RBFS], p1[PGPU_MAX_RBFS];
  double a[PGPU_MAX_RBFS][9];
};

__device__ __forceinline__ double kernel_sum(const RbfSet& rs, const double* x, const double* y) {
  double s = 0;
  for (int r = 0; r < rs.n; ++r) {
    double d0 = x[0] - y[0], d1 = x[1] - y[1], d2 = x[2] - y[2];
    const double* a = rs.a[r];
    double t0 = a[0] * d0 + a[1] * d1 + a[2] * d2;
    double t1 = a[3] * d0 + a[4] * d1 + a[5] * d2;
    double t2 = a[6] * d0 + a[7] * d1 + a[8] * d2;
    KParams<double> kp{rs.p0[r], rs.p1[r]};
    s += rbf_value_rt<double>(rs.kind[r], t0 * t0 + t1 * t1 + t2 * t2, kp);
  }
  return s;
}

// ---- fits with gradient points -------------------------------------------------------------
// The system's rows are the value points (type -1) followed by three rows per gradient point
// (types 0-2: the derivative along x, y, z). Domains, level sets and the polynomial points are
// lists of rows.

// Monomial row (type -1) or its derivative along axis `type`, degree <= 2, in the column order
// of monomial_basis.hpp:171-247 (entries past the basis size are unused).
__host__ __device__ inline void poly_row(int type, double x, double y, double z, double* m) {
  if (type < 0) {
    const double v[10] = {1.0, x, y, z, x * x, x * y, x * z, y * y, y * z, z * z};
    for (int k = 0; k < 10; ++k) m[k] = v[k];
  } else if (type == 0) {
    const double v[10] = {0.0, 1.0, 0.0, 0.0, 2.0 * x, y, z, 0.0, 0.0, 0.0};
    for (int k = 0; k < 10; ++k) m[k] = v[k];
  } else if (type == 1) {
    const double v[10] = {0.0, 0.0, 1.0, 0.0, 0.0, x, 0.0, 2.0 * y, z, 0.0};
    for (int k = 0; k < 10; ++k) m[k] = v[k];
  } else {
    const double v[10] = {0.0, 0.0, 0.0, 1.0, 0.0, 0.0, x, 0.0, y, 2.0 * z};
    for (int k = 0; k < 10; ++k) m[k] = v[k];
  }
}

// Entry of A between two rows, summed over the RBFs, without the nugget (mat_a.hpp:10-61):
// value-value phi(A d); value-gradient -(A^T grad phi(A d))_j with d = x (value) - y (gradient
// point); gradient-gradient -(A^T H(A d) A)_ij with d = y_i - y_j. The gradient of phi at t is
// g(|t|^2) t and its Hessian ha I + hb t t^T (rbf_gcoef, rbf_hess).
__host__ __device__ inline double row_entry(const RbfSet& rs, int ta, const double* pa, int tb,
                                            const double* pb) {
  if (ta >= 0 && tb < 0) {
    const int tt = ta;
    ta = tb;
    tb = tt;
    const double* pp = pa;
    pa = pb;
    pb = pp;
  }
  const double d0 = pa[0] - pb[0], d1 = pa[1] - pb[1], d2 = pa[2] - pb[2];
  double s = 0;
  for (int r = 0; r < rs.n; ++r) {
    const double* a = rs.a[r];
    const double t0 = a[0] * d0 + a[1] * d1 + a[2] * d2;
    const double t1 = a[3] * d0 + a[4] * d1 + a[5] * d2;
    const double t2 = a[6] * d0 + a[7] * d1 + a[8] * d2;
    const double r2 = t0 * t0 + t1 * t1 + t2 * t2;
    KParams<double> kp{rs.p0[r], rs.p1[r]};
    if (ta < 0 && tb < 0) {
      s += dispatch_kind(rs.kind[r], [&]<int K>() { return rbf_value<K>(r2, kp); });
    } else if (ta < 0) {
      const double g = dispatch_kind(rs.kind[r], [&]<int K>() { return rbf_gcoef<K>(r2, kp); });
      s -= g * (a[tb] * t0 + a[3 + tb] * t1 + a[6 + tb] * t2);
    } else {
      double ha = 0, hb = 0;
      dispatch_kind(rs.kind[r], [&]<int K>() {
        rbf_hess<K>(r2, kp, ha, hb);
        return 0;
      });
      const double ata = a[ta] * a[tb] + a[3 + ta] * a[3 + tb] + a[6 + ta] * a[6 + tb];
      const double ua = a[ta] * t0 + a[3 + ta] * t1 + a[6 + ta] * t2;
      const double ub = a[tb] * t0 + a[3 + tb] * t1 + a[6 + tb] * t2;
      s -= ha * ata + hb * ua * ub;
    }
  }
  return s;
}

// Positions and types of the rows: the mu points, then each gradient point three times.
__global__ void rows_kernel(const double* __restrict__ pts, Index mu, const double* __restrict__ gpts,
                            Index sigma, double* __restrict__ pos, int* __restrict__ type) {
  const Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= mu + 3 * sigma) return;
  const double* p = i < mu ? pts + 3 * i : gpts + 3 * ((i - mu) / 3);
  pos[3 * i] = p[0];
  pos[3 * i + 1] = p[1];
  pos[3 * i + 2] = p[2];
  type[i] = i < mu ? -1 : static_cast<int>((i - mu) % 3);
}

// Lagrange rows of every row: the monomial (or derivative) row times the coefficients.
__global__ void lagrange_rows_kernel(int l, const double* __restrict__ pos, const int* __restrict__ type,
                                     Index rows, const double* __restrict__ coeffs,
                                     double* __restrict__ lag) {
  const Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= rows) return;
  double m[10];
  poly_row(type[i], pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], m);
  for (int c = 0; c < l; ++c) {
    double s = 0;
    for (int r = 0; r < l; ++r) s += m[r] * coeffs[r * l + c];
    lag[i * l + c] = s;
  }
}

// u_g[k] = A(poly row k, row g) and v_g = A11 L_g for every row g.
__global__ void uv_rows_kernel(RbfSet rs, const double* __restrict__ pos, const int* __restrict__ type,
                               Index rows, const double* __restrict__ poly_pos,
                               const int* __restrict__ poly_type, int l, const double* __restrict__ a11,
                               const double* __restrict__ lag, double* __restrict__ u,
                               double* __restrict__ v) {
  const Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= rows) return;
  for (int k = 0; k < l; ++k)
    u[i * l + k] = row_entry(rs, poly_type[k], poly_pos + 3 * k, type[i], pos + 3 * i);
  for (int k = 0; k < l; ++k) {
    double s = 0;
    for (int kk = 0; kk < l; ++kk) s += a11[k * l + kk] * lag[i * l + kk];
    v[i * l + k] = s;
  }
}

// u_i[k] = sum_r K_r(p_k - x_i), v_i = A11 L_i, per global point i.
__global__ void uv_kernel(RbfSet rs, const double* __restrict__ pts, Index mu,
                          const double* __restrict__ poly_pts, int l,
                          const double* __restrict__ a11, const double* __restrict__ lag,
                          double* __restrict__ u, double* __restrict__ v) {
  Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= mu) return;
  const double* x = pts + 3 * i;
  for (int k = 0; k < l; ++k) u[i * l + k] = kernel_sum(rs, poly_pts + 3 * k, x);
  for (int k = 0; k < l; ++k) {
    double s = 0;
    for (int kk = 0; kk < l; ++kk) s += a11[k * l + kk] * lag[i * l + kk];
    v[i * l + k] = s;
  }
}

// Lagrange rows: lag_i = monomials(x_i) * coeffs.
__global__ void lagrange_kernel(int degree, int l, const double* __restrict__ pts, Index mu,
                                const double* __restrict__ coeffs, double* __restrict__ lag) {
  Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= mu) return;
  const double x = pts[3 * i], y = pts[3 * i + 1], z = pts[3 * i + 2];
  double m[10] = {1, x, y, z, x * x, x * y, x * z, y * y, y * z, z * z};
  (void)degree;
  for (int c = 0; c < l; ++c) {
    double s = 0;
    for (int r = 0; r < l; ++r) s += m[r] * coeffs[r * l + c];
    lag[i * l + c] = s;
  }
}

// The points as the division of an anisotropic model sees them, A p, rounded like the host
// restatement: (a0 p0 + a1 p1) + a2 p2 per row of A.
__global__ void transform_points_kernel(const double* __restrict__ pts, Index n, Mat3 a,
                                        double* __restrict__ out) {
  const Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double p0 = pts[3 * i], p1 = pts[3 * i + 1], p2 = pts[3 * i + 2];
  for (int r = 0; r < 3; ++r)
    out[3 * i + r] = __dadd_rn(__dadd_rn(__dmul_rn(a.a[3 * r], p0), __dmul_rn(a.a[3 * r + 1], p1)),
                               __dmul_rn(a.a[3 * r + 2], p2));
}

template <class T>
__global__ void frame_kernel(const double* __restrict__ pts, Index n, Mat3 a, double ox, double oy,
                             double oz, P4<T>* __restrict__ out) {
  Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double tx, ty, tz;
  mat3_vec(a.a, pts[3 * i], pts[3 * i + 1], pts[3 * i + 2], tx, ty, tz);
  out[i] = P4<T>{static_cast<T>(tx - ox), static_cast<T>(ty - oy), static_cast<T>(tz - oz), T(0)};
}

__device__ __forceinline__ void tile_of(Index t, int& bi, int& bj) {
  // Lower-triangular tile enumeration: t = bi (bi + 1) / 2 + bj, bj <= bi.
  int b = static_cast<int>((sqrt(8.0 * static_cast<double>(t) + 1.0) - 1.0) * 0.5);
  while (static_cast<Index>(b + 1) * (b + 2) / 2 <= t) ++b;
  while (static_cast<Index>(b) * (b + 1) / 2 > t) --b;
  bi = b;
  bj = static_cast<int>(t - static_cast<Index>(b) * (b + 1) / 2);
}

// Assembles Q^T A Q (lower tiles) for all domains; padding rows/columns become identity.
template <class T, int KIND>
__global__ void assemble_kernel(KParams<T> kp, const P4<T>* __restrict__ frame,
                                const int* __restrict__ nsz, const int* __restrict__ lds,
                                const Index* __restrict__ mat_off, T* __restrict__ mats,
                                const Index* __restrict__ pt_off, const Index* __restrict__ pts,
                                int l, int first, int last, double nugget,
                                const double* __restrict__ lag, const double* __restrict__ u,
                                const double* __restrict__ v, int tiles_in_x) {
  // tiles_in_x: grid (tile, domain), so that the blocks running together are the tiles of a
  // few domains and their gathered point data stays in L2; otherwise grid (domain, tile).
  const Index d = tiles_in_x ? blockIdx.y : blockIdx.x;
  const int n = nsz[d], ld = lds[d];
  int bi, bj;
  tile_of(tiles_in_x ? blockIdx.x : blockIdx.y, bi, bj);
  if (bi * NB >= ld) return;
  T* m = mats + mat_off[d];
  const Index* dp = pts + pt_off[d] + l;  // non-polynomial points
  // The tile's 32 rows and 32 columns (positions, Lagrange values, u, v) staged once.
  // The polynomial correction runs in the matrix's type: FP32 matrices hold an FP32 kernel
  // value, so FP64 correction terms (at 1/64 of the FP32 rate) would add cost, not accuracy.
  __shared__ P4<T> s_xr[NB], s_xc[NB];
  __shared__ T s_lr[NB][kMaxL], s_ur[NB][kMaxL], s_lc[NB][kMaxL], s_uc[NB][kMaxL],
      s_vc[NB][kMaxL];
  const int t = threadIdx.x;
  if (t < NB) {
    const int r = bi * NB + t;
    if (r < n) {
      const Index g = dp[r];
      s_xr[t] = frame[g];
      if (last)
        for (int k = 0; k < l; ++k) {
          s_lr[t][k] = static_cast<T>(lag[g * l + k]);
          s_ur[t][k] = static_cast<T>(u[g * l + k]);
        }
    }
  } else if (t < 2 * NB) {
    const int c = bj * NB + (t - NB);
    if (c < n) {
      const Index g = dp[c];
      s_xc[t - NB] = frame[g];
      if (last)
        for (int k = 0; k < l; ++k) {
          s_lc[t - NB][k] = static_cast<T>(lag[g * l + k]);
          s_uc[t - NB][k] = static_cast<T>(u[g * l + k]);
          s_vc[t - NB][k] = static_cast<T>(v[g * l + k]);
        }
    }
  }
  __syncthreads();
  const int rr = t & 31;
  const int r = bi * NB + rr;  // lanes walk down a column (coalesced)
  for (int cc = t >> 5; cc < NB; cc += blockDim.x >> 5) {
    const int c = bj * NB + cc;
    T* dst = m + r + static_cast<Index>(c) * ld;
    if (r >= n || c >= n) {
      *dst = (r == c) ? T(1) : T(0);
      continue;
    }
    const P4<T> xr = s_xr[rr], xc = s_xc[cc];
    T dx = xr.x - xc.x, dy = xr.y - xc.y, dz = xr.z - xc.z;
    T val = rbf_value<KIND>(dx * dx + dy * dy + dz * dz, kp);
    T acc = first ? T(0) : *dst;
    acc += val;
    if (last) {
      if (r == c) acc += static_cast<T>(nugget);
      T corr = 0;
      for (int k = 0; k < l; ++k)
        corr += -s_ur[rr][k] * s_lc[cc][k] - s_lr[rr][k] * s_uc[cc][k] + s_lr[rr][k] * s_vc[cc][k];
      acc += corr;
    }
    *dst = acc;
  }
}

// Q^T A Q of every domain of a fit with gradient points (lower tiles, FP64 entries from
// row_entry, nugget on the value rows' diagonal), with the same correction terms as
// assemble_kernel; padding rows/columns become identity.
template <class T>
__global__ void assemble_rows_kernel(RbfSet rs, const double* __restrict__ pos,
                                     const int* __restrict__ type, const int* __restrict__ nsz,
                                     const int* __restrict__ lds, const Index* __restrict__ mat_off,
                                     T* __restrict__ mats, const Index* __restrict__ pt_off,
                                     const Index* __restrict__ pts, int l, double nugget,
                                     const double* __restrict__ lag, const double* __restrict__ u,
                                     const double* __restrict__ v, int tiles_in_x) {
  const Index d = tiles_in_x ? blockIdx.y : blockIdx.x;
  const int n = nsz[d], ld = lds[d];
  int bi, bj;
  tile_of(tiles_in_x ? blockIdx.x : blockIdx.y, bi, bj);
  if (bi * NB >= ld) return;
  T* m = mats + mat_off[d];
  const Index* dp = pts + pt_off[d] + l;
  const int rr = threadIdx.x & 31;
  const int r = bi * NB + rr;
  for (int cc = threadIdx.x >> 5; cc < NB; cc += blockDim.x >> 5) {
    const int c = bj * NB + cc;
    T* dst = m + r + static_cast<Index>(c) * ld;
    if (r >= n || c >= n) {
      *dst = (r == c) ? T(1) : T(0);
      continue;
    }
    const Index gr = dp[r], gc = dp[c];
    double acc = row_entry(rs, type[gr], pos + 3 * gr, type[gc], pos + 3 * gc);
    if (r == c && type[gr] < 0) acc += nugget;
    for (int k = 0; k < l; ++k)
      acc += -u[gr * l + k] * lag[gc * l + k] - lag[gr * l + k] * u[gc * l + k] +
             lag[gr * l + k] * v[gc * l + k];
    *dst = static_cast<T>(acc);
  }
}

template <class T>
__global__ void potrf_diag_kernel(int kb, const int* __restrict__ lds,
                                  const Index* __restrict__ mat_off, T* __restrict__ mats,
                                  int* __restrict__ info) {
  // 128 threads: lane = row of the 32 x 32 diagonal block, warp w updates the columns c = w
  // (mod 4), so the four sub-partitions share the trailing updates of each step (a single warp
  // would run them all through one sub-partition's FP64 pipe).
  const Index d = blockIdx.x;
  const int ld = lds[d];
  if (kb * NB >= ld) return;
  constexpr int kWarps = 4;
  __shared__ T a[NB][NB + 1];
  __shared__ T rpiv, floor_sh;
  T* m = mats + mat_off[d] + static_cast<Index>(kb * NB) * ld + kb * NB;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int c = w; c < NB; c += kWarps) a[lane][c] = m[lane + static_cast<Index>(c) * ld];
  __syncthreads();
  int modified = 0;
  // FP32 factors: pivots below 2^-20 of the block's largest diagonal entry are raised to it, so
  // that an ill-conditioned domain matrix gives a bounded (approximate) factor instead of one
  // that overflows.
  if (threadIdx.x == 0) {
    T floor_d = T(0);
    if constexpr (sizeof(T) == 4) {
      T dmax = T(0);
      for (int j = 0; j < NB; ++j) dmax = fmax(dmax, fabs(a[j][j]));
      floor_d = dmax * T(9.5367431640625e-07);
    }
    floor_sh = floor_d;
  }
  __syncthreads();
  const T floor_d = floor_sh;
  // The column below each pivot is scaled by the pivot's reciprocal, formed once: a division
  // per lane and column would cost a multi-instruction sequence each, and FP64 instructions
  // issue at 1/64 of the FP32 rate on this part.
  for (int j = 0; j < NB; ++j) {
    if (threadIdx.x == 0) {
      T dj = a[j][j];
      if (!(dj > floor_d)) {
        // Modified pivot (the matrix lost definiteness to rounding): the preconditioner only
        // needs an approximate factor, so continue with |d| (or 1 when d vanished), at least
        // the floor above.
        dj = fabs(dj) > T(0) ? T(fabs(dj)) : T(1);
        if (dj < floor_d) dj = floor_d;
        ++modified;
      }
      const T sj = sqrt(dj);
      a[j][j] = sj;
      rpiv = T(1) / sj;
    }
    __syncthreads();
    if (w == 0 && lane > j) a[lane][j] *= rpiv;
    __syncthreads();
    if (lane > j) {
      const T lj = a[lane][j];
      for (int c = j + 1 + ((w - j - 1) % kWarps + kWarps) % kWarps; c <= lane; c += kWarps)
        a[lane][c] -= lj * a[c][j];
    }
    __syncthreads();
  }
  for (int c = w; c < NB; c += kWarps) {
    m[lane + static_cast<Index>(c) * ld] = (lane >= c) ? a[lane][c] : T(0);
  }
  if (threadIdx.x == 0 && modified) atomicAdd(info + d, modified);
}

template <class T>
__global__ void trsm_panel_kernel(int kb, const int* __restrict__ lds,
                                  const Index* __restrict__ mat_off, T* __restrict__ mats) {
  const Index d = blockIdx.x;
  const int ld = lds[d];
  const int r = (kb + 1) * NB + blockIdx.y * blockDim.x + threadIdx.x;
  __shared__ T lkk[NB][NB + 1];
  __shared__ T rdiag[NB];  // reciprocals of the diagonal block's pivots
  if ((kb + 1) * NB + static_cast<int>(blockIdx.y * blockDim.x) >= ld) return;
  T* m = mats + mat_off[d];
  for (int e = threadIdx.x; e < NB * NB; e += blockDim.x) {
    int rr = e % NB, cc = e / NB;
    lkk[rr][cc] = m[(kb * NB + rr) + static_cast<Index>(kb * NB + cc) * ld];
  }
  __syncthreads();
  if (threadIdx.x < NB) rdiag[threadIdx.x] = T(1) / lkk[threadIdx.x][threadIdx.x];
  __syncthreads();
  if (r >= ld) return;
  T x[NB];
#pragma unroll
  for (int c = 0; c < NB; ++c) x[c] = m[r + static_cast<Index>(kb * NB + c) * ld];
#pragma unroll
  for (int c = 0; c < NB; ++c) {
    T s = x[c];
#pragma unroll
    for (int k = 0; k < c; ++k) s -= x[k] * lkk[c][k];
    x[c] = s * rdiag[c];
  }
#pragma unroll
  for (int c = 0; c < NB; ++c) m[r + static_cast<Index>(kb * NB + c) * ld] = x[c];
}

// Trailing update with the panels [kb0, kb0 + np) of the factor, C(i, j) -= sum_q L(i, q)
// L(j, q)^T over 32 x 32 tiles. col != 0: only block column c = kb0 + np, block rows i >= c
// (the left-looking update of the next panel inside a group); otherwise every lower tile with
// i, j >= kb0 + np. Grouping np panels per trailing update reads and writes the trailing
// matrices once per group instead of once per panel.
template <class T>
__global__ void syrk_update_kernel(int kb0, int np, int col, const int* __restrict__ lds,
                                   const Index* __restrict__ mat_off, T* __restrict__ mats) {
  const Index d = blockIdx.x;
  const int ld = lds[d];
  const int nbd = ld / NB;
  const int first = kb0 + np;
  if (first >= nbd) return;
  int bi, bj;
  if (col) {
    bi = first + static_cast<int>(blockIdx.y);
    bj = first;
    if (bi >= nbd) return;
  } else {
    const int rem = nbd - first;
    const Index ntiles = static_cast<Index>(rem) * (rem + 1) / 2;
    if (static_cast<Index>(blockIdx.y) >= ntiles) return;
    int ti, tj;
    tile_of(blockIdx.y, ti, tj);
    bi = first + ti;
    bj = first + tj;
  }
  T* m = mats + mat_off[d];
  __shared__ T pi[NB][NB + 1];  // pi[k][i] = L(bi*NB + i, q*NB + k)
  __shared__ T pj[NB][NB + 1];
  const int i = threadIdx.x & 31;
  const int jy = threadIdx.x >> 5;  // 0..7
  T acc[4] = {T(0), T(0), T(0), T(0)};
  for (int q = kb0; q < kb0 + np; ++q) {
    __syncthreads();
    for (int e = threadIdx.x; e < NB * NB; e += blockDim.x) {
      const int rr = e % NB, kk = e / NB;
      pi[kk][rr] = m[(bi * NB + rr) + static_cast<Index>(q * NB + kk) * ld];
      pj[kk][rr] = m[(bj * NB + rr) + static_cast<Index>(q * NB + kk) * ld];
    }
    __syncthreads();
#pragma unroll 8
    for (int k = 0; k < NB; ++k) {
      const T a = pi[k][i];
#pragma unroll
      for (int qq = 0; qq < 4; ++qq) acc[qq] += a * pj[k][jy + 8 * qq];
    }
  }
#pragma unroll
  for (int qq = 0; qq < 4; ++qq) {
    const int j = jy + 8 * qq;
    m[(bi * NB + i) + static_cast<Index>(bj * NB + j) * ld] -= acc[qq];
  }
}

// Trailing update of a panel group over 64 x 64 tiles (register-tiled: 256 threads, 4 x 4
// outputs each), C(i, j) -= sum over the panels [kb0, kb0 + np) of L(i, q) L(j, q)^T for the
// lower tiles from block kb0 + np on. Tiles cover two 32-blocks per side; rows or columns past
// the domain's last block are skipped, and so is the part of a diagonal tile above the
// diagonal blocks.
template <class T>
__global__ void __launch_bounds__(256)
    syrk64_update_kernel(int kb0, int np, const int* __restrict__ lds,
                         const Index* __restrict__ mat_off, T* __restrict__ mats) {
  const Index d = blockIdx.x;
  const int ld = lds[d];
  const int nbd = ld / NB;
  const int first = kb0 + np;
  if (first >= nbd) return;
  const int rem2 = (nbd - first + 1) / 2;
  const Index ntiles = static_cast<Index>(rem2) * (rem2 + 1) / 2;
  if (static_cast<Index>(blockIdx.y) >= ntiles) return;
  int ti, tj;
  tile_of(blockIdx.y, ti, tj);
  const int r0 = (first + 2 * ti) * NB, c0 = (first + 2 * tj) * NB;
  T* m = mats + mat_off[d];
  __shared__ __align__(16) T sa[NB][64 + 4];  // sa[k][r] = L(r0 + r, q*NB + k)
  __shared__ __align__(16) T sb[NB][64 + 4];  // sb[k][c] = L(c0 + c, q*NB + k)
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  T acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = T(0);
  for (int q = kb0; q < kb0 + np; ++q) {
    __syncthreads();
    for (int e = threadIdx.x; e < 64 * NB; e += blockDim.x) {
      const int rr = e % 64, kk = e / 64;
      const Index col = static_cast<Index>(q * NB + kk) * ld;
      sa[kk][rr] = (r0 + rr < ld) ? m[(r0 + rr) + col] : T(0);
      sb[kk][rr] = (c0 + rr < ld) ? m[(c0 + rr) + col] : T(0);
    }
    __syncthreads();
#pragma unroll 8
    for (int k = 0; k < NB; ++k) {
      T av[4], bv[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) av[a] = sa[k][ty * 4 + a];
#pragma unroll
      for (int b = 0; b < 4; ++b) bv[b] = sb[k][tx * 4 + b];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] += av[a] * bv[b];
    }
  }
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int r = r0 + ty * 4 + a;
    if (r >= ld) continue;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int c = c0 + tx * 4 + b;
      if (c >= ld || c / NB > r / NB) continue;  // past the domain, or an upper block
      m[r + static_cast<Index>(c) * ld] -= acc[a][b];
    }
  }
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src, unsigned src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(
                   static_cast<unsigned>(__cvta_generic_to_shared(dst))),
               "l"(src), "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// FP32 trailing update of a panel group over 128 x 128 tiles: C(i, j) -= sum over the group's
// columns of L(i, k) L(j, k) for the lower tiles of the trailing matrix (rows and columns from
// (kb0 + np) * 32). 256 threads, 8 x 8 outputs each; the group's columns stream through a
// three-stage cp.async pipeline in chunks of 16 (rows contiguous, as in the factor). The grid
// is (tile, domain), tiles fastest, so the blocks running together share one domain's panels in
// L2. Rows past the domain load zeros; a diagonal tile writes its 32-blocks on and below the
// diagonal only.
constexpr int kTile = 128, kChunk = 16, kStages = 3;
constexpr size_t kSyrk128Smem = 2ull * kStages * kChunk * kTile * sizeof(float);

__global__ void __launch_bounds__(256, 2)
    syrk128_update_kernel(int kb0, int np, const int* __restrict__ lds,
                          const Index* __restrict__ mat_off, float* __restrict__ mats) {
  const Index d = blockIdx.y;
  const int ld = lds[d];
  const int first = (kb0 + np) * NB;
  if (first >= ld) return;
  const int nt = (ld - first + kTile - 1) / kTile;
  if (static_cast<Index>(blockIdx.x) >= static_cast<Index>(nt) * (nt + 1) / 2) return;
  int ti, tj;
  tile_of(blockIdx.x, ti, tj);
  const int r0 = first + ti * kTile, c0 = first + tj * kTile;
  float* mat = mats + mat_off[d];
  const float* panel = mat + static_cast<Index>(kb0 * NB) * ld;
  extern __shared__ float4 syrk_smem[];
  float* sa = reinterpret_cast<float*>(syrk_smem);  // [stage][k][row]
  float* sb = sa + kStages * kChunk * kTile;        // [stage][k][col]
  const int tid = threadIdx.x;
  const int nk = np * NB / kChunk;

  auto load_chunk = [&](int stage, int kc) {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int idx = tid + 256 * e;
      const int which = idx >> 9, w = idx & 511, k = w >> 5, r4 = (w & 31) * 4;
      const int row = (which ? c0 : r0) + r4;
      const bool have = row < ld;
      const float* src = have ? panel + static_cast<Index>(kc + k) * ld + row : panel;
      float* dst = (which ? sb : sa) + (stage * kChunk + k) * kTile + r4;
      cp_async16(dst, src, have ? 16u : 0u);
    }
  };

  float acc[8][8];
#pragma unroll
  for (int a = 0; a < 8; ++a)
#pragma unroll
    for (int b = 0; b < 8; ++b) acc[a][b] = 0.0f;
  const int tr = tid & 15, tc = tid >> 4;  // rows 8 tr .., columns 8 tc ..

#pragma unroll
  for (int st = 0; st < kStages - 1; ++st) {
    if (st < nk) load_chunk(st, st * kChunk);
    cp_async_commit();
  }
  for (int kk = 0; kk < nk; ++kk) {
    cp_async_wait<kStages - 2>();
    __syncthreads();
    const int nxt = kk + kStages - 1;
    if (nxt < nk) load_chunk(nxt % kStages, nxt * kChunk);
    cp_async_commit();
    const int st = kk % kStages;
    const float* a_s = sa + st * kChunk * kTile + 8 * tr;
    const float* b_s = sb + st * kChunk * kTile + 8 * tc;
#pragma unroll
    for (int k = 0; k < kChunk; ++k) {
      const float4 a0 = *reinterpret_cast<const float4*>(a_s + k * kTile);
      const float4 a1 = *reinterpret_cast<const float4*>(a_s + k * kTile + 4);
      const float4 b0 = *reinterpret_cast<const float4*>(b_s + k * kTile);
      const float4 b1 = *reinterpret_cast<const float4*>(b_s + k * kTile + 4);
      const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int b = 0; b < 8; ++b) acc[a][b] = fmaf(av[a], bv[b], acc[a][b]);
    }
  }
  cp_async_wait<0>();

  const int r = r0 + 8 * tr;  // eight rows inside one 32-block
  if (r >= ld) return;
#pragma unroll
  for (int b = 0; b < 8; ++b) {
    const int c = c0 + 8 * tc + b;
    if (c >= ld || c / NB > r / NB) continue;
    float4* dst = reinterpret_cast<float4*>(mat + r + static_cast<Index>(c) * ld);
    float4 x0 = dst[0], x1 = dst[1];
    x0.x -= acc[0][b];
    x0.y -= acc[1][b];
    x0.z -= acc[2][b];
    x0.w -= acc[3][b];
    x1.x -= acc[4][b];
    x1.y -= acc[5][b];
    x1.z -= acc[6][b];
    x1.w -= acc[7][b];
    dst[0] = x0;
    dst[1] = x1;
  }
}

// The same trailing update on the tensor cores (tcgen05, kind::tf32): each 128 x 128 tile of
// the trailing matrix is one M = 128, N = 128 accumulator in TMEM, C(i, j) -= A B^T with A the
// tile's 128 rows and B its 128 columns of the group's panels (B = A on diagonal tiles). FP32
// accuracy from TF32 head/tail splits of both operands: A B ~ Ah Bh + Ah Bl + Al Bh.
// Pipeline per 16-column chunk: the raw panel columns (rows contiguous) stream into shared
// memory by cp.async one chunk ahead (two raw stages); each thread then splits its row of the
// chunk into head and tail in the MMA's K-major core-matrix layout (two operand stages, each
// released by the commit of its MMAs), and one thread issues the MMAs. The epilogue reads the
// accumulator (warp w: TMEM lanes 32 w .. + 31, its rows) and subtracts it from the tile in
// global memory (coalesced per column). Rows past the domain load zeros; a diagonal tile writes
// its 32-blocks on and below the diagonal only. Every wait is bounded; a wait that runs out
// sets *err and the block finishes its MMAs in flight, frees its TMEM and returns without
// writing.
constexpr int kTcRaw = 2;                              // raw chunk stages
constexpr int kTcOps = 2;                              // operand (head/tail) stages
constexpr int kTcChunkFloats = kTile * kChunk;         // 2048 floats: 8 KB
constexpr int kTcRawFloats = 2 * kTcChunkFloats;       // A and B columns of one chunk
constexpr int kTcOpFloats = 4 * kTcChunkFloats;        // A head, A tail, B head, B tail
constexpr size_t kTcDataBytes =
    (static_cast<size_t>(kTcRaw) * kTcRawFloats + static_cast<size_t>(kTcOps) * kTcOpFloats) * sizeof(float);
constexpr size_t kSyrkTcSmem = kTcDataBytes + 64 + 1024;  // barriers, TMEM address, alignment
constexpr uint32_t kSyrkIdesc = tc::idesc_tf32(128, 128);

__global__ void __launch_bounds__(128, 2)
    syrk_tc_kernel(int kb0, int np, const int* __restrict__ lds, const Index* __restrict__ mat_off,
                   float* __restrict__ mats, int* __restrict__ err) {
  const Index d = blockIdx.y;
  const int ld = lds[d];
  const int first = (kb0 + np) * NB;
  if (first >= ld) return;
  const int nt = (ld - first + kTile - 1) / kTile;
  if (static_cast<Index>(blockIdx.x) >= static_cast<Index>(nt) * (nt + 1) / 2) return;
  int ti, tj;
  tile_of(blockIdx.x, ti, tj);
  const int r0 = first + ti * kTile, c0 = first + tj * kTile;
  const bool diag = ti == tj;
  float* mat = mats + mat_off[d];
  const float* panel = mat + static_cast<Index>(kb0 * NB) * ld;
  extern __shared__ unsigned char syrk_tc_smem[];
  unsigned char* base = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(syrk_tc_smem) + 1023) & ~static_cast<uintptr_t>(1023));
  float* ops = reinterpret_cast<float*>(base);         // [kTcOps][4][128 x 16] core-matrix layout
  float* raw = ops + kTcOps * kTcOpFloats;              // [kTcRaw][A|B][16 k][128 rows]
  uint64_t* bars = reinterpret_cast<uint64_t*>(base + kTcDataBytes);
  uint32_t* misc = reinterpret_cast<uint32_t*>(bars + kTcOps + 1);
  auto op_bar = [&](int s) { return tc::smem_u32(&bars[s]); };
  const uint32_t final_bar = tc::smem_u32(&bars[kTcOps]);
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;

  if (tid == 0) {
    for (int s = 0; s <= kTcOps; ++s) tc::mbar_init(tc::smem_u32(&bars[s]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     tc::smem_u32(&misc[0])),
                 "r"(128)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = misc[0];

  // Raw copy of chunk kk: 16 columns x 128 rows of A (and of B off the diagonal), 16 B pieces.
  const int nk = np * NB / kChunk;
  auto load_raw = [&](int kk) {
    float* dst = raw + (kk % kTcRaw) * kTcRawFloats;
    const int kc = kk * kChunk;
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int idx = tid + 128 * e;  // 0 .. 1023: operand, column, four rows
      const int which = idx >> 9, w = idx & 511, k = w >> 5, r4 = (w & 31) * 4;
      if (which == 1 && diag) continue;
      const int row = (which ? c0 : r0) + r4;
      const bool have = row < ld;
      const float* src = have ? panel + static_cast<Index>(kc + k) * ld + row : panel;
      tc::cp_async16(tc::smem_u32(dst + which * kTcChunkFloats + k * kTile + r4), src,
                     have ? 16u : 0u);
    }
    tc::cp_async_commit();
  };

  bool ok = true;
  load_raw(0);
  for (int kk = 0; kk < nk; ++kk) {
    if (kk + 1 < nk) load_raw(kk + 1);
    else tc::cp_async_commit();
    tc::cp_async_wait<1>();  // chunk kk has landed
    const int s = kk % kTcOps;
    // The operand stage's previous MMAs (chunk kk - kTcOps) have read it.
    const bool waited = kk < kTcOps ||
                        tc::mbar_wait(op_bar(s), ((kk / kTcOps) - 1) & 1, tc::kWaitPolls);
    if (__syncthreads_or(!waited)) {
      ok = false;
      break;
    }
    float* a_hi = ops + s * kTcOpFloats;
    float* a_lo = a_hi + kTcChunkFloats;
    float* b_hi = diag ? a_hi : a_lo + kTcChunkFloats;
    float* b_lo = diag ? a_lo : b_hi + kTcChunkFloats;
    const float* rc = raw + (kk % kTcRaw) * kTcRawFloats;
#pragma unroll
    for (int op = 0; op < 2; ++op) {
      if (op == 1 && diag) break;
      const float* col = rc + op * kTcChunkFloats + tid;
      float* hi = op ? b_hi : a_hi;
      float* lo = op ? b_lo : a_lo;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float x0 = col[(4 * j) * kTile], x1 = col[(4 * j + 1) * kTile];
        const float x2 = col[(4 * j + 2) * kTile], x3 = col[(4 * j + 3) * kTile];
        const float4 h{tc::tf32_round(x0), tc::tf32_round(x1), tc::tf32_round(x2), tc::tf32_round(x3)};
        const int off = tc::core_off(tid, 4 * j);
        *reinterpret_cast<float4*>(hi + off) = h;
        *reinterpret_cast<float4*>(lo + off) = float4{x0 - h.x, x1 - h.y, x2 - h.z, x3 - h.w};
      }
    }
    tc::fence_proxy_async();
    __syncthreads();  // operands written; the raw stage of chunk kk may be refilled
    if (tid == 0) {
      tc::tc_fence_after();
      const uint32_t ah = tc::smem_u32(a_hi), al = tc::smem_u32(a_lo);
      const uint32_t bh = tc::smem_u32(b_hi), bl = tc::smem_u32(b_lo);
#pragma unroll
      for (int ks = 0; ks < 2; ++ks) {
        const uint32_t ko = static_cast<uint32_t>(ks * 256);
        tc::mma_tf32(tmem, tc::make_desc(ah + ko), tc::make_desc(bh + ko), kSyrkIdesc,
                     (kk == 0 && ks == 0) ? 0u : 1u);
        tc::mma_tf32(tmem, tc::make_desc(ah + ko), tc::make_desc(bl + ko), kSyrkIdesc, 1u);
        tc::mma_tf32(tmem, tc::make_desc(al + ko), tc::make_desc(bh + ko), kSyrkIdesc, 1u);
      }
      tc::mma_commit(op_bar(s));
    }
  }
  tc::cp_async_wait<0>();
  // All MMAs complete before the accumulator is read or TMEM is freed.
  if (tid == 0) tc::mma_commit(final_bar);
  const bool done = tc::mbar_wait(final_bar, 0, tc::kWaitPolls);
  if (__syncthreads_or(!done)) ok = false;
  if (!ok) {
    if (tid == 0) atomicExch(err, 1);
  } else {
    tc::tc_fence_after();
    const int row = r0 + 32 * warp + lane;
#pragma unroll 1
    for (int u = 0; u < kTile / 32; ++u) {
      float v[32];
      tc::tmem_ld16(tmem + (static_cast<uint32_t>(32 * warp) << 16) + static_cast<uint32_t>(32 * u), v);
      tc::tmem_ld16(tmem + (static_cast<uint32_t>(32 * warp) << 16) + static_cast<uint32_t>(32 * u + 16),
                    v + 16);
      if (row < ld) {
        float cur[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int c = c0 + 32 * u + j;
          cur[j] = (c < ld && c / NB <= row / NB) ? mat[row + static_cast<Index>(c) * ld] : 0.0f;
        }
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int c = c0 + 32 * u + j;
          if (c < ld && c / NB <= row / NB) mat[row + static_cast<Index>(c) * ld] = cur[j] - v[j];
        }
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(128)
                 : "memory");
  }
}

// FP32 left-looking update of one block column inside a panel group: C(i, j) -= sum over the
// group's panels [kb0, kb0 + np) of L(i, k) L(j, k) for the 32 columns of block column
// kb0 + np and every row from that block down. 128-row tiles, 256 threads with 4 x 4 outputs
// each, the trailing update's cp.async pipeline; grid (row tile, domain).
constexpr size_t kPanelSmem = static_cast<size_t>(kStages) * kChunk * (kTile + NB) * sizeof(float);

__global__ void __launch_bounds__(256, 4)
    panel_update_kernel(int kb0, int np, const int* __restrict__ lds,
                        const Index* __restrict__ mat_off, float* __restrict__ mats) {
  const Index d = blockIdx.y;
  const int ld = lds[d];
  const int c0 = (kb0 + np) * NB;
  const int r0 = c0 + static_cast<int>(blockIdx.x) * kTile;
  if (r0 >= ld) return;
  float* mat = mats + mat_off[d];
  const float* panel = mat + static_cast<Index>(kb0 * NB) * ld;
  extern __shared__ float4 panel_smem[];
  float* sa = reinterpret_cast<float*>(panel_smem);  // [stage][k][row]
  float* sb = sa + kStages * kChunk * kTile;         // [stage][k][column]
  const int tid = threadIdx.x;
  const int nk = np * NB / kChunk;

  auto load_chunk = [&](int stage, int kc) {
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const int idx = tid + 256 * e;
      const int k = idx >> 5, r4 = (idx & 31) * 4;
      const int row = r0 + r4;
      const bool have = row < ld;
      const float* src = have ? panel + static_cast<Index>(kc + k) * ld + row : panel;
      cp_async16(sa + (stage * kChunk + k) * kTile + r4, src, have ? 16u : 0u);
    }
    if (tid < 128) {  // the block column's own 32 rows: c0 + 32 <= ld
      const int k = tid >> 3, c4 = (tid & 7) * 4;
      cp_async16(sb + (stage * kChunk + k) * NB + c4, panel + static_cast<Index>(kc + k) * ld + c0 + c4, 16u);
    }
  };

  float acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0f;
  const int tr = tid & 31, tc = tid >> 5;  // rows 4 tr .., columns 4 tc ..

#pragma unroll
  for (int st = 0; st < kStages - 1; ++st) {
    if (st < nk) load_chunk(st, st * kChunk);
    cp_async_commit();
  }
  for (int kk = 0; kk < nk; ++kk) {
    cp_async_wait<kStages - 2>();
    __syncthreads();
    const int nxt = kk + kStages - 1;
    if (nxt < nk) load_chunk(nxt % kStages, nxt * kChunk);
    cp_async_commit();
    const int st = kk % kStages;
    const float* a_s = sa + st * kChunk * kTile + 4 * tr;
    const float* b_s = sb + st * kChunk * NB + 4 * tc;
#pragma unroll
    for (int k = 0; k < kChunk; ++k) {
      const float4 av = *reinterpret_cast<const float4*>(a_s + k * kTile);
      const float4 bv = *reinterpret_cast<const float4*>(b_s + k * NB);
      const float a4[4] = {av.x, av.y, av.z, av.w};
      const float b4[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = fmaf(a4[a], b4[b], acc[a][b]);
    }
  }
  cp_async_wait<0>();

  const int r = r0 + 4 * tr;
  if (r >= ld) return;
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    float4* dst = reinterpret_cast<float4*>(mat + r + static_cast<Index>(c0 + 4 * tc + b) * ld);
    float4 x = *dst;
    x.x -= acc[0][b];
    x.y -= acc[1][b];
    x.z -= acc[2][b];
    x.w -= acc[3][b];
    *dst = x;
  }
}

// Replaces every 32x32 diagonal block of the Cholesky factor by its inverse (lower triangular),
// so that the triangular solves apply the diagonal blocks as small matrix-vector products
// instead of 32-step dependent substitutions.
template <class T>
__global__ void invert_diag_kernel(const int* __restrict__ lds, const Index* __restrict__ mat_off,
                                   T* __restrict__ mats) {
  const Index d = blockIdx.x;
  const int ld = lds[d];
  const int kb = blockIdx.y;
  if (kb * NB >= ld) return;
  __shared__ T a[NB][NB + 1];
  __shared__ T inv[NB][NB + 1];
  T* m = mats + mat_off[d] + static_cast<Index>(kb * NB) * ld + kb * NB;
  const int lane = threadIdx.x;
  for (int c = 0; c < NB; ++c) a[lane][c] = m[lane + static_cast<Index>(c) * ld];
  __syncwarp();
  // Column `lane` of the inverse by forward substitution.
  const int j = lane;
  for (int i = 0; i < NB; ++i) {
    T v;
    if (i < j) {
      v = T(0);
    } else if (i == j) {
      v = T(1) / a[j][j];
    } else {
      T s = T(0);
      for (int k = j; k < i; ++k) s += a[i][k] * inv[k][j];
      v = -s / a[i][i];
    }
    inv[i][j] = v;
  }
  __syncwarp();
  for (int c = 0; c < NB; ++c) m[lane + static_cast<Index>(c) * ld] = inv[lane][c];
}

// Solves L L^T x = b in place (x in shared memory, ld entries) with the factor whose diagonal
// blocks hold their inverses. Block-sequential; within a block the diagonal block is a 32x32
// product (warp 0, loads issued before the shuffles) and the off-diagonal part is spread over
// the whole thread block.
// kb0 > 0: the right-hand side is zero above block kb0, and only the solution from block kb0
// down is wanted (its forward sweep starts there and its backward sweep stops there).
template <class T>
__device__ void chol_solve_inplace(double* x, const T* __restrict__ m, int ld, int kb0 = 0) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int nb = ld / NB;
  // Forward: L y = b.
  for (int kb = kb0; kb < nb; ++kb) {
    const int base = kb * NB;
    if (warp == 0) {
      // y_blk = L_kk^{-1} b_blk (the inverted diagonal block, lower triangular).
      const double bi = x[base + lane];
      double yi = 0;
#pragma unroll 8
      for (int jj = 0; jj < NB; ++jj) {
        const double a = jj <= lane ? static_cast<double>(m[(base + lane) + static_cast<Index>(base + jj) * ld]) : 0.0;
        yi += a * __shfl_sync(0xffffffffu, bi, jj);
      }
      x[base + lane] = yi;
    }
    __syncthreads();
    for (int r = (kb + 1) * NB + tid; r < ld; r += blockDim.x) {
      double s = 0;
#pragma unroll 8
      for (int c = 0; c < NB; ++c) s += static_cast<double>(m[r + static_cast<Index>(base + c) * ld]) * x[base + c];
      x[r] -= s;
    }
    __syncthreads();
  }
  // Backward: L^T x = y.
  for (int kb = nb - 1; kb >= kb0; --kb) {
    const int base = kb * NB;
    for (int c = warp; c < NB; c += nw) {
      const int col = base + c;
      double s = 0;
      for (int r = (kb + 1) * NB + lane; r < ld; r += 32)
        s += static_cast<double>(m[r + static_cast<Index>(col) * ld]) * x[r];
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) x[col] -= s;
    }
    __syncthreads();
    if (warp == 0) {
      // x_blk = L_kk^{-T} y_blk: lane i sums inv[j][i] y_j over j >= i (column i of the block).
      const double yi = x[base + lane];
      double zi = 0;
#pragma unroll 8
      for (int jj = 0; jj < NB; ++jj) {
        const double a = jj >= lane ? static_cast<double>(m[(base + jj) + static_cast<Index>(base + lane) * ld]) : 0.0;
        zi += a * __shfl_sync(0xffffffffu, yi, jj);
      }
      x[base + lane] = zi;
    }
    __syncthreads();
  }
}

// The same solve for an FP32 factor, in FP32 (the factor's own precision; FP64 arithmetic runs
// at 1/64 of the FP32 rate here and would bound the sweep). Each 32-column panel is streamed
// once per sweep with float4 loads: rows below the diagonal block in the forward sweep,
// columns in the backward sweep (four columns per warp, a dot product each).
__device__ void chol_solve_f32(float* x, const float* __restrict__ m, int ld) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int nb = ld / NB;
  // Forward: L y = b.
  for (int kb = 0; kb < nb; ++kb) {
    const int base = kb * NB;
    if (warp == 0) {
      // y_blk = L_kk^{-1} b_blk; lane i holds row i of the inverted (lower) diagonal block.
      const float bi = x[base + lane];
      const float* row = m + base + lane + static_cast<Index>(base) * ld;
      float yi = 0.0f;
#pragma unroll 1
      for (int j0 = 0; j0 < NB; j0 += 8) {
        float a[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) a[q] = j0 + q <= lane ? row[static_cast<Index>(j0 + q) * ld] : 0.0f;
#pragma unroll
        for (int q = 0; q < 8; ++q) yi = fmaf(a[q], __shfl_sync(0xffffffffu, bi, j0 + q), yi);
      }
      x[base + lane] = yi;
    }
    __syncthreads();
    const float* panel = m + static_cast<Index>(base) * ld;
#pragma unroll 1
    for (int r = base + NB + 4 * tid; r < ld; r += 4 * blockDim.x) {
      float4 s = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll 4
      for (int c = 0; c < NB; ++c) {
        const float4 v = *reinterpret_cast<const float4*>(panel + r + static_cast<Index>(c) * ld);
        const float xc = x[base + c];
        s.x = fmaf(v.x, xc, s.x);
        s.y = fmaf(v.y, xc, s.y);
        s.z = fmaf(v.z, xc, s.z);
        s.w = fmaf(v.w, xc, s.w);
      }
      float4* xr = reinterpret_cast<float4*>(x + r);
      float4 t = *xr;
      t.x -= s.x;
      t.y -= s.y;
      t.z -= s.z;
      t.w -= s.w;
      *xr = t;
    }
    __syncthreads();
  }
  // Backward: L^T x = y.
  for (int kb = nb - 1; kb >= 0; --kb) {
    const int base = kb * NB, below = base + NB;
    for (int c0 = 4 * warp; c0 < NB; c0 += 4 * nw) {
      float s[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll 2
      for (int r = below + 4 * lane; r < ld; r += 128) {
        const float4 xr = *reinterpret_cast<const float4*>(x + r);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float4 v =
              *reinterpret_cast<const float4*>(m + r + static_cast<Index>(base + c0 + q) * ld);
          s[q] = fmaf(v.x, xr.x, fmaf(v.y, xr.y, fmaf(v.z, xr.z, fmaf(v.w, xr.w, s[q]))));
        }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        for (int o = 16; o > 0; o >>= 1) s[q] += __shfl_xor_sync(0xffffffffu, s[q], o);
        if (lane == 0) x[base + c0 + q] -= s[q];
      }
    }
    __syncthreads();
    if (warp == 0) {
      // x_blk = L_kk^{-T} y_blk; lane i holds column i of the inverted diagonal block.
      const float yi = x[base + lane];
      const float* col = m + base + static_cast<Index>(base + lane) * ld;
      float zi = 0.0f;
#pragma unroll 1
      for (int j0 = 0; j0 < NB; j0 += 8) {
        const float4 v0 = *reinterpret_cast<const float4*>(col + j0);
        const float4 v1 = *reinterpret_cast<const float4*>(col + j0 + 4);
        const float a[8] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const float yj = __shfl_sync(0xffffffffu, yi, j0 + q);
          if (j0 + q >= lane) zi = fmaf(a[q], yj, zi);
        }
      }
      x[base + lane] = zi;
    }
    __syncthreads();
  }
}

// Column j of (L L^T)^{-1} for every j (grid = n blocks): the coarse grid keeps the explicit
// inverse so that each coarse solve is one matrix-vector product spread over the GPU. Block j
// solves for e_j from its diagonal block down (the forward solution is zero above row j, and
// the symmetric inverse needs rows i >= j only) and writes entry (i, j) and its mirror (j, i):
// n^3 / 3 multiply-adds in all instead of n^3.
template <class T>
__global__ void chol_inverse_kernel(const T* __restrict__ m, int ld, int n, double* __restrict__ inv) {
  extern __shared__ double sh[];
  double* x = sh;
  const int j = blockIdx.x;
  for (int i = threadIdx.x; i < ld; i += blockDim.x) x[i] = (i == j) ? 1.0 : 0.0;
  __syncthreads();
  chol_solve_inplace(x, m, ld, j / NB);
  for (int i = j + threadIdx.x; i < n; i += blockDim.x) {
    inv[static_cast<Index>(j) * n + i] = x[i];
    inv[static_cast<Index>(i) * n + j] = x[i];
  }
}

// Coarse right-hand side: x_i = d_{l+i} - sum_k L_ik d_k (Q^T d), d_k the polynomial points.
__global__ void coarse_rhs_kernel(const Index* __restrict__ dp, int n, int l,
                                  const double* __restrict__ lag, const double* __restrict__ resid,
                                  double* __restrict__ x, double* __restrict__ dh_out) {
  __shared__ double dh[16];
  if (threadIdx.x < l) dh[threadIdx.x] = resid[dp[threadIdx.x]];
  __syncthreads();
  if (blockIdx.x == 0 && threadIdx.x < l) dh_out[threadIdx.x] = dh[threadIdx.x];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Index g = dp[l + i];
  double s = resid[g];
  for (int k = 0; k < l; ++k) s -= lag[g * l + k] * dh[k];
  x[i] = s;
}

// y = S x for a symmetric n x n matrix (column j contiguous): one warp per output entry.
__global__ void symv_kernel(const double* __restrict__ s, int n, const double* __restrict__ x,
                            double* __restrict__ y) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= n) return;
  const double* col = s + static_cast<Index>(warp) * n;
  double acc = 0;
  for (int j = lane; j < n; j += 32) acc += col[j] * x[j];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) y[warp] = acc;
}

// lambda = Q gamma scattered to every coarse point; out[k] = lambda_head_k, out[16+k] = sum_i
// u_ik gamma_i (for the polynomial solve on the host).
__global__ void coarse_finish_kernel(const Index* __restrict__ dp, int n, int l,
                                     const double* __restrict__ lag, const double* __restrict__ u,
                                     const double* __restrict__ gamma, double* __restrict__ weights,
                                     double* __restrict__ out) {
  __shared__ double red[2][32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  for (int i = tid; i < n; i += blockDim.x) weights[dp[l + i]] = gamma[i];
  for (int k = 0; k < l; ++k) {
    double s1 = 0, s2 = 0;
    for (int i = tid; i < n; i += blockDim.x) {
      const Index g = dp[l + i];
      s1 += lag[g * l + k] * gamma[i];
      s2 += u[g * l + k] * gamma[i];
    }
    for (int o = 16; o > 0; o >>= 1) {
      s1 += __shfl_xor_sync(0xffffffffu, s1, o);
      s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    __syncthreads();
    if (lane == 0) {
      red[0][warp] = s1;
      red[1][warp] = s2;
    }
    __syncthreads();
    if (tid == 0) {
      double a = 0, b = 0;
      for (int w = 0; w < nw; ++w) {
        a += red[0][w];
        b += red[1][w];
      }
      out[k] = -a;
      out[16 + k] = b;
      weights[dp[k]] = -a;
    }
  }
}

// Fine (or coarse) solve of every domain: gather the residuals, form Q^T d, solve with the
// Cholesky factor, expand lambda = Q gamma and scatter the owned entries
// (fine_grid.hpp:97-156, coarse_grid.hpp:91-131).
template <class T>
__global__ void __launch_bounds__(256, 4) ras_solve_kernel(const int* __restrict__ nsz, const int* __restrict__ lds,
                                 const Index* __restrict__ mat_off, const T* __restrict__ mats,
                                 const Index* __restrict__ pt_off, const Index* __restrict__ pts,
                                 const char* __restrict__ inner, int l,
                                 const double* __restrict__ lag, const double* __restrict__ u,
                                 const double* __restrict__ resid, double* __restrict__ weights,
                                 int coarse, double* __restrict__ coarse_out) {
  extern __shared__ double sh[];
  const Index d = blockIdx.x;
  const int n = nsz[d], ld = lds[d];
  const Index* dp = pts + pt_off[d];
  const char* din = inner + pt_off[d];
  const T* m = mats + mat_off[d];
  double* dh = sh;                           // l (polynomial-point residuals)
  double* red = sh + 16;                     // 2 x 32 reduction scratch
  T* x = reinterpret_cast<T*>(sh + 80);      // ld, in the factor's precision
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;

  for (int k = tid; k < l; k += blockDim.x) dh[k] = resid[dp[k]];
  __syncthreads();
  for (int i = tid; i < ld; i += blockDim.x) {
    double s = 0;
    if (i < n) {
      const Index g = dp[l + i];
      s = resid[g];
      for (int k = 0; k < l; ++k) s -= lag[g * l + k] * dh[k];
    }
    x[i] = static_cast<T>(s);
  }
  __syncthreads();
  if constexpr (std::is_same_v<T, float>)
    chol_solve_f32(x, m, ld);
  else
    chol_solve_inplace(x, m, ld);
  // lambda_head_k = -sum_i L_ik gamma_i ; for the coarse grid also s_k = sum_i u_ik gamma_i.
  for (int k = 0; k < l; ++k) {
    double s1 = 0, s2 = 0;
    for (int i = tid; i < n; i += blockDim.x) {
      const Index g = dp[l + i];
      s1 += lag[g * l + k] * x[i];
      if (coarse) s2 += u[g * l + k] * x[i];
    }
    for (int o = 16; o > 0; o >>= 1) {
      s1 += __shfl_xor_sync(0xffffffffu, s1, o);
      s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if (lane == 0) {
      red[warp] = s1;
      red[32 + warp] = s2;
    }
    __syncthreads();
    if (tid == 0) {
      double a = 0, b = 0;
      for (int w = 0; w < nw; ++w) {
        a += red[w];
        b += red[32 + w];
      }
      dh[k] = -a;  // lambda_head
      if (coarse) {
        coarse_out[k] = -a;
        coarse_out[16 + k] = b;
      }
    }
    __syncthreads();
  }
  if (n == 0) {
    for (int k = tid; k < l; k += blockDim.x) dh[k] = 0.0;
    if (coarse && tid < l) {
      coarse_out[tid] = 0.0;
      coarse_out[16 + tid] = 0.0;
    }
    __syncthreads();
  }
  for (int i = tid; i < n; i += blockDim.x)
    if (coarse || din[l + i]) weights[dp[l + i]] = x[i];
  for (int k = tid; k < l; k += blockDim.x)
    if (coarse || din[k]) weights[dp[k]] = dh[k];
}

// PGPU_SYRK_TC=0 in the environment keeps the FP32 trailing updates on the CUDA cores.
bool syrk_tc_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("PGPU_SYRK_TC");
    return e == nullptr || std::atoi(e) != 0;
  }();
  return on;
}

RbfSet rbf_set(const ModelDesc& m) {
  RbfSet rs{};
  rs.n = static_cast<int>(m.rbfs.size());
  for (int r = 0; r < rs.n; ++r) {
    rs.kind[r] = m.rbfs[r].kind;
    rs.p0[r] = m.rbfs[r].p[0];
    rs.p1[r] = m.rbfs[r].p[1];
    for (int k = 0; k < 9; ++k) rs.a[r][k] = m.rbfs[r].a[k];
  }
  return rs;
}

}  // namespace

template <class T>
RasPreconditioner<T>::RasPreconditioner(const ModelDesc& model, const double* points_host,
                                        const double* points_dev, Index mu, const Bbox3& bbox)
    : RasPreconditioner(model, points_host, points_dev, mu, nullptr, nullptr, 0, bbox) {}

template <class T>
RasPreconditioner<T>::RasPreconditioner(const ModelDesc& model, const double* points_host,
                                        const double* points_dev, Index mu,
                                        const double* grad_host, const double* grad_dev,
                                        Index sigma, const Bbox3& bbox)
    : model_(model), l_(model.l()), mu_(mu), sigma_(sigma), rows_(mu + 3 * sigma), bbox_(bbox),
      points_dev_(points_dev), grad_dev_(grad_dev) {
  constexpr double kFineToCoarseRatio = 10.0;
  constexpr Index kNCoarsestPoints = 2048;
  n_levels_ = std::max(static_cast<int>(std::ceil(std::log(static_cast<double>(rows_) / kNCoarsestPoints) /
                                                  std::log(kFineToCoarseRatio))),
                       0) +
              1;
  point_idcs_.resize(n_levels_);
  grad_point_idcs_.resize(n_levels_);
  fine_.resize(n_levels_);
  {
    auto& gtop = grad_point_idcs_[n_levels_ - 1];
    gtop.resize(sigma_);
    for (Index i = 0; i < sigma_; ++i) gtop[i] = i;
  }
  // Degree 1 with one point and gradient points (ras_preconditioner.hpp:80-84): the Lagrange
  // functionals are the point's value and the first gradient point's derivatives.
  const bool special = l_ > 0 && model_.poly_degree == 1 && mu_ == 1 && sigma_ >= 1;
  if (l_ > 0 && mu_ < l_ && !special) throw_invalid("too few points for the polynomial degree");

  // Polynomial points and the Lagrange basis (ras_preconditioner.hpp:76-106).
  if (l_ > 0) {
    poly_idcs_ = special ? std::vector<Index>{0}
                         : unisolvent_point_set(points_host, mu_, model_.poly_degree);
    if (special) {
      poly_rows_ = {0, mu_, mu_ + 1, mu_ + 2};
      std::vector<double> rows(static_cast<size_t>(l_) * l_);
      double m[10];
      poly_row(-1, points_host[0], points_host[1], points_host[2], m);
      for (int c = 0; c < l_; ++c) rows[c] = m[c];
      for (int t = 0; t < 3; ++t) {
        poly_row(t, grad_host[0], grad_host[1], grad_host[2], m);
        for (int c = 0; c < l_; ++c) rows[(t + 1) * l_ + c] = m[c];
      }
      lagrange_coeffs_ = lagrange_coeffs_of(rows, l_);
    } else {
      poly_rows_ = poly_idcs_;
      std::vector<double> pp;
      for (auto i : poly_idcs_)
        for (int k = 0; k < 3; ++k) pp.push_back(points_host[3 * i + k]);
      lagrange_coeffs_ = lagrange_coeffs(model_.poly_degree, pp.data(), l_);
    }
    auto& top = point_idcs_[n_levels_ - 1];
    top = poly_idcs_;
    top.reserve(mu_);
    std::vector<char> is_poly(mu_, 0);
    for (auto i : poly_idcs_) is_poly[i] = 1;
    for (Index i = 0; i < mu_; ++i)
      if (!is_poly[i]) top.push_back(i);
  } else {
    auto& top = point_idcs_[n_levels_ - 1];
    top.resize(mu_);
    for (Index i = 0; i < mu_; ++i) top[i] = i;
  }

  // Points used for the geometric division: A-transformed when the model has one
  // anisotropic RBF (ras_preconditioner.hpp:108-119).
  const bool aniso = model_.rbfs.size() == 1 && !model_.rbfs[0].aniso_is_identity();
  auto n_coarse_of = [&](int level) {
    const double finest = std::log(static_cast<double>(rows_)) / std::log(kFineToCoarseRatio);
    const double coarsest = std::log(static_cast<double>(kNCoarsestPoints)) / std::log(kFineToCoarseRatio);
    return static_cast<Index>(
        std::pow(kFineToCoarseRatio, coarsest + (level - 1) * (finest - coarsest) / (n_levels_ - 1)));
  };

  // The levels are divided on the device (ras_divide.cu) unless PGPU_RAS_HOST_DIVIDE is set:
  // then the host divides them (ras_host.cpp, finest first) on a helper thread and publishes
  // each level's domains as soon as they exist, while this thread runs the device set-up of
  // the levels already published.
  const bool host_division = sigma_ > 0 || std::getenv("PGPU_RAS_HOST_DIVIDE") != nullptr;
  std::vector<double> a_points, a_grad_points;
  const double* div_points = points_host;
  const double* div_grad_points = grad_host;
  if (host_division && aniso) {
    const double* a = model_.rbfs[0].a;
    auto transform = [&](const double* in, Index n, std::vector<double>& out) {
      out.resize(3 * n);
      for (Index i = 0; i < n; ++i) {
        const double* p = in + 3 * i;
        for (int r = 0; r < 3; ++r) out[3 * i + r] = a[3 * r] * p[0] + a[3 * r + 1] * p[1] + a[3 * r + 2] * p[2];
      }
    };
    transform(points_host, mu_, a_points);
    div_points = a_points.data();
    if (sigma_ > 0) {
      transform(grad_host, sigma_, a_grad_points);
      div_grad_points = a_grad_points.data();
    }
  }
  std::vector<std::vector<Domain>> level_domains(n_levels_);
  std::mutex div_mu;
  std::condition_variable div_cv;
  int published = n_levels_;  // levels >= published are available
  std::exception_ptr div_error;
  const int omp_threads = omp_get_max_threads();
  std::thread divide_thread;
  if (host_division) divide_thread = std::thread([&] {
    omp_set_num_threads(omp_threads);
    try {
      for (int level = n_levels_ - 1; level >= 1; --level) {
        const double t0 = wall_seconds();
        const Index n_coarse = n_coarse_of(level);
        // The coarse points of this level (the next level's point set) are chosen on a second
        // thread while this one divides the level; each takes half of the host threads.
        std::pair<std::vector<Index>, std::vector<Index>> coarse;
        std::exception_ptr coarse_error;
        const int half = std::max(1, omp_threads / 2);
        std::thread coarse_thread([&] {
          omp_set_num_threads(half);
          try {
            coarse = DomainDivider::choose_coarse_points(div_points, div_grad_points,
                                                         point_idcs_[level], grad_point_idcs_[level],
                                                         poly_idcs_, n_coarse);
          } catch (...) {
            coarse_error = std::current_exception();
          }
        });
        omp_set_num_threads(std::max(1, omp_threads - half));
        double t1 = 0;
        try {
          DomainDivider divider(div_points, div_grad_points, point_idcs_[level],
                                grad_point_idcs_[level], poly_idcs_);
          t1 = wall_seconds();
          std::lock_guard<std::mutex> lk(div_mu);
          level_domains[level] = std::move(divider.domains());
          published = level;
        } catch (...) {
          coarse_thread.join();
          throw;
        }
        div_cv.notify_all();
        coarse_thread.join();
        omp_set_num_threads(omp_threads);
        if (coarse_error) std::rethrow_exception(coarse_error);
        if (verbose())
          std::printf("ras level %d: %zu points, %zu domains, divide %.3f s, divide + coarse points %.3f s\n",
                      level, point_idcs_[level].size(), level_domains[level].size(), t1 - t0,
                      wall_seconds() - t0);
        std::lock_guard<std::mutex> lk(div_mu);
        point_idcs_[level - 1] = std::move(coarse.first);
        grad_point_idcs_[level - 1] = std::move(coarse.second);
      }
    } catch (...) {
      std::lock_guard<std::mutex> lk(div_mu);
      div_error = std::current_exception();
      published = 0;
    }
    {
      std::lock_guard<std::mutex> lk(div_mu);
      published = 0;
    }
    div_cv.notify_all();
  });
  struct Joiner {
    std::thread& t;
    ~Joiner() {
      if (t.joinable()) t.join();
    }
  } joiner{divide_thread};
  auto wait_level = [&](int level) {
    std::unique_lock<std::mutex> lk(div_mu);
    div_cv.wait(lk, [&] { return published <= level; });
    if (div_error) std::rethrow_exception(div_error);
  };
  const double t_dev = wall_seconds();

  // Device-side per-point data.
  const int l = l_;
  if (sigma_ > 0)
    setup_rows(points_host, grad_host);
  else
    setup_polynomial(points_host, points_dev);

  if (host_division) {
    for (int level = n_levels_ - 1; level >= 1; --level) {
      wait_level(level);
      fine_[level] = std::make_unique<DomainBatch<T>>();
      if (sigma_ > 0)
        build_batch_rows(*fine_[level], level_domains[level]);
      else
        build_batch(*fine_[level], level_domains[level]);
    }
    divide_thread.join();
    if (div_error) std::rethrow_exception(div_error);
  } else if (n_levels_ > 1) {
    DevBuf<double> a_dev;
    const double* coords = points_dev;
    if (aniso) {
      Mat3 a;
      for (int k = 0; k < 9; ++k) a.a[k] = model_.rbfs[0].a[k];
      a_dev.resize(3 * mu_);
      transform_points_kernel<<<blocks_for(mu_, 256), 256, 0, stream()>>>(points_dev, mu_, a, a_dev.data());
      PGPU_LAUNCH_CHECK();
      coords = a_dev.data();
    }
    DeviceDivider divider(coords, mu_, poly_idcs_);
    for (int level = n_levels_ - 1; level >= 1; --level) {
      const double t0 = verbose() ? (sync(), wall_seconds()) : 0.0;
      divider.set_level(point_idcs_[level]);
      LevelDomains ld;
      divider.divide(ld);
      point_idcs_[level - 1] = divider.choose_coarse_points(n_coarse_of(level));
      if (verbose())
        std::printf("ras level %d: %zu points, %zu domains, device divide + coarse points %.3f s\n",
                    level, point_idcs_[level].size(), ld.sizes.size(), wall_seconds() - t0);
      fine_[level] = std::make_unique<DomainBatch<T>>();
      build_batch(*fine_[level], ld.sizes, std::move(ld.pts), std::move(ld.inner));
    }
  }
  {
    Domain cd;
    cd.point_indices = point_idcs_[0];
    cd.inner_point.assign(cd.point_indices.size(), 1);
    if (special) {
      // The coarse grid's first rows are the Lagrange functionals (its polynomial solve inverts
      // them): the first gradient point leads the coarse gradient points.
      auto& g = grad_point_idcs_[0];
      g.erase(std::remove(g.begin(), g.end(), Index{0}), g.end());
      g.insert(g.begin(), Index{0});
    }
    cd.grad_point_indices = grad_point_idcs_[0];
    cd.inner_grad_point.assign(cd.grad_point_indices.size(), 1);
    std::vector<Domain> v{cd};
    if (sigma_ > 0)
      build_batch_rows(coarse_, v);
    else
      build_batch(coarse_, v);
    coarse_n_ = std::max(static_cast<int>(cd.point_indices.size() + 3 * cd.grad_point_indices.size()) - l_, 0);
    const int cld = std::max(NB, ((coarse_n_ + NB - 1) / NB) * NB);
    // With several levels the coarse grid is solved 2L-1 times per application: keep an explicit
    // inverse (one matrix-vector product per solve). A single-level preconditioner solves once
    // per application and keeps the factor.
    use_coarse_inverse_ = n_levels_ > 1 && coarse_n_ > 0;
    if (use_coarse_inverse_) {
      coarse_inv_.resize(static_cast<Index>(coarse_n_) * coarse_n_);
      const double cn = static_cast<double>(coarse_n_);
      ProfScope ps("ras_coarse_inverse_f64", 2.0 * cn * cn * cn / 3.0);
      chol_inverse_kernel<double><<<coarse_n_, 256, cld * sizeof(double), stream()>>>(
          coarse_.mats.data(), cld, coarse_n_, coarse_inv_.data());
      PGPU_LAUNCH_CHECK();
      coarse_.mats.release();
    }
    coarse_x_.resize(std::max(coarse_n_, 1));
    coarse_g_.resize(std::max(coarse_n_, 1));
    coarse_out_.resize(48);
    coarse_out_.zero();
  }

  // Level row sets on the device (for the residual-update evaluators): the level's points,
  // then three rows per gradient point.
  level_idx_dev_.resize(n_levels_);
  level_pts_dev_.resize(n_levels_);
  level_grad_pts_dev_.resize(n_levels_);
  for (int level = 0; level < n_levels_; ++level) {
    const auto& idx = point_idcs_[level];
    const auto& gidx = grad_point_idcs_[level];
    std::vector<Index> rows(idx);
    for (Index j : gidx)
      for (int c = 0; c < 3; ++c) rows.push_back(mu_ + 3 * j + c);
    level_idx_dev_[level].upload(rows);
    std::vector<double> lp(3 * idx.size());
    for (size_t i = 0; i < idx.size(); ++i)
      for (int k = 0; k < 3; ++k) lp[3 * i + k] = points_host[3 * idx[i] + k];
    level_pts_dev_[level].upload(lp);
    if (!gidx.empty()) {
      std::vector<double> gp(3 * gidx.size());
      for (size_t i = 0; i < gidx.size(); ++i)
        for (int k = 0; k < 3; ++k) gp[3 * i + k] = grad_host[3 * gidx[i] + k];
      level_grad_pts_dev_[level].upload(gp);
    }
  }

  if (n_levels_ > 1 && l > 0) {
    // Orthonormalised monomials and their images (ras_preconditioner.hpp:168-188).
    const Index R = rows_;
    p_.resize(R * l);
    monomial_basis(model_.poly_degree, points_dev, mu_, grad_dev_, sigma_, p_.data());
    for (int i = 0; i < l; ++i) {
      double* ci = p_.data() + static_cast<Index>(i) * R;
      double nrm = norm2(ci, R);
      scal(R, 1.0 / nrm, ci);
      for (int j = i + 1; j < l; ++j) {
        double* cj = p_.data() + static_cast<Index>(j) * R;
        axpy(R, -dot(ci, cj, R), ci, cj);
      }
    }
    ap_.resize(R * l);
    Evaluator<T> ev(model_, bbox_, INFINITY, INFINITY);
    ev.set_points(points_dev, mu_, grad_dev_, sigma_);
    DevBuf<double> w(R + l);
    for (int i = 0; i < l; ++i) {
      w.zero();
      copy(w.data(), p_.data() + static_cast<Index>(i) * R, R);
      ev.set_weights(w.data());
      ev.evaluate(ap_.data() + static_cast<Index>(i) * R, false);
    }
  }
  if (verbose()) {
    sync();
    std::printf("ras device setup (lagrange, factors, coarse inverse, AP) %.3f s\n",
                wall_seconds() - t_dev);
  }
  work_res_.resize(rows_);
  work_w_.resize(rows_ + l);
  work_tot_.resize(rows_ + l);
  work_fit_.resize(rows_);
  work_src_w_.resize(rows_ + l);
  sync();
}

// Rows of a fit with gradient points: positions and types on the device, the Lagrange rows,
// u and v over all rows, and A11 among the polynomial rows (with the nugget on value rows).
template <class T>
void RasPreconditioner<T>::setup_rows(const double* points_host, const double* grad_host) {
  const Index R = rows_;
  const int l = l_;
  row_pos_.resize(3 * R);
  row_type_.resize(R);
  rows_kernel<<<blocks_for(R, 256), 256, 0, stream()>>>(points_dev_, mu_, grad_dev_, sigma_,
                                                        row_pos_.data(), row_type_.data());
  PGPU_LAUNCH_CHECK();
  if (l == 0) return;
  auto row_of = [&](Index g, double* p) {
    const double* src = g < mu_ ? points_host + 3 * g : grad_host + 3 * ((g - mu_) / 3);
    p[0] = src[0];
    p[1] = src[1];
    p[2] = src[2];
    return g < mu_ ? -1 : static_cast<int>((g - mu_) % 3);
  };
  std::vector<double> ppos(3 * l);
  std::vector<int> ptype(l);
  for (int k = 0; k < l; ++k) ptype[k] = row_of(poly_rows_[k], ppos.data() + 3 * k);
  const RbfSet rs = rbf_set(model_);
  a11_.assign(l * l, 0.0);
  for (int i = 0; i < l; ++i)
    for (int j = 0; j < l; ++j)
      a11_[i * l + j] = row_entry(rs, ptype[i], ppos.data() + 3 * i, ptype[j], ppos.data() + 3 * j) +
                        ((i == j && ptype[i] < 0) ? model_.nugget : 0.0);
  DevBuf<double> coeffs, dpp, da11;
  DevBuf<int> dpt;
  coeffs.upload(lagrange_coeffs_);
  dpp.upload(ppos);
  dpt.upload(ptype);
  da11.upload(a11_);
  lagrange_.resize(R * l);
  lagrange_rows_kernel<<<blocks_for(R, 256), 256, 0, stream()>>>(l, row_pos_.data(), row_type_.data(),
                                                                 R, coeffs.data(), lagrange_.data());
  PGPU_LAUNCH_CHECK();
  u_.resize(R * l);
  v_.resize(R * l);
  uv_rows_kernel<<<blocks_for(R, 128), 128, 0, stream()>>>(rs, row_pos_.data(), row_type_.data(), R,
                                                           dpp.data(), dpt.data(), l, da11.data(),
                                                           lagrange_.data(), u_.data(), v_.data());
  PGPU_LAUNCH_CHECK();
  sync();
}

// Domains of a fit with gradient points as row lists: the points (polynomial points first),
// then the three rows of each gradient point, each row inheriting its point's inner flag
// (fine_grid.hpp:63-70).
template <class T>
template <class U>
void RasPreconditioner<T>::build_batch_rows(DomainBatch<U>& b, const std::vector<Domain>& domains) {
  std::vector<Index> sizes, pts;
  std::vector<char> inner;
  for (const auto& dom : domains) {
    sizes.push_back(dom.num_points() + 3 * dom.num_grad_points());
    pts.insert(pts.end(), dom.point_indices.begin(), dom.point_indices.end());
    inner.insert(inner.end(), dom.inner_point.begin(), dom.inner_point.end());
    for (Index i = 0; i < dom.num_grad_points(); ++i)
      for (int c = 0; c < 3; ++c) {
        pts.push_back(mu_ + 3 * dom.grad_point_indices[i] + c);
        inner.push_back(dom.inner_grad_point[i]);
      }
  }
  DevBuf<Index> dpts;
  DevBuf<char> dinner;
  dpts.upload(pts);
  dinner.upload(inner);
  build_batch(b, sizes, std::move(dpts), std::move(dinner));
}

template <class T>
void RasPreconditioner<T>::setup_polynomial(const double* points_host, const double* points_dev) {
  const int l = l_;
  if (l > 0) {
    DevBuf<double> coeffs;
    coeffs.upload(lagrange_coeffs_);
    lagrange_.resize(mu_ * l);
    lagrange_kernel<<<blocks_for(mu_, 256), 256, 0, stream()>>>(model_.poly_degree, l, points_dev,
                                                                mu_, coeffs.data(), lagrange_.data());
    PGPU_LAUNCH_CHECK();
    // A11 on the host (l x l, nugget on the diagonal).
    a11_.assign(l * l, 0.0);
    for (int i = 0; i < l; ++i)
      for (int j = 0; j < l; ++j) {
        const double* x = points_host + 3 * poly_idcs_[i];
        const double* y = points_host + 3 * poly_idcs_[j];
        double s = (i == j) ? model_.nugget : 0.0;
        for (const auto& rb : model_.rbfs) {
          double dd[3] = {x[0] - y[0], x[1] - y[1], x[2] - y[2]};
          double t[3];
          for (int r = 0; r < 3; ++r) t[r] = rb.a[3 * r] * dd[0] + rb.a[3 * r + 1] * dd[1] + rb.a[3 * r + 2] * dd[2];
          KParams<double> kp{rb.p[0], rb.p[1]};
          s += dispatch_kind(rb.kind, [&]<int K>() { return rbf_value<K>(t[0] * t[0] + t[1] * t[1] + t[2] * t[2], kp); });
        }
        a11_[i * l + j] = s;
      }
    std::vector<double> pp;
    for (auto i : poly_idcs_)
      for (int k = 0; k < 3; ++k) pp.push_back(points_host[3 * i + k]);
    DevBuf<double> dpp, da11;
    dpp.upload(pp);
    da11.upload(a11_);
    u_.resize(mu_ * l);
    v_.resize(mu_ * l);
    uv_kernel<<<blocks_for(mu_, 128), 128, 0, stream()>>>(rbf_set(model_), points_dev, mu_, dpp.data(),
                                                          l, da11.data(), lagrange_.data(), u_.data(),
                                                          v_.data());
    PGPU_LAUNCH_CHECK();
    sync();
  }
}

// A preconditioner over one domain holding all points (the reference's FineGrid / CoarseGrid
// unit tests, test/preconditioner/test_fine_grid.cpp and test_coarse_grid.cpp): level 1 is that
// domain as a fine-grid domain with the given inner flags, level 0 the same points as the coarse
// grid. The first l entries of `order` are the polynomial points.
template <class T>
RasPreconditioner<T>::RasPreconditioner(const ModelDesc& model, const double* points_host,
                                        const double* points_dev, Index mu,
                                        const std::vector<Index>& order,
                                        const std::vector<char>& inner, bool coarse_inverse)
    : model_(model), l_(model.l()), mu_(mu), rows_(mu), n_levels_(2),
      bbox_(Bbox3::from_host_points(points_host, mu)), points_dev_(points_dev) {
  if (static_cast<Index>(order.size()) != mu || static_cast<Index>(inner.size()) != mu)
    throw_invalid("order and inner must have one entry per point");
  if (mu < l_) throw_invalid("too few points for the polynomial degree");
  point_idcs_.resize(2);
  grad_point_idcs_.resize(2);
  fine_.resize(2);
  poly_idcs_.assign(order.begin(), order.begin() + l_);
  poly_rows_ = poly_idcs_;
  if (l_ > 0) {
    std::vector<double> pp;
    for (auto i : poly_idcs_)
      for (int k = 0; k < 3; ++k) pp.push_back(points_host[3 * i + k]);
    lagrange_coeffs_ = lagrange_coeffs(model_.poly_degree, pp.data(), l_);
  }
  setup_polynomial(points_host, points_dev);
  Domain d;
  d.point_indices = order;
  d.inner_point = inner;
  fine_[1] = std::make_unique<DomainBatch<T>>();
  build_batch(*fine_[1], std::vector<Domain>{d});
  Domain cd;
  cd.point_indices = order;
  cd.inner_point.assign(mu, 1);
  build_batch(coarse_, std::vector<Domain>{cd});
  coarse_n_ = std::max(static_cast<int>(mu) - l_, 0);
  use_coarse_inverse_ = coarse_inverse && coarse_n_ > 0;
  if (use_coarse_inverse_) {
    const int cld = std::max(NB, ((coarse_n_ + NB - 1) / NB) * NB);
    coarse_inv_.resize(static_cast<Index>(coarse_n_) * coarse_n_);
    chol_inverse_kernel<double><<<coarse_n_, 256, cld * sizeof(double), stream()>>>(
        coarse_.mats.data(), cld, coarse_n_, coarse_inv_.data());
    PGPU_LAUNCH_CHECK();
  }
  coarse_x_.resize(std::max(coarse_n_, 1));
  coarse_g_.resize(std::max(coarse_n_, 1));
  coarse_out_.resize(48);
  coarse_out_.zero();
  sync();
}

template <class T>
void RasPreconditioner<T>::solve_domain(bool coarse, const double* residuals, double* weights) {
  solve_level(coarse ? 0 : 1, residuals, weights);
}

template <class T>
RasPreconditioner<T>::~RasPreconditioner() = default;

template <class T>
Index RasPreconditioner<T>::n_domains() const {
  Index s = 0;
  for (const auto& f : fine_)
    if (f) s += f->n_dom;
  return s;
}

template <class T>
template <class U>
void RasPreconditioner<T>::build_batch(DomainBatch<U>& b, const std::vector<Domain>& domains) {
  std::vector<Index> sizes, pts;
  std::vector<char> inner;
  for (const auto& dom : domains) {
    sizes.push_back(dom.num_points());
    pts.insert(pts.end(), dom.point_indices.begin(), dom.point_indices.end());
    inner.insert(inner.end(), dom.inner_point.begin(), dom.inner_point.end());
  }
  DevBuf<Index> dpts;
  DevBuf<char> dinner;
  dpts.upload(pts);
  dinner.upload(inner);
  build_batch(b, sizes, std::move(dpts), std::move(dinner));
}

template <class T>
template <class U>
void RasPreconditioner<T>::build_batch(DomainBatch<U>& b, const std::vector<Index>& sizes,
                                       DevBuf<Index>&& pts, DevBuf<char>&& inner) {
  const int l = l_;
  b.n_dom = static_cast<Index>(sizes.size());
  std::vector<int> n(b.n_dom), ld(b.n_dom);
  std::vector<Index> mat_off(b.n_dom + 1), pt_off(b.n_dom + 1);
  Index moff = 0, poff = 0;
  b.max_n = 0;
  for (Index d = 0; d < b.n_dom; ++d) {
    const int m = static_cast<int>(sizes[d]);
    n[d] = std::max(m - l, 0);
    ld[d] = std::max(NB, ((n[d] + NB - 1) / NB) * NB);
    b.max_n = std::max(b.max_n, ld[d]);
    mat_off[d] = moff;
    moff += static_cast<Index>(ld[d]) * ld[d];
    b.factor_flops += static_cast<double>(n[d]) * n[d] * n[d] / 3.0;
    b.solve_bytes += static_cast<double>(n[d]) * n[d] * sizeof(U);  // two triangle sweeps
    pt_off[d] = poff;
    poff += m;
  }
  if (static_cast<Index>(pts.size()) != poff || static_cast<Index>(inner.size()) != poff)
    throw_runtime("domain point lists do not match the domain sizes");
  mat_off[b.n_dom] = moff;
  pt_off[b.n_dom] = poff;
  b.total_points = poff;
  b.n.upload(n);
  b.ld.upload(ld);
  b.mat_off.upload(mat_off);
  b.pt_off.upload(pt_off);
  b.pts = std::move(pts);
  b.inner = std::move(inner);
  b.mats.resize(moff);
  b.info.resize(b.n_dom);
  b.info.zero();
  if (b.n_dom == 0) return;

  // Assembly, one pass per RBF in its own frame (fits with gradient points: one pass over the
  // rows with every RBF).
  ProfScope ps(sizeof(U) == 4 ? "ras_factor_f32" : "ras_factor_f64", b.factor_flops);
  const int nbmax = b.max_n / NB;
  const Index ntiles = static_cast<Index>(nbmax) * (nbmax + 1) / 2;
  if (sigma_ > 0) {
    const int tiles_in_x = b.n_dom <= 65535 ? 1 : 0;
    if (!tiles_in_x && ntiles > 65535) throw_runtime("domain too large for the batched assembly");
    const dim3 grid = tiles_in_x ? dim3(static_cast<unsigned>(ntiles), static_cast<unsigned>(b.n_dom))
                                 : dim3(static_cast<unsigned>(b.n_dom), static_cast<unsigned>(ntiles));
    assemble_rows_kernel<U><<<grid, 256, 0, stream()>>>(
        rbf_set(model_), row_pos_.data(), row_type_.data(), b.n.data(), b.ld.data(),
        b.mat_off.data(), b.mats.data(), b.pt_off.data(), b.pts.data(), l, model_.nugget,
        lagrange_.data(), u_.data(), v_.data(), tiles_in_x);
    PGPU_LAUNCH_CHECK();
  }
  for (size_t r = 0; r < model_.rbfs.size() && sigma_ == 0; ++r) {
    const auto& rb = model_.rbfs[r];
    Mat3 a;
    for (int k = 0; k < 9; ++k) a.a[k] = rb.a[k];
    double tmin[3] = {INFINITY, INFINITY, INFINITY}, tmax[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int c = 0; c < 8; ++c) {
      double p[3] = {(c & 1) ? bbox_.max[0] : bbox_.min[0], (c & 2) ? bbox_.max[1] : bbox_.min[1],
                     (c & 4) ? bbox_.max[2] : bbox_.min[2]};
      for (int q = 0; q < 3; ++q) {
        double v = a.a[3 * q] * p[0] + a.a[3 * q + 1] * p[1] + a.a[3 * q + 2] * p[2];
        tmin[q] = std::min(tmin[q], v);
        tmax[q] = std::max(tmax[q], v);
      }
    }
    double o[3];
    for (int q = 0; q < 3; ++q) o[q] = bbox_.empty() ? 0.0 : 0.5 * (tmin[q] + tmax[q]);
    DevBuf<P4<U>> frame(mu_);
    frame_kernel<U><<<blocks_for(mu_, 256), 256, 0, stream()>>>(points_dev_, mu_, a, o[0], o[1], o[2],
                                                                frame.data());
    PGPU_LAUNCH_CHECK();
    KParams<U> kp{static_cast<U>(rb.p[0]), static_cast<U>(rb.p[1])};
    const int first = r == 0, last = r + 1 == model_.rbfs.size();
    const int tiles_in_x = b.n_dom <= 65535 ? 1 : 0;
    if (!tiles_in_x && ntiles > 65535) throw_runtime("domain too large for the batched assembly");
    const dim3 grid = tiles_in_x ? dim3(static_cast<unsigned>(ntiles), static_cast<unsigned>(b.n_dom))
                                 : dim3(static_cast<unsigned>(b.n_dom), static_cast<unsigned>(ntiles));
    dispatch_kind(rb.kind, [&]<int K>() {
      assemble_kernel<U, K><<<grid, 256, 0, stream()>>>(
          kp, frame.data(), b.n.data(), b.ld.data(), b.mat_off.data(), b.mats.data(),
          b.pt_off.data(), b.pts.data(), l, first, last, model_.nugget, lagrange_.data(),
          u_.data(), v_.data(), tiles_in_x);
      return 0;
    });
    PGPU_LAUNCH_CHECK();
  }

  DevBuf<int> tc_err;  // timeout flag of the tensor-core trailing updates
  // Blocked Cholesky over all domains, in groups of kGroup panels: inside a group each panel is
  // updated left-looking by the group's earlier panels, factored and solved below; then one
  // trailing update applies the whole group.
  constexpr int kGroup = 4;
  const unsigned nd = static_cast<unsigned>(b.n_dom);
  for (int g0 = 0; g0 < nbmax; g0 += kGroup) {
    const int np = std::min(kGroup, nbmax - g0);
    for (int p = 0; p < np; ++p) {
      const int kb = g0 + p;
      if (p > 0) {
        if (std::is_same_v<U, float> && nd <= 65535) {
          const int gx = (b.max_n - kb * NB + kTile - 1) / kTile;
          panel_update_kernel<<<dim3(static_cast<unsigned>(gx), nd), 256, kPanelSmem, stream()>>>(
              g0, p, b.ld.data(), b.mat_off.data(), reinterpret_cast<float*>(b.mats.data()));
        } else {
          syrk_update_kernel<U><<<dim3(nd, static_cast<unsigned>(nbmax - kb)), 256, 0, stream()>>>(
              g0, p, 1, b.ld.data(), b.mat_off.data(), b.mats.data());
        }
        PGPU_LAUNCH_CHECK();
      }
      potrf_diag_kernel<U><<<nd, 128, 0, stream()>>>(kb, b.ld.data(), b.mat_off.data(),
                                                    b.mats.data(), b.info.data());
      PGPU_LAUNCH_CHECK();
      const int rows_below = b.max_n - (kb + 1) * NB;
      if (rows_below <= 0) continue;
      dim3 gp(nd, static_cast<unsigned>((rows_below + 127) / 128));
      trsm_panel_kernel<U><<<gp, 128, 0, stream()>>>(kb, b.ld.data(), b.mat_off.data(), b.mats.data());
      PGPU_LAUNCH_CHECK();
    }
    const int rem = nbmax - g0 - np;
    if (rem <= 0) continue;
    if (std::is_same_v<U, float> && nd <= 65535 && syrk_tc_enabled()) {
      const int nt = (rem * NB + kTile - 1) / kTile;
      dim3 gs(static_cast<unsigned>(nt * (nt + 1) / 2), nd);
      static std::once_flag attr_flag;
      std::call_once(attr_flag, [] {
        PGPU_CUDA(cudaFuncSetAttribute(syrk_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(kSyrkTcSmem)));
      });
      if (tc_err.size() == 0) {
        tc_err.resize(1);
        tc_err.zero();
      }
      syrk_tc_kernel<<<gs, 128, kSyrkTcSmem, stream()>>>(
          g0, np, b.ld.data(), b.mat_off.data(), reinterpret_cast<float*>(b.mats.data()),
          tc_err.data());
    } else if (std::is_same_v<U, float> && nd <= 65535) {
      const int nt = (rem * NB + kTile - 1) / kTile;
      dim3 gs(static_cast<unsigned>(nt * (nt + 1) / 2), nd);
      syrk128_update_kernel<<<gs, 256, kSyrk128Smem, stream()>>>(
          g0, np, b.ld.data(), b.mat_off.data(), reinterpret_cast<float*>(b.mats.data()));
    } else {
      const int rem2 = (rem + 1) / 2;
      dim3 gs(nd, static_cast<unsigned>(static_cast<Index>(rem2) * (rem2 + 1) / 2));
      syrk64_update_kernel<U><<<gs, 256, 0, stream()>>>(g0, np, b.ld.data(), b.mat_off.data(),
                                                        b.mats.data());
    }
    PGPU_LAUNCH_CHECK();
  }
  invert_diag_kernel<U><<<dim3(static_cast<unsigned>(b.n_dom), nbmax), 32, 0, stream()>>>(
      b.ld.data(), b.mat_off.data(), b.mats.data());
  PGPU_LAUNCH_CHECK();
  if (tc_err.size() > 0) {
    int e = 0;
    PGPU_CUDA(cudaMemcpyAsync(&e, tc_err.data(), sizeof(int), cudaMemcpyDeviceToHost, stream()));
    sync();
    if (e != 0) throw Error(PGPU_TIMEOUT, "tensor-core Cholesky update: a bounded wait ran out");
  }
}

template <class T>
void RasPreconditioner<T>::solve_level(int level, const double* residuals, double* weights) {
  fill(weights, rows_ + l_, 0.0);
  if (level > 0) {
    DomainBatch<T>& b = *fine_[level];
    if (b.n_dom == 0) return;
    const size_t smem = (static_cast<size_t>(b.max_n) + 16 + 64) * sizeof(double);
    ProfScope ps(sizeof(T) == 4 ? "ras_solve_f32" : "ras_solve_f64",
                 2.0 * b.solve_bytes / sizeof(T), b.solve_bytes);
    ras_solve_kernel<T><<<static_cast<unsigned>(b.n_dom), 256, smem, stream()>>>(
        b.n.data(), b.ld.data(), b.mat_off.data(), b.mats.data(), b.pt_off.data(), b.pts.data(),
        b.inner.data(), l_, lagrange_.data(), u_.data(), residuals, weights, 0, nullptr);
    PGPU_LAUNCH_CHECK();
    return;
  }
  // Coarse grid (coarse_grid.hpp:91-131): gamma = (Q^T A Q)^{-1} Q^T d with the explicit FP64
  // inverse, lambda = Q gamma on every coarse point, then the polynomial coefficients.
  const int n = coarse_n_, l = l_;
  const Index* dp = coarse_.pts.data();
  ProfScope ps("ras_coarse_f64", 2.0 * n * static_cast<double>(n), 8.0 * n * static_cast<double>(n));
  coarse_rhs_kernel<<<blocks_for(std::max(n, 1), 256), 256, 0, stream()>>>(
      dp, n, l, lagrange_.data(), residuals, coarse_x_.data(), coarse_out_.data() + 32);
  PGPU_LAUNCH_CHECK();
  if (use_coarse_inverse_) {
    symv_kernel<<<blocks_for(static_cast<Index>(n) * 32, 256), 256, 0, stream()>>>(
        coarse_inv_.data(), n, coarse_x_.data(), coarse_g_.data());
    PGPU_LAUNCH_CHECK();
    coarse_finish_kernel<<<1, 256, 0, stream()>>>(dp, n, l, lagrange_.data(), u_.data(),
                                                  coarse_g_.data(), weights, coarse_out_.data());
    PGPU_LAUNCH_CHECK();
  } else {
    const size_t smem = (static_cast<size_t>(coarse_.max_n) + 16 + 64) * sizeof(double);
    ras_solve_kernel<double><<<1, 256, smem, stream()>>>(
        coarse_.n.data(), coarse_.ld.data(), coarse_.mat_off.data(), coarse_.mats.data(),
        coarse_.pt_off.data(), coarse_.pts.data(), coarse_.inner.data(), l, lagrange_.data(),
        u_.data(), residuals, weights, 1, coarse_out_.data());
    PGPU_LAUNCH_CHECK();
  }
  if (l > 0) {
    // Polynomial part: solve P_top c = d_head - A_top lambda (coarse_grid.hpp:124-127).
    double h[48];
    PGPU_CUDA(cudaMemcpyAsync(h, coarse_out_.data(), 48 * sizeof(double), cudaMemcpyDeviceToHost,
                              stream()));
    sync();
    std::vector<double> rhs(l);
    for (int k = 0; k < l; ++k) {
      double a_lambda = h[16 + k];
      for (int j = 0; j < l; ++j) a_lambda += a11_[k * l + j] * h[j];
      rhs[k] = h[32 + k] - a_lambda;
    }
    // c = P_top^{-1} rhs; lagrange_coeffs_ holds P_top^{-1} (row-major).
    std::vector<double> c(l, 0.0);
    for (int i = 0; i < l; ++i)
      for (int k = 0; k < l; ++k) c[i] += lagrange_coeffs_[i * l + k] * rhs[k];
    PGPU_CUDA(cudaMemcpyAsync(weights + rows_, c.data(), l * sizeof(double), cudaMemcpyHostToDevice,
                              stream()));
    sync();
  }
}

template <class T>
Evaluator<T>& RasPreconditioner<T>::evaluator(int src_level, int trg_level) {
  auto key = std::make_pair(src_level, trg_level);
  auto it = evaluators_.find(key);
  if (it == evaluators_.end()) {
    auto ev = std::make_unique<Evaluator<T>>(model_, bbox_, INFINITY, INFINITY);
    ev->set_sources(level_pts_dev_[src_level].data(),
                    static_cast<Index>(point_idcs_[src_level].size()),
                    level_grad_pts_dev_[src_level].data(),
                    static_cast<Index>(grad_point_idcs_[src_level].size()));
    ev->set_targets(level_pts_dev_[trg_level].data(),
                    static_cast<Index>(point_idcs_[trg_level].size()),
                    level_grad_pts_dev_[trg_level].data(),
                    static_cast<Index>(grad_point_idcs_[trg_level].size()));
    it = evaluators_.emplace(key, std::move(ev)).first;
  }
  return *it->second;
}

template <class T>
void RasPreconditioner<T>::update_residuals(int src_level, int trg_level, const double* weights,
                                            double* residuals) {
  const Index ns = static_cast<Index>(point_idcs_[src_level].size() + 3 * grad_point_idcs_[src_level].size());
  const Index nt = static_cast<Index>(point_idcs_[trg_level].size() + 3 * grad_point_idcs_[trg_level].size());
  gather(weights, level_idx_dev_[src_level].data(), ns, work_src_w_.data());
  if (l_ > 0) copy(work_src_w_.data() + ns, weights + rows_, l_);
  auto& ev = evaluator(src_level, trg_level);
  ev.set_weights(work_src_w_.data());
  ev.evaluate(work_fit_.data());
  scal(nt, -1.0, work_fit_.data());
  scatter_add(work_fit_.data(), level_idx_dev_[trg_level].data(), nt, residuals);
}

template <class T>
void RasPreconditioner<T>::orthogonalize(double* weights, double* residuals) {
  if (l_ == 0) return;
  std::vector<double> dotv(l_);
  tall_gemv_t(p_.data(), rows_, l_, weights, dotv.data());
  std::vector<double> neg(l_);
  for (int k = 0; k < l_; ++k) neg[k] = -dotv[k];
  tall_gemv_add(p_.data(), rows_, l_, neg.data(), weights);
  tall_gemv_add(ap_.data(), rows_, l_, dotv.data(), residuals);
}

template <class T>
void RasPreconditioner<T>::apply(const double* v, double* out) {
  double* r = work_res_.data();
  const Index M = rows_ + l_;
  copy(r, v, rows_);
  if (n_levels_ == 1) {
    solve_level(0, r, out);
    return;
  }
  double* w = work_w_.data();
  double* tot = out;
  fill(tot, M, 0.0);
  const int L = n_levels_;
  solve_level(0, r, w);
  update_residuals(0, L - 1, w, r);
  axpy(M, 1.0, w, tot);
  for (int level = 1; level < L - 1; ++level) {
    solve_level(level, r, w);
    update_residuals(level, L - 1, w, r);
    axpy(M, 1.0, w, tot);
    orthogonalize(tot, r);
    solve_level(0, r, w);
    update_residuals(0, L - 1, w, r);
    axpy(M, 1.0, w, tot);
  }
  for (int level = L - 1; level >= 1; --level) {
    solve_level(level, r, w);
    update_residuals(level, level - 1, w, r);
    axpy(M, 1.0, w, tot);
    orthogonalize(tot, r);
    solve_level(0, r, w);
    if (level > 1) update_residuals(0, level - 1, w, r);
    axpy(M, 1.0, w, tot);
  }
}

template <class T>
static void ras_domain_solve_t(const ModelDesc& model, const double* points, Index n,
                               const std::vector<Index>& order, const std::vector<char>& inner,
                               bool coarse, bool use_inverse, const double* rhs, double* out) {
  DevBuf<double> pts, r, w;
  pts.upload(points, static_cast<size_t>(3 * n));
  r.upload(rhs, n);
  w.resize(n + model.l());
  RasPreconditioner<T> ras(model, points, pts.data(), n, order, inner, use_inverse);
  ras.solve_domain(coarse, r.data(), w.data());
  w.download(out, n + model.l());
  sync();
}

template class RasPreconditioner<double>;
template class RasPreconditioner<float>;

void ras_domain_solve(const ModelDesc& model, const double* points, Index n, const Index* order,
                      const unsigned char* inner, bool coarse, bool use_inverse, bool mixed,
                      const double* rhs, double* out) {
  std::vector<Index> ord(order, order + n);
  std::vector<char> seen(n, 0);
  for (Index i : ord) {
    if (i < 0 || i >= n || seen[i]) throw_invalid("order must be a permutation of 0 .. n-1");
    seen[i] = 1;
  }
  std::vector<char> inn(inner, inner + n);
  if (mixed)
    ras_domain_solve_t<float>(model, points, n, ord, inn, coarse, use_inverse, rhs, out);
  else
    ras_domain_solve_t<double>(model, points, n, ord, inn, coarse, use_inverse, rhs, out);
}

}  // namespace pgpu
