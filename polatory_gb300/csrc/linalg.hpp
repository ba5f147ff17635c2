// Device vector kernels: fused Krylov (multi-dot, multi-axpy + norm), reductions and small
// tall-skinny products. All reductions are two-stage with a fixed order (deterministic).
#pragma once

#include "common.hpp"

namespace pgpu {

// out_host[i] = V_i . w for i < k, V_i = V + i * ld (FP64). One pass over the k vectors.
void multi_dot(const double* V, Index ld, int k, const double* w, Index n, double* out_host);
// w -= sum_i h[i] V_i ; returns ||w||_2^2 (one pass).
double multi_axpy_sub_norm2(const double* V, Index ld, int k, const double* h, double* w, Index n);
// x += sum_i y[i] Z_i.
void multi_axpy(const double* Z, Index ld, int k, const double* y, double* x, Index n);
// y = A x for a dense row-major n x n matrix (one warp per row).
void dense_gemv(const double* A, Index n, const double* x, double* y);
// Generic helpers.
double dot(const double* x, const double* y, Index n);
double norm2(const double* x, Index n);
double inf_norm_diff(const double* x, const double* y, Index n);  // max |x - y|
void axpy(Index n, double a, const double* x, double* y);        // y += a x
void axpby(Index n, double a, const double* x, double b, double* y);  // y = a x + b y
void scal(Index n, double a, double* x);
void fill(double* x, Index n, double v);
void copy(double* dst, const double* src, Index n);
// dst[i] = src[idx[i]]
void gather(const double* src, const Index* idx, Index n, double* dst);
// dst[idx[i]] = src[i]
void scatter(const double* src, const Index* idx, Index n, double* dst);
// dst[idx[i]] += src[i]
void scatter_add(const double* src, const Index* idx, Index n, double* dst);
// Tall-skinny products with P (rows x l, column-major, ld = rows):
//   y += P c     and    out_host = P^T v
void tall_gemv_add(const double* P, Index rows, int l, const double* c_host, double* y);
void tall_gemv_t(const double* P, Index rows, int l, const double* v, double* out_host);

// Monomial basis (polynomial/monomial_basis.hpp:31-262, 3-D column order 1,x,y,z,x^2,xy,xz,
// y^2,yz,z^2): P has mu + 3 sigma rows; gradient rows are d/dx, d/dy, d/dz.
void monomial_basis(int degree, const double* pts, Index mu, const double* gpts, Index sigma,
                    double* P);
// out[i] += sum_k P_k(x_i) c_k (value rows) and the gradient rows for grad points.
void poly_eval_add(int degree, const double* c_host, const double* pts, Index mu,
                   const double* gpts, Index sigma, double* out);

}  // namespace pgpu
