// Device vector kernels. The Krylov kernels are HBM-bound: multi_dot reads each basis vector
// once (the w segment of a block stays in shared memory), multi_axpy_sub_norm2 reads the basis
// and w once and writes w once, folding the norm into the same pass (src/krylov/gmres.cpp:20-31).
#include "common.hpp"
#include "linalg.hpp"
#include "profile.hpp"

namespace pgpu {

namespace {

constexpr int kRedThreads = 256;
constexpr int kSeg = 2048;  // rows per block in multi_dot (16 KB of w in shared memory)

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum with a fixed combination order; result valid in thread 0.
__device__ __forceinline__ double block_sum(double v, double* sh) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double r = 0;
  if (threadIdx.x < 32) {
    r = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    r = warp_sum(r);
  }
  return r;
}

__global__ void multi_dot_kernel(const double* __restrict__ V, Index ld, int k,
                                 const double* __restrict__ w, Index n,
                                 double* __restrict__ part) {
  __shared__ double sw[kSeg];
  __shared__ double sh[32];
  const Index beg = static_cast<Index>(blockIdx.x) * kSeg;
  const int cnt = static_cast<int>(min(static_cast<Index>(kSeg), n - beg));
  for (int r = threadIdx.x; r < cnt; r += blockDim.x) sw[r] = w[beg + r];
  __syncthreads();
  for (int i = 0; i < k; ++i) {
    const double* v = V + static_cast<Index>(i) * ld + beg;
    double s = 0;
    for (int r = threadIdx.x; r < cnt; r += blockDim.x) s += v[r] * sw[r];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) part[static_cast<Index>(i) * gridDim.x + blockIdx.x] = s;
  }
}

__global__ void reduce_rows_kernel(const double* __restrict__ part, int nblk, int k,
                                   double* __restrict__ out) {
  __shared__ double sh[32];
  const int i = blockIdx.x;
  double s = 0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) s += part[static_cast<Index>(i) * nblk + b];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) out[i] = s;
}

__global__ void multi_axpy_sub_norm2_kernel(const double* __restrict__ V, Index ld, int k,
                                            const double* __restrict__ h, double* __restrict__ w,
                                            Index n, double* __restrict__ part, double sign,
                                            int want_norm) {
  __shared__ double sh[32];
  __shared__ double shh[256];
  for (int i = threadIdx.x; i < k; i += blockDim.x) shh[i] = h[i];
  __syncthreads();
  double s = 0;
  for (Index r = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x; r < n;
       r += static_cast<Index>(gridDim.x) * blockDim.x) {
    double acc = w[r];
    for (int i = 0; i < k; ++i) acc += sign * shh[i] * V[static_cast<Index>(i) * ld + r];
    w[r] = acc;
    s += acc * acc;
  }
  if (want_norm) {
    s = block_sum(s, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
  }
}

__global__ void dot_kernel(const double* __restrict__ x, const double* __restrict__ y, Index n,
                           double* __restrict__ part, int mode) {
  __shared__ double sh[32];
  double s = 0;
  for (Index r = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x; r < n;
       r += static_cast<Index>(gridDim.x) * blockDim.x) {
    if (mode == 0) s += x[r] * y[r];
    else s = fmax(s, fabs(x[r] - y[r]));
  }
  if (mode == 0) {
    s = block_sum(s, sh);
  } else {
    for (int o = 16; o > 0; o >>= 1) s = fmax(s, __shfl_xor_sync(0xffffffffu, s, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
      s = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
      for (int o = 16; o > 0; o >>= 1) s = fmax(s, __shfl_xor_sync(0xffffffffu, s, o));
    }
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void axpby_kernel(Index n, double a, const double* __restrict__ x, double b,
                             double* __restrict__ y) {
  Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) y[i] = a * x[i] + b * y[i];
}

__global__ void fill_kernel(double* x, Index n, double v) {
  Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) x[i] = v;
}

__global__ void gather_kernel(const double* __restrict__ src, const Index* __restrict__ idx,
                              Index n, double* __restrict__ dst) {
  Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[idx[i]];
}

__global__ void scatter_kernel(const double* __restrict__ src, const Index* __restrict__ idx,
                               Index n, double* __restrict__ dst, int add) {
  Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) {
    if (add) dst[idx[i]] += src[i];
    else dst[idx[i]] = src[i];
  }
}

struct SmallVec {
  double v[16];
};

__global__ void tall_gemv_add_kernel(const double* __restrict__ P, Index rows, int l, SmallVec c,
                                     double* __restrict__ y) {
  Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= rows) return;
  double s = 0;
  for (int k = 0; k < l; ++k) s += P[static_cast<Index>(k) * rows + i] * c.v[k];
  y[i] += s;
}

// Evaluates monomials (and their gradients) of degree <= 2 at a point.
__device__ __forceinline__ void monomials(int degree, double x, double y, double z, double* m) {
  m[0] = 1.0;
  if (degree >= 1) {
    m[1] = x;
    m[2] = y;
    m[3] = z;
  }
  if (degree >= 2) {
    m[4] = x * x;
    m[5] = x * y;
    m[6] = x * z;
    m[7] = y * y;
    m[8] = y * z;
    m[9] = z * z;
  }
}

__device__ __forceinline__ void monomial_grads(int degree, double x, double y, double z,
                                               double* gx, double* gy, double* gz) {
  gx[0] = gy[0] = gz[0] = 0.0;
  if (degree >= 1) {
    gx[1] = 1.0; gy[1] = 0.0; gz[1] = 0.0;
    gx[2] = 0.0; gy[2] = 1.0; gz[2] = 0.0;
    gx[3] = 0.0; gy[3] = 0.0; gz[3] = 1.0;
  }
  if (degree >= 2) {
    gx[4] = 2.0 * x; gy[4] = 0.0;     gz[4] = 0.0;
    gx[5] = y;       gy[5] = x;       gz[5] = 0.0;
    gx[6] = z;       gy[6] = 0.0;     gz[6] = x;
    gx[7] = 0.0;     gy[7] = 2.0 * y; gz[7] = 0.0;
    gx[8] = 0.0;     gy[8] = z;       gz[8] = y;
    gx[9] = 0.0;     gy[9] = 0.0;     gz[9] = 2.0 * z;
  }
}

__global__ void monomial_basis_kernel(int degree, int l, const double* __restrict__ pts, Index mu,
                                      const double* __restrict__ gpts, Index sigma,
                                      double* __restrict__ P) {
  Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  const Index rows = mu + 3 * sigma;
  if (i < mu) {
    double m[10];
    monomials(degree, pts[3 * i], pts[3 * i + 1], pts[3 * i + 2], m);
    for (int k = 0; k < l; ++k) P[static_cast<Index>(k) * rows + i] = m[k];
  } else if (i < mu + sigma) {
    Index j = i - mu;
    double gx[10], gy[10], gz[10];
    monomial_grads(degree, gpts[3 * j], gpts[3 * j + 1], gpts[3 * j + 2], gx, gy, gz);
    for (int k = 0; k < l; ++k) {
      P[static_cast<Index>(k) * rows + mu + 3 * j] = gx[k];
      P[static_cast<Index>(k) * rows + mu + 3 * j + 1] = gy[k];
      P[static_cast<Index>(k) * rows + mu + 3 * j + 2] = gz[k];
    }
  }
}

__global__ void poly_eval_add_kernel(int degree, int l, SmallVec c, const double* __restrict__ pts,
                                     Index mu, const double* __restrict__ gpts, Index sigma,
                                     double* __restrict__ out) {
  Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < mu) {
    double m[10];
    monomials(degree, pts[3 * i], pts[3 * i + 1], pts[3 * i + 2], m);
    double s = 0;
    for (int k = 0; k < l; ++k) s += m[k] * c.v[k];
    out[i] += s;
  } else if (i < mu + sigma) {
    Index j = i - mu;
    double gx[10], gy[10], gz[10];
    monomial_grads(degree, gpts[3 * j], gpts[3 * j + 1], gpts[3 * j + 2], gx, gy, gz);
    double sx = 0, sy = 0, sz = 0;
    for (int k = 0; k < l; ++k) {
      sx += gx[k] * c.v[k];
      sy += gy[k] * c.v[k];
      sz += gz[k] * c.v[k];
    }
    out[mu + 3 * j] += sx;
    out[mu + 3 * j + 1] += sy;
    out[mu + 3 * j + 2] += sz;
  }
}

int reduce_blocks(Index n) {
  Index b = (n + kRedThreads - 1) / kRedThreads;
  Index cap = 4 * num_sms();
  if (b > cap) b = cap;
  return static_cast<int>(b < 1 ? 1 : b);
}

double finish_reduce(const DevBuf<double>& part, int nblk, int mode) {
  std::vector<double> h(nblk);
  part.download(h.data(), nblk);
  sync();
  double s = 0;
  for (int b = 0; b < nblk; ++b) {
    if (mode == 0) s += h[b];
    else s = std::max(s, h[b]);
  }
  return s;
}

}  // namespace

void multi_dot(const double* V, Index ld, int k, const double* w, Index n, double* out_host) {
  if (k == 0) return;
  const int nblk = blocks_for(n, kSeg);
  DevBuf<double> part(static_cast<size_t>(nblk) * k);
  DevBuf<double> out(k);
  ProfScope ps("krylov_multidot", 2.0 * k * n, (k + 1.0) * n * sizeof(double));
  multi_dot_kernel<<<nblk, kRedThreads, 0, stream()>>>(V, ld, k, w, n, part.data());
  PGPU_LAUNCH_CHECK();
  reduce_rows_kernel<<<k, kRedThreads, 0, stream()>>>(part.data(), nblk, k, out.data());
  PGPU_LAUNCH_CHECK();
  out.download(out_host, k);
  sync();
}

double multi_axpy_sub_norm2(const double* V, Index ld, int k, const double* h, double* w,
                            Index n) {
  if (k > 256) throw_runtime("multi_axpy: too many vectors");
  DevBuf<double> dh;
  dh.upload(h, k);
  const int nblk = reduce_blocks(n);
  DevBuf<double> part(nblk);
  ProfScope ps("krylov_axpy_norm", 2.0 * (k + 1) * n, (k + 2.0) * n * sizeof(double));
  multi_axpy_sub_norm2_kernel<<<nblk, kRedThreads, 0, stream()>>>(V, ld, k, dh.data(), w, n,
                                                                  part.data(), -1.0, 1);
  PGPU_LAUNCH_CHECK();
  return finish_reduce(part, nblk, 0);
}

void multi_axpy(const double* Z, Index ld, int k, const double* y, double* x, Index n) {
  if (k == 0) return;
  if (k > 256) throw_runtime("multi_axpy: too many vectors");
  DevBuf<double> dy;
  dy.upload(y, k);
  const int nblk = reduce_blocks(n);
  ProfScope ps("krylov_solution", 2.0 * k * n, (k + 2.0) * n * sizeof(double));
  multi_axpy_sub_norm2_kernel<<<nblk, kRedThreads, 0, stream()>>>(Z, ld, k, dy.data(), x, n,
                                                                  nullptr, 1.0, 0);
  PGPU_LAUNCH_CHECK();
}

double dot(const double* x, const double* y, Index n) {
  if (n == 0) return 0.0;
  const int nblk = reduce_blocks(n);
  DevBuf<double> part(nblk);
  dot_kernel<<<nblk, kRedThreads, 0, stream()>>>(x, y, n, part.data(), 0);
  PGPU_LAUNCH_CHECK();
  return finish_reduce(part, nblk, 0);
}

double norm2(const double* x, Index n) { return std::sqrt(dot(x, x, n)); }

double inf_norm_diff(const double* x, const double* y, Index n) {
  if (n == 0) return 0.0;
  const int nblk = reduce_blocks(n);
  DevBuf<double> part(nblk);
  dot_kernel<<<nblk, kRedThreads, 0, stream()>>>(x, y, n, part.data(), 1);
  PGPU_LAUNCH_CHECK();
  return finish_reduce(part, nblk, 1);
}

void axpy(Index n, double a, const double* x, double* y) { axpby(n, a, x, 1.0, y); }

void axpby(Index n, double a, const double* x, double b, double* y) {
  if (n == 0) return;
  axpby_kernel<<<blocks_for(n, 256), 256, 0, stream()>>>(n, a, x, b, y);
  PGPU_LAUNCH_CHECK();
}

void scal(Index n, double a, double* x) { axpby(n, 0.0, x, a, x); }

void fill(double* x, Index n, double v) {
  if (n == 0) return;
  fill_kernel<<<blocks_for(n, 256), 256, 0, stream()>>>(x, n, v);
  PGPU_LAUNCH_CHECK();
}

void copy(double* dst, const double* src, Index n) {
  if (n == 0) return;
  PGPU_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToDevice, stream()));
}

void gather(const double* src, const Index* idx, Index n, double* dst) {
  if (n == 0) return;
  gather_kernel<<<blocks_for(n, 256), 256, 0, stream()>>>(src, idx, n, dst);
  PGPU_LAUNCH_CHECK();
}

void scatter(const double* src, const Index* idx, Index n, double* dst) {
  if (n == 0) return;
  scatter_kernel<<<blocks_for(n, 256), 256, 0, stream()>>>(src, idx, n, dst, 0);
  PGPU_LAUNCH_CHECK();
}

void scatter_add(const double* src, const Index* idx, Index n, double* dst) {
  if (n == 0) return;
  scatter_kernel<<<blocks_for(n, 256), 256, 0, stream()>>>(src, idx, n, dst, 1);
  PGPU_LAUNCH_CHECK();
}

void tall_gemv_add(const double* P, Index rows, int l, const double* c_host, double* y) {
  if (rows == 0 || l == 0) return;
  SmallVec c{};
  for (int k = 0; k < l; ++k) c.v[k] = c_host[k];
  tall_gemv_add_kernel<<<blocks_for(rows, 256), 256, 0, stream()>>>(P, rows, l, c, y);
  PGPU_LAUNCH_CHECK();
}

void tall_gemv_t(const double* P, Index rows, int l, const double* v, double* out_host) {
  if (l == 0) return;
  if (rows == 0) {
    for (int k = 0; k < l; ++k) out_host[k] = 0.0;
    return;
  }
  multi_dot(P, rows, l, v, rows, out_host);
}

void monomial_basis(int degree, const double* pts, Index mu, const double* gpts, Index sigma,
                    double* P) {
  int l = degree < 0 ? 0 : (degree + 1) * (degree + 2) * (degree + 3) / 6;
  if (l == 0 || mu + sigma == 0) return;
  monomial_basis_kernel<<<blocks_for(mu + sigma, 256), 256, 0, stream()>>>(degree, l, pts, mu,
                                                                           gpts, sigma, P);
  PGPU_LAUNCH_CHECK();
}

void poly_eval_add(int degree, const double* c_host, const double* pts, Index mu,
                   const double* gpts, Index sigma, double* out) {
  int l = degree < 0 ? 0 : (degree + 1) * (degree + 2) * (degree + 3) / 6;
  if (l == 0 || mu + sigma == 0) return;
  SmallVec c{};
  for (int k = 0; k < l; ++k) c.v[k] = c_host[k];
  poly_eval_add_kernel<<<blocks_for(mu + sigma, 256), 256, 0, stream()>>>(degree, l, c, pts, mu,
                                                                          gpts, sigma, out);
  PGPU_LAUNCH_CHECK();
}

namespace {
__global__ void dense_gemv_kernel(const double* __restrict__ a, Index n, const double* __restrict__ x,
                                  double* __restrict__ y) {
  const Index row = (static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  double s = 0;
  for (Index j = lane; j < n; j += 32) s += a[row * n + j] * x[j];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) y[row] = s;
}
}  // namespace

void dense_gemv(const double* A, Index n, const double* x, double* y) {
  if (n <= 0) return;
  dense_gemv_kernel<<<blocks_for(32 * n, 256), 256, 0, stream()>>>(A, n, x, y);
  PGPU_LAUNCH_CHECK();
}

}  // namespace pgpu
