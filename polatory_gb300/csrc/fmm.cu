// Interpolation-based FMM on the GPU (value sources -> value targets).
//
// Tree: points (already in the anisotropy frame) get 3 x Lf-bit Morton keys of their leaf cell in
// the cube of src/fmm/utility.hpp:18-33 (make_box); keys are radix-sorted and run-length encoded
// into the non-empty cells of every level (the uniform-depth tree of the reference's group tree).
// Far field: tensor-product Chebyshev interpolation of order p (p^3 nodes per cell):
//   P2M   M_c[a]  = sum_j w_j S_a(xi_j)                       (leaf cells)
//   M2M   M_P[a] += sum_b M_c[b] S_a(child node b in P)        (separable, 3 passes)
//   M2L   L_t[a] += sum_b K_o[a][b] M_s[b]  for the cells s of t's interaction list, where o is
//         the offset s - t in cell units and K_o[a][b] = phi(r_k (x_a - x_b) - 2 r_k o) depends
//         only on (level, o): one dense p^3 x p^3 matrix per offset, shared by all pairs.
//   L2L   L_c[b] += sum_a L_P[a] S_a(child node b in P)
//   L2P   u(x)  += sum_a L_t[a] S_a(xi)
// Near field (P2P): the 27 neighbour leaves (separation criterion 1, fmm/kernel.hpp:71),
// sources staged in shared memory one tile at a time.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>
#include <vector>

#include "fmm.hpp"
#include "linalg.hpp"
#include "m2l_tc.hpp"
#include "profile.hpp"

namespace pgpu {

namespace {

constexpr int kMaxP = 8;
constexpr int kNOff = 343;  // 7^3 offsets in [-3, 3]^3
constexpr int kTT = 32;     // target cells per M2L tile

template <class T>
struct Cheb {
  int p;
  T tkm[kMaxP][kMaxP];   // T_k(x_m) [m][k]
  T wlo[kMaxP][kMaxP];   // S_a(-0.5 + 0.5 x_b) [a][b]
  T whi[kMaxP][kMaxP];   // S_a(+0.5 + 0.5 x_b) [a][b]
};

// 1-D Chebyshev interpolation basis S_m(x) = 1/p + 2/p sum_{k>=1} T_k(x_m) T_k(x).
double cheb_node(int p, int m) { return std::cos((2.0 * m + 1.0) * M_PI / (2.0 * p)); }

double cheb_s_host(int p, int m, double x) {
  double xm = cheb_node(p, m);
  double s = 1.0 / p;
  double t0 = 1.0, t1 = x, u0 = 1.0, u1 = xm;
  for (int k = 1; k < p; ++k) {
    s += 2.0 / p * t1 * u1;
    double t2 = 2 * x * t1 - t0;
    double u2 = 2 * xm * u1 - u0;
    t0 = t1;
    t1 = t2;
    u0 = u1;
    u1 = u2;
  }
  return s;
}

template <class T>
Cheb<T> make_cheb(int p) {
  Cheb<T> c{};
  c.p = p;
  for (int m = 0; m < p; ++m) {
    double xm = cheb_node(p, m);
    double t0 = 1.0, t1 = xm;
    c.tkm[m][0] = T(1);
    if (p > 1) c.tkm[m][1] = static_cast<T>(xm);
    for (int k = 2; k < p; ++k) {
      double t2 = 2 * xm * t1 - t0;
      c.tkm[m][k] = static_cast<T>(t2);
      t0 = t1;
      t1 = t2;
    }
  }
  for (int a = 0; a < p; ++a)
    for (int b = 0; b < p; ++b) {
      double xb = cheb_node(p, b);
      c.wlo[a][b] = static_cast<T>(cheb_s_host(p, a, -0.5 + 0.5 * xb));
      c.whi[a][b] = static_cast<T>(cheb_s_host(p, a, 0.5 + 0.5 * xb));
    }
  return c;
}

template <int P, class T>
__device__ __forceinline__ void cheb_basis(const Cheb<T>& c, T x, T* s) {
  T t[P];
  t[0] = T(1);
  if (P > 1) t[1] = x;
#pragma unroll
  for (int k = 2; k < P; ++k) t[k] = T(2) * x * t[k - 1] - t[k - 2];
#pragma unroll
  for (int m = 0; m < P; ++m) {
    T v = T(0);
#pragma unroll
    for (int k = 1; k < P; ++k) v += c.tkm[m][k] * t[k];
    s[m] = (T(1) + T(2) * v) / T(P);
  }
}

// The basis and its derivative: dS_m/dx = 2/p sum_{k>=1} T_k(x_m) k U_{k-1}(x), with U the
// Chebyshev polynomials of the second kind (T_k' = k U_{k-1}).
template <int P, class T>
__device__ __forceinline__ void cheb_basis_d(const Cheb<T>& c, T x, T* s, T* ds) {
  T t[P], u[P];
  t[0] = T(1);
  u[0] = T(1);
  if (P > 1) {
    t[1] = x;
    u[1] = T(2) * x;
  }
#pragma unroll
  for (int k = 2; k < P; ++k) {
    t[k] = T(2) * x * t[k - 1] - t[k - 2];
    u[k] = T(2) * x * u[k - 1] - u[k - 2];
  }
#pragma unroll
  for (int m = 0; m < P; ++m) {
    T v = T(0), dv = T(0);
#pragma unroll
    for (int k = 1; k < P; ++k) {
      v += c.tkm[m][k] * t[k];
      dv += c.tkm[m][k] * T(k) * u[k - 1];
    }
    s[m] = (T(1) + T(2) * v) / T(P);
    ds[m] = T(2) * dv / T(P);
  }
}

// ---- Morton keys --------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint64_t spread3(uint64_t x) {
  x &= 0x1fffffULL;
  x = (x | (x << 32)) & 0x1f00000000ffffULL;
  x = (x | (x << 16)) & 0x1f0000ff0000ffULL;
  x = (x | (x << 8)) & 0x100f00f00f00f00fULL;
  x = (x | (x << 4)) & 0x10c30c30c30c30c3ULL;
  x = (x | (x << 2)) & 0x1249249249249249ULL;
  return x;
}

__host__ __device__ __forceinline__ uint64_t compact3(uint64_t x) {
  x &= 0x1249249249249249ULL;
  x = (x ^ (x >> 2)) & 0x10c30c30c30c30c3ULL;
  x = (x ^ (x >> 4)) & 0x100f00f00f00f00fULL;
  x = (x ^ (x >> 8)) & 0x1f0000ff0000ffULL;
  x = (x ^ (x >> 16)) & 0x1f00000000ffffULL;
  x = (x ^ (x >> 32)) & 0x1fffffULL;
  return x;
}

__host__ __device__ __forceinline__ uint64_t morton(uint64_t x, uint64_t y, uint64_t z) {
  return spread3(x) | (spread3(y) << 1) | (spread3(z) << 2);
}

__device__ __forceinline__ void unmorton(uint64_t k, int& x, int& y, int& z) {
  x = static_cast<int>(compact3(k));
  y = static_cast<int>(compact3(k >> 1));
  z = static_cast<int>(compact3(k >> 2));
}

struct Box {
  double min[3];
  double width;
};

__global__ void keys_kernel(const P4<double>* __restrict__ pos, Index n, Box box, int lf,
                            uint64_t* __restrict__ keys, Index* __restrict__ idx) {
  Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double cells = static_cast<double>(1 << lf);
  const double inv = cells / box.width;
  P4<double> p = pos[i];
  int c[3];
  double v[3] = {static_cast<double>(p.x), static_cast<double>(p.y), static_cast<double>(p.z)};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    double f = floor((v[k] - box.min[k]) * inv);
    f = fmin(fmax(f, 0.0), cells - 1.0);
    c[k] = static_cast<int>(f);
  }
  keys[i] = morton(c[0], c[1], c[2]);
  idx[i] = i;
}

// Sorted positions relative to the centre of their leaf cell.
template <class T>
__global__ void gather_rel_pos_kernel(const P4<double>* __restrict__ pos,
                                      const Index* __restrict__ perm,
                                      const uint64_t* __restrict__ keys, int shift, Index n,
                                      Box box, int lf, P4<T>* __restrict__ out) {
  Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const P4<double> p = pos[perm[i]];
  const uint64_t k = keys[i] >> shift;
  const double wk = box.width / static_cast<double>(1 << lf);
  const double cx = box.min[0] + (static_cast<double>(compact3(k)) + 0.5) * wk;
  const double cy = box.min[1] + (static_cast<double>(compact3(k >> 1)) + 0.5) * wk;
  const double cz = box.min[2] + (static_cast<double>(compact3(k >> 2)) + 0.5) * wk;
  out[i] = P4<T>{static_cast<T>(p.x - cx), static_cast<T>(p.y - cy), static_cast<T>(p.z - cz), T(0)};
}

template <class T>
__global__ void gather_w_kernel(const T* __restrict__ w, const Index* __restrict__ perm, Index n,
                                T* __restrict__ out) {
  Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) out[i] = w[perm[i]];
}

// Gradient-source weights (three per source) into the sorted order.
template <class T>
__global__ void gather_w3_kernel(const T* __restrict__ g, const Index* __restrict__ perm, Index n,
                                 T* __restrict__ out) {
  Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Index j = perm[i];
  out[3 * i] = g[3 * j];
  out[3 * i + 1] = g[3 * j + 1];
  out[3 * i + 2] = g[3 * j + 2];
}

__global__ void rle_flags_kernel(const uint64_t* __restrict__ keys, Index n, int shift,
                                 Index* __restrict__ flags) {
  Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  flags[i] = (i == 0 || (keys[i] >> shift) != (keys[i - 1] >> shift)) ? 1 : 0;
}

__global__ void rle_scatter_kernel(const uint64_t* __restrict__ keys, Index n, int shift,
                                   const Index* __restrict__ scan, uint64_t* __restrict__ ukeys,
                                   Index* __restrict__ start, Index* __restrict__ parent) {
  Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Index u = scan[i] - 1;
  if (parent) parent[i] = u;
  if (i == 0 || (keys[i] >> shift) != (keys[i - 1] >> shift)) {
    ukeys[u] = keys[i] >> shift;
    start[u] = i;
  }
}

__device__ __forceinline__ Index find_key(const uint64_t* __restrict__ keys, Index n, uint64_t k) {
  Index lo = 0, hi = n;
  while (lo < hi) {
    Index mid = (lo + hi) >> 1;
    if (keys[mid] < k) lo = mid + 1;
    else hi = mid;
  }
  return (lo < n && keys[lo] == k) ? lo : -1;
}

// M2L interaction table: children of the parent's neighbours that are not adjacent.
__global__ void m2l_table_kernel(const uint64_t* __restrict__ tkeys, Index nt,
                                 const uint64_t* __restrict__ skeys, Index ns, int level,
                                 int* __restrict__ table, Index* __restrict__ count) {
  Index t = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  int cx, cy, cz;
  unmorton(tkeys[t], cx, cy, cz);
  const int px = cx >> 1, py = cy >> 1, pz = cz >> 1;
  const int n = 1 << level;
  int* row = table + t * kNOff;
  Index cnt = 0;
  for (int dx = -1; dx <= 1; ++dx)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dz = -1; dz <= 1; ++dz)
        for (int e = 0; e < 8; ++e) {
          int qx = 2 * (px + dx) + (e & 1), qy = 2 * (py + dy) + ((e >> 1) & 1),
              qz = 2 * (pz + dz) + ((e >> 2) & 1);
          if (qx < 0 || qy < 0 || qz < 0 || qx >= n || qy >= n || qz >= n) continue;
          int ox = qx - cx, oy = qy - cy, oz = qz - cz;
          if (abs(ox) <= 1 && abs(oy) <= 1 && abs(oz) <= 1) continue;
          Index s = find_key(skeys, ns, morton(qx, qy, qz));
          if (s < 0) continue;
          row[(ox + 3) * 49 + (oy + 3) * 7 + (oz + 3)] = static_cast<int>(s);
          ++cnt;
        }
  count[t] = cnt;
}

__global__ void p2p_table_kernel(const uint64_t* __restrict__ tkeys, Index nt,
                                 const uint64_t* __restrict__ skeys, Index ns, int level,
                                 int* __restrict__ table) {
  Index t = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  int cx, cy, cz;
  unmorton(tkeys[t], cx, cy, cz);
  const int n = 1 << level;
  int j = 0;
  for (int dx = -1; dx <= 1; ++dx)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dz = -1; dz <= 1; ++dz) {
        int qx = cx + dx, qy = cy + dy, qz = cz + dz;
        int s = -1;
        if (qx >= 0 && qy >= 0 && qz >= 0 && qx < n && qy < n && qz < n)
          s = static_cast<int>(find_key(skeys, ns, morton(qx, qy, qz)));
        table[t * 27 + j++] = s;
      }
}

template <int KIND, class T>
__global__ void m2l_matrix_kernel(KParams<T> kp, int p, double r, const double* __restrict__ nodes,
                                  T* __restrict__ K) {
  const Index p3 = static_cast<Index>(p) * p * p;
  const Index total = kNOff * p3 * p3;
  for (Index e = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x; e < total;
       e += static_cast<Index>(gridDim.x) * blockDim.x) {
    const Index o = e / (p3 * p3);
    const Index ab = e % (p3 * p3);
    const int a = static_cast<int>(ab / p3), b = static_cast<int>(ab % p3);
    const int ox = static_cast<int>(o / 49) - 3, oy = static_cast<int>((o / 7) % 7) - 3,
              oz = static_cast<int>(o % 7) - 3;
    const int ax = a / (p * p), ay = (a / p) % p, az = a % p;
    const int bx = b / (p * p), by = (b / p) % p, bz = b % p;
    double dx = r * (nodes[ax] - nodes[bx]) - 2.0 * r * ox;
    double dy = r * (nodes[ay] - nodes[by]) - 2.0 * r * oy;
    double dz = r * (nodes[az] - nodes[bz]) - 2.0 * r * oz;
    KParams<double> kd{static_cast<double>(kp.p0), static_cast<double>(kp.p1)};
    K[e] = static_cast<T>(rbf_value<KIND>(dx * dx + dy * dy + dz * dz, kd));
  }
}

// ---- passes ------------------------------------------------------------------------------

template <int P, class T>
__global__ void __launch_bounds__(256)
    p2m_kernel(Cheb<T> ch, const P4<T>* __restrict__ spos, const T* __restrict__ sw,
               const Index* __restrict__ leaf_start, const uint64_t* __restrict__ leaf_keys,
               Box box, int lf, T* __restrict__ M) {
  constexpr int P3 = P * P * P;
  const Index leaf = blockIdx.x;
  __shared__ T s_b[32][3][P];
  __shared__ T s_w[32];
  (void)leaf_keys;
  const double wk = box.width / static_cast<double>(1 << lf);
  const T ctr[3] = {T(0), T(0), T(0)};  // tree positions are relative to the leaf centre
  const T inv_r = static_cast<T>(2.0 / wk);
  const Index beg = leaf_start[leaf], end = leaf_start[leaf + 1];
  T acc[(P3 + 255) / 256];
#pragma unroll
  for (int q = 0; q < (P3 + 255) / 256; ++q) acc[q] = T(0);
  for (Index base = beg; base < end; base += 32) {
    const int cnt = static_cast<int>(min(static_cast<Index>(32), end - base));
    __syncthreads();
    if (threadIdx.x < 3 * cnt) {
      const int j = threadIdx.x / 3, d = threadIdx.x % 3;
      P4<T> pt = spos[base + j];
      T x = (d == 0 ? pt.x : (d == 1 ? pt.y : pt.z));
      cheb_basis<P>(ch, (x - ctr[d]) * inv_r, s_b[j][d]);
    }
    if (threadIdx.x < cnt) s_w[threadIdx.x] = sw[base + threadIdx.x];
    __syncthreads();
#pragma unroll
    for (int q = 0; q < (P3 + 255) / 256; ++q) {
      const int a = threadIdx.x + 256 * q;
      if (a < P3) {
        const int ax = a / (P * P), ay = (a / P) % P, az = a % P;
        T s = T(0);
        for (int j = 0; j < cnt; ++j) s += s_w[j] * s_b[j][0][ax] * s_b[j][1][ay] * s_b[j][2][az];
        acc[q] += s;
      }
    }
  }
#pragma unroll
  for (int q = 0; q < (P3 + 255) / 256; ++q) {
    const int a = threadIdx.x + 256 * q;
    if (a < P3) M[leaf * P3 + a] = acc[q];
  }
}

// P2M of gradient sources (dipoles): the potential of weight G at y is G . grad_y phi(x - y),
// which the interpolation turns into sum_n (G . grad S_n(y)) phi(x - y_n): each source adds
// G . grad S_n(y) to node n (frame coordinates; the chain rule's 2 / w factor included).
template <int P, class T>
__global__ void __launch_bounds__(256)
    p2m_dipole_kernel(Cheb<T> ch, const P4<T>* __restrict__ spos, const T* __restrict__ sw3,
                      const Index* __restrict__ leaf_start, Box box, int lf, T* __restrict__ M) {
  constexpr int P3 = P * P * P;
  const Index leaf = blockIdx.x;
  __shared__ T s_b[32][3][P];
  __shared__ T s_d[32][3][P];
  __shared__ T s_g[32][3];
  const double wk = box.width / static_cast<double>(1 << lf);
  const T inv_r = static_cast<T>(2.0 / wk);
  const Index beg = leaf_start[leaf], end = leaf_start[leaf + 1];
  T acc[(P3 + 255) / 256];
#pragma unroll
  for (int q = 0; q < (P3 + 255) / 256; ++q) acc[q] = T(0);
  for (Index base = beg; base < end; base += 32) {
    const int cnt = static_cast<int>(min(static_cast<Index>(32), end - base));
    __syncthreads();
    if (threadIdx.x < 3 * cnt) {
      const int j = threadIdx.x / 3, d = threadIdx.x % 3;
      const P4<T> pt = spos[base + j];
      const T x = (d == 0 ? pt.x : (d == 1 ? pt.y : pt.z));
      cheb_basis_d<P>(ch, x * inv_r, s_b[j][d], s_d[j][d]);
      s_g[j][d] = sw3[3 * (base + j) + d] * inv_r;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < (P3 + 255) / 256; ++q) {
      const int a = threadIdx.x + 256 * q;
      if (a < P3) {
        const int ax = a / (P * P), ay = (a / P) % P, az = a % P;
        T s = T(0);
        for (int j = 0; j < cnt; ++j)
          s += s_g[j][0] * s_d[j][0][ax] * s_b[j][1][ay] * s_b[j][2][az] +
               s_g[j][1] * s_b[j][0][ax] * s_d[j][1][ay] * s_b[j][2][az] +
               s_g[j][2] * s_b[j][0][ax] * s_b[j][1][ay] * s_d[j][2][az];
        acc[q] += s;
      }
    }
  }
#pragma unroll
  for (int q = 0; q < (P3 + 255) / 256; ++q) {
    const int a = threadIdx.x + 256 * q;
    if (a < P3) M[leaf * P3 + a] = acc[q];
  }
}

// Separable transfer of one p^3 tensor: out[a] = sum_b Wx[ax][bx] Wy[ay][by] Wz[az][bz] in[b]
// (transpose = false) or the transposed map (transpose = true). Uses two scratch tensors.
template <int P, class T>
__device__ __forceinline__ T sep_transfer(const T (*wx)[kMaxP], const T (*wy)[kMaxP],
                                          const T (*wz)[kMaxP], bool transpose, T* in, T* t1,
                                          T* t2) {
  constexpr int P3 = P * P * P;
  const int a = threadIdx.x;
  const int ax = a / (P * P), ay = (a / P) % P, az = a % P;
  // pass z
  if (a < P3) {
    T s = T(0);
#pragma unroll
    for (int b = 0; b < P; ++b) s += (transpose ? wz[b][az] : wz[az][b]) * in[(ax * P + ay) * P + b];
    t1[a] = s;
  }
  __syncthreads();
  if (a < P3) {
    T s = T(0);
#pragma unroll
    for (int b = 0; b < P; ++b) s += (transpose ? wy[b][ay] : wy[ay][b]) * t1[(ax * P + b) * P + az];
    t2[a] = s;
  }
  __syncthreads();
  T s = T(0);
  if (a < P3) {
#pragma unroll
    for (int b = 0; b < P; ++b) s += (transpose ? wx[b][ax] : wx[ax][b]) * t2[(b * P + ay) * P + az];
  }
  __syncthreads();
  return s;
}

template <int P, class T>
__global__ void m2m_kernel(Cheb<T> ch, const Index* __restrict__ child_start,
                           const uint64_t* __restrict__ child_keys, const T* __restrict__ Mc,
                           T* __restrict__ Mp) {
  constexpr int P3 = P * P * P;
  __shared__ T s_in[P3], s_t1[P3], s_t2[P3];
  const Index parent = blockIdx.x;
  const Index c0 = child_start[parent], c1 = child_start[parent + 1];
  T acc = T(0);
  for (Index c = c0; c < c1; ++c) {
    const uint64_t k = child_keys[c];
    for (int e = threadIdx.x; e < P3; e += blockDim.x) s_in[e] = Mc[c * P3 + e];
    __syncthreads();
    const T(*wx)[kMaxP] = (k & 1) ? ch.whi : ch.wlo;
    const T(*wy)[kMaxP] = (k & 2) ? ch.whi : ch.wlo;
    const T(*wz)[kMaxP] = (k & 4) ? ch.whi : ch.wlo;
    acc += sep_transfer<P>(wx, wy, wz, false, s_in, s_t1, s_t2);
  }
  if (threadIdx.x < P3) Mp[parent * P3 + threadIdx.x] = acc;
}

template <int P, class T>
__global__ void l2l_kernel(Cheb<T> ch, const Index* __restrict__ parent_of,
                           const uint64_t* __restrict__ child_keys, const T* __restrict__ Lp,
                           T* __restrict__ Lc) {
  constexpr int P3 = P * P * P;
  __shared__ T s_in[P3], s_t1[P3], s_t2[P3];
  const Index c = blockIdx.x;
  const Index parent = parent_of[c];
  const uint64_t k = child_keys[c];
  for (int e = threadIdx.x; e < P3; e += blockDim.x) s_in[e] = Lp[parent * P3 + e];
  __syncthreads();
  const T(*wx)[kMaxP] = (k & 1) ? ch.whi : ch.wlo;
  const T(*wy)[kMaxP] = (k & 2) ? ch.whi : ch.wlo;
  const T(*wz)[kMaxP] = (k & 4) ? ch.whi : ch.wlo;
  T v = sep_transfer<P>(wx, wy, wz, true, s_in, s_t1, s_t2);
  if (threadIdx.x < P3) Lc[c * P3 + threadIdx.x] += v;
}

// M2L over a tile of kTT target cells: every non-adjacent offset o with at least one source in
// the tile is applied as a dense (p^3 x p^3) x (p^3 x kTT) product with K_o streamed in 8-row
// chunks through shared memory; the local expansions stay in registers across all offsets.
template <int D, class T>
__global__ void __launch_bounds__(256)
    m2l_kernel(const T* __restrict__ K, const int* __restrict__ table, Index nt,
               const T* __restrict__ Ms, T* __restrict__ L, int groups, T* __restrict__ part) {
  constexpr int P3 = D;  // operator dimension: p^3 (dense) or the compressed rank
  constexpr int NC = P3 / 8;  // row chunks
  // blockIdx.y selects a contiguous group of offsets; with several groups each block writes a
  // partial expansion that m2l_reduce_kernel sums in a fixed order.
  const int o_beg = static_cast<int>((static_cast<long>(blockIdx.y) * kNOff) / groups);
  const int o_end = static_cast<int>((static_cast<long>(blockIdx.y + 1) * kNOff) / groups);
  extern __shared__ unsigned char smem_raw[];
  T* s_m = reinterpret_cast<T*>(smem_raw);  // [P3][kTT + 1]
  T* s_k = s_m + P3 * (kTT + 1);            // [8][P3]
  __shared__ int s_src[kTT];
  const Index t0 = static_cast<Index>(blockIdx.x) * kTT;
  const int r = threadIdx.x >> 5;  // row within chunk
  const int t = threadIdx.x & 31;  // target within tile
  T acc[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) acc[c] = T(0);

  for (int o = o_beg; o < o_end; ++o) {
    const int ox = o / 49 - 3, oy = (o / 7) % 7 - 3, oz = o % 7 - 3;
    if (abs(ox) <= 1 && abs(oy) <= 1 && abs(oz) <= 1) continue;
    __syncthreads();
    if (threadIdx.x < kTT) {
      const Index tt = t0 + threadIdx.x;
      s_src[threadIdx.x] = tt < nt ? table[tt * kNOff + o] : -1;
    }
    __syncthreads();
    const bool any = __syncthreads_or(threadIdx.x < kTT && s_src[threadIdx.x] >= 0);
    if (!any) continue;
    for (int e = threadIdx.x; e < P3 * kTT; e += blockDim.x) {
      const int tt = e / P3, b = e % P3;
      const int s = s_src[tt];
      s_m[b * (kTT + 1) + tt] = s >= 0 ? Ms[static_cast<Index>(s) * P3 + b] : T(0);
    }
    const T* ko = K + static_cast<Index>(o) * P3 * P3;
#pragma unroll 1
    for (int c = 0; c < NC; ++c) {
      __syncthreads();
      for (int e = threadIdx.x; e < 8 * P3; e += blockDim.x) s_k[e] = ko[static_cast<Index>(c) * 8 * P3 + e];
      __syncthreads();
      T s = T(0);
      const T* krow = s_k + r * P3;
#pragma unroll 8
      for (int b = 0; b < P3; ++b) s += krow[b] * s_m[b * (kTT + 1) + t];
      // acc[c] with a runtime c: select through a switch-free unrolled update
#pragma unroll
      for (int cc = 0; cc < NC; ++cc)
        if (cc == c) acc[cc] += s;
    }
  }
  const Index tt = t0 + t;
  if (tt < nt) {
    if (groups == 1) {
#pragma unroll
      for (int c = 0; c < NC; ++c) L[tt * P3 + c * 8 + r] += acc[c];
    } else {
      T* pg = part + (static_cast<Index>(blockIdx.y) * nt + tt) * P3;
#pragma unroll
      for (int c = 0; c < NC; ++c) pg[c * 8 + r] = acc[c];
    }
  }
}

// Register-tiled M2L (D = p^3 <= 216). A block owns 64 target cells; thread (ag, tg) owns the
// RA consecutive rows ag*RA.. of the local expansions of the 4 targets tg*4.., accumulated in
// registers across every offset. For each offset, K_o is streamed through shared memory in
// column chunks of BK. The kernels are even (phi(d) = phi(-d)), so column b of K_o is row b of
// K_{-o} and is read contiguously from the operator of the opposite offset (index 342 - o).
template <int D, class T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 2 : 1)
    m2l_tiled_kernel(const T* __restrict__ K, const int* __restrict__ table, Index nt,
                     const T* __restrict__ Ms, T* __restrict__ L, int groups, T* __restrict__ part) {
  constexpr int RA = (D + 15) / 16;
  constexpr int DP = RA * 16;
  constexpr int BK = sizeof(T) == 8 ? 8 : ((D % 24 == 0) ? 24 : 16);
  constexpr int TT = 64;
  __shared__ __align__(16) T s_kt[BK][DP];
  __shared__ __align__(16) T s_m[BK][TT];
  __shared__ int s_src[TT];
  const int o_beg = static_cast<int>((static_cast<long>(blockIdx.y) * kNOff) / groups);
  const int o_end = static_cast<int>((static_cast<long>(blockIdx.y + 1) * kNOff) / groups);
  const Index t0 = static_cast<Index>(blockIdx.x) * TT;
  const int ag = threadIdx.x >> 4;  // 0..15
  const int tg = threadIdx.x & 15;  // 0..15
  T acc[RA][4];
#pragma unroll
  for (int i = 0; i < RA; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
  // Padding rows of the operator chunk stay zero.
  if constexpr (DP > D) {
    for (int e = threadIdx.x; e < BK * (DP - D); e += blockDim.x)
      s_kt[e / (DP - D)][D + e % (DP - D)] = T(0);
  }

  for (int o = o_beg; o < o_end; ++o) {
    const int ox = o / 49 - 3, oy = (o / 7) % 7 - 3, oz = o % 7 - 3;
    if (abs(ox) <= 1 && abs(oy) <= 1 && abs(oz) <= 1) continue;
    __syncthreads();
    if (threadIdx.x < TT) {
      const Index tt = t0 + threadIdx.x;
      s_src[threadIdx.x] = tt < nt ? table[tt * kNOff + o] : -1;
    }
    const bool any = __syncthreads_or(threadIdx.x < TT && t0 + threadIdx.x < nt &&
                                      table[(t0 + threadIdx.x) * kNOff + o] >= 0);
    if (!any) continue;
    const T* kt = K + static_cast<Index>(kNOff - 1 - o) * D * D;  // row b of K_{-o} = column b of K_o
    for (int b0 = 0; b0 < D; b0 += BK) {
      const int bk = min(BK, D - b0);
      __syncthreads();
      for (int e = threadIdx.x; e < bk * D; e += blockDim.x) {
        const int bb = e / D, a = e % D;
        s_kt[bb][a] = kt[static_cast<Index>(b0 + bb) * D + a];
      }
      for (int e = threadIdx.x; e < bk * TT; e += blockDim.x) {
        const int t = e / bk, bb = e % bk;
        const int s = s_src[t];
        s_m[bb][t] = s >= 0 ? Ms[static_cast<Index>(s) * D + b0 + bb] : T(0);
      }
      __syncthreads();
      for (int bb = 0; bb < bk; ++bb) {
        T kv[RA];
#pragma unroll
        for (int i = 0; i < RA; ++i) kv[i] = s_kt[bb][ag * RA + i];
        T mv[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) mv[j] = s_m[bb][tg * 4 + j];
#pragma unroll
        for (int i = 0; i < RA; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[i][j] += kv[i] * mv[j];
      }
    }
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const Index tt = t0 + tg * 4 + j;
    if (tt >= nt) continue;
    T* dst = groups == 1 ? L + tt * D : part + (static_cast<Index>(blockIdx.y) * nt + tt) * D;
#pragma unroll
    for (int i = 0; i < RA; ++i) {
      const int a = ag * RA + i;
      if (a < D) {
        if (groups == 1) dst[a] += acc[i][j];
        else dst[a] = acc[i][j];
      }
    }
  }
}

// x[i] *= s (a level's multipole expansions, for operators stored at radius 1).
template <class T>
__global__ void scale_expansions_kernel(T* __restrict__ x, Index n, T s) {
  const Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) x[i] *= s;
}

template <class T>
__global__ void m2l_reduce_kernel(const T* __restrict__ part, int groups, Index n,
                                  T* __restrict__ L) {
  Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T s = T(0);
  for (int g = 0; g < groups; ++g) s += part[static_cast<Index>(g) * n + i];
  L[i] += s;
}

// Targets per block in the near field and L2P: leaves crowded with targets (evaluation points
// falling into few source leaves) are split into chunks of this size.
constexpr int kP2PChunk = 256;

template <int P, class T>
__global__ void __launch_bounds__(128)
    l2p_kernel(Cheb<T> ch, const P4<T>* __restrict__ tpos, const Index* __restrict__ perm,
               const Index* __restrict__ leaf_start, const int* __restrict__ chunk_leaf,
               Box box, int lf, const T* __restrict__ L, double* __restrict__ out) {
  constexpr int P3 = P * P * P;
  __shared__ T s_l[P3];
  // One block per chunk of at most kP2PChunk targets of one leaf (the P2P chunk table).
  const Index leaf = chunk_leaf[2 * blockIdx.x];
  for (int e = threadIdx.x; e < P3; e += blockDim.x) s_l[e] = L[leaf * P3 + e];
  __syncthreads();
  const double wk = box.width / static_cast<double>(1 << lf);
  const T ctr[3] = {T(0), T(0), T(0)};  // tree positions are relative to the leaf centre
  const T inv_r = static_cast<T>(2.0 / wk);
  const Index beg = leaf_start[leaf] + static_cast<Index>(chunk_leaf[2 * blockIdx.x + 1]) * kP2PChunk;
  const Index end = min(leaf_start[leaf + 1], beg + kP2PChunk);
  for (Index i = beg + threadIdx.x; i < end; i += blockDim.x) {
    P4<T> pt = tpos[i];
    T sx[P], sy[P], sz[P];
    cheb_basis<P>(ch, (pt.x - ctr[0]) * inv_r, sx);
    cheb_basis<P>(ch, (pt.y - ctr[1]) * inv_r, sy);
    cheb_basis<P>(ch, (pt.z - ctr[2]) * inv_r, sz);
    T v = T(0);
#pragma unroll
    for (int ax = 0; ax < P; ++ax) {
      T vy = T(0);
#pragma unroll
      for (int ay = 0; ay < P; ++ay) {
        T vz = T(0);
#pragma unroll
        for (int az = 0; az < P; ++az) vz += s_l[(ax * P + ay) * P + az] * sz[az];
        vy += vz * sy[ay];
      }
      v += vy * sx[ax];
    }
    out[perm[i]] += static_cast<double>(v);
  }
}

// L2P for gradient targets: out3[3 perm[i] + k] += d/dx_k of the local expansion at the target
// (the anisotropy frame's gradient; the caller maps it back with A^T).
template <int P, class T>
__global__ void __launch_bounds__(128)
    l2p_grad_kernel(Cheb<T> ch, const P4<T>* __restrict__ tpos, const Index* __restrict__ perm,
                    const Index* __restrict__ leaf_start, const int* __restrict__ chunk_leaf,
                    Box box, int lf, const T* __restrict__ L, double* __restrict__ out3) {
  constexpr int P3 = P * P * P;
  __shared__ T s_l[P3];
  const Index leaf = chunk_leaf[2 * blockIdx.x];
  for (int e = threadIdx.x; e < P3; e += blockDim.x) s_l[e] = L[leaf * P3 + e];
  __syncthreads();
  const double wk = box.width / static_cast<double>(1 << lf);
  const T inv_r = static_cast<T>(2.0 / wk);
  const Index beg = leaf_start[leaf] + static_cast<Index>(chunk_leaf[2 * blockIdx.x + 1]) * kP2PChunk;
  const Index end = min(leaf_start[leaf + 1], beg + kP2PChunk);
  for (Index i = beg + threadIdx.x; i < end; i += blockDim.x) {
    const P4<T> pt = tpos[i];
    T sx[P], sy[P], sz[P], dx[P], dy[P], dz[P];
    cheb_basis_d<P>(ch, pt.x * inv_r, sx, dx);
    cheb_basis_d<P>(ch, pt.y * inv_r, sy, dy);
    cheb_basis_d<P>(ch, pt.z * inv_r, sz, dz);
    T gx = T(0), gy = T(0), gz = T(0);
#pragma unroll
    for (int ax = 0; ax < P; ++ax) {
      T vy = T(0), vyz = T(0), vdy = T(0);
#pragma unroll
      for (int ay = 0; ay < P; ++ay) {
        T vz = T(0), vdz = T(0);
#pragma unroll
        for (int az = 0; az < P; ++az) {
          const T l = s_l[(ax * P + ay) * P + az];
          vz += l * sz[az];
          vdz += l * dz[az];
        }
        vy += vz * sy[ay];
        vdy += vz * dy[ay];
        vyz += vdz * sy[ay];
      }
      gx += vy * dx[ax];
      gy += vdy * sx[ax];
      gz += vyz * sx[ax];
    }
    const Index o = 3 * perm[i];
    out3[o] += static_cast<double>(gx * inv_r);
    out3[o + 1] += static_cast<double>(gy * inv_r);
    out3[o + 2] += static_cast<double>(gz * inv_r);
  }
}

// Near field for gradient targets: out3[3 tperm[i] + k] += sum_j w_j d/dx_k phi(x_i - y_j) over
// the 27 neighbour leaves (anisotropy frame), one target per thread, source tiles in shared
// memory.
template <int KIND, class T>
__global__ void __launch_bounds__(128)
    p2p_grad_kernel(KParams<T> kp, const P4<T>* __restrict__ tpos, const Index* __restrict__ tperm,
                    const Index* __restrict__ tleaf_start, const int* __restrict__ chunk_leaf,
                    const int* __restrict__ table, const P4<T>* __restrict__ spos,
                    const T* __restrict__ sw, const Index* __restrict__ sleaf_start, T wleaf,
                    double* __restrict__ out3) {
  __shared__ P4<T> s_p[128];
  __shared__ int s_nb[27];
  const int leaf = chunk_leaf[2 * blockIdx.x];
  if (threadIdx.x < 27) s_nb[threadIdx.x] = table[static_cast<Index>(leaf) * 27 + threadIdx.x];
  __syncthreads();
  const Index tb = tleaf_start[leaf] + static_cast<Index>(chunk_leaf[2 * blockIdx.x + 1]) * kP2PChunk;
  const Index te = min(tleaf_start[leaf + 1], tb + kP2PChunk);
  for (Index i0 = tb; i0 < te; i0 += blockDim.x) {
    const Index i = i0 + threadIdx.x;
    const bool active = i < te;
    const P4<T> t = active ? tpos[i] : P4<T>{T(0), T(0), T(0), T(0)};
    double tot[3] = {0.0, 0.0, 0.0};
    for (int nb = 0; nb < 27; ++nb) {
      const int s = s_nb[nb];
      if (s < 0) continue;
      const T tx = t.x - static_cast<T>(nb / 9 - 1) * wleaf;
      const T ty = t.y - static_cast<T>((nb / 3) % 3 - 1) * wleaf;
      const T tz = t.z - static_cast<T>(nb % 3 - 1) * wleaf;
      const Index sb = sleaf_start[s], se = sleaf_start[s + 1];
      for (Index base = sb; base < se; base += 128) {
        const int cnt = static_cast<int>(min(static_cast<Index>(128), se - base));
        __syncthreads();
        if (threadIdx.x < cnt) {
          P4<T> p = spos[base + threadIdx.x];
          p.w = sw[base + threadIdx.x];
          s_p[threadIdx.x] = p;
        }
        __syncthreads();
        T ax = T(0), ay = T(0), az = T(0);
        for (int j = 0; j < cnt; ++j) {
          const P4<T> q = s_p[j];
          acc_grad_from_value<KIND>(tx - q.x, ty - q.y, tz - q.z, q.w, kp, ax, ay, az);
        }
        tot[0] += ax;
        tot[1] += ay;
        tot[2] += az;
      }
    }
    if (active) {
      const Index o = 3 * tperm[i];
      out3[o] += tot[0];
      out3[o + 1] += tot[1];
      out3[o + 2] += tot[2];
    }
  }
}

// Near field of gradient sources (weights G, three per source, anisotropy frame): value targets
// take G . grad_y phi, gradient targets -H G (kernels.cuh: acc_value_from_grad,
// acc_grad_from_grad); out has one or three entries per target.
template <int KIND, class T, bool GRAD_TARGETS>
__global__ void __launch_bounds__(128)
    p2p_dipole_kernel(KParams<T> kp, const P4<T>* __restrict__ tpos, const Index* __restrict__ tperm,
                      const Index* __restrict__ tleaf_start, const int* __restrict__ chunk_leaf,
                      const int* __restrict__ table, const P4<T>* __restrict__ spos,
                      const T* __restrict__ sw3, const Index* __restrict__ sleaf_start, T wleaf,
                      double* __restrict__ out) {
  __shared__ P4<T> s_p[128];
  __shared__ T s_g[128][3];
  __shared__ int s_nb[27];
  const int leaf = chunk_leaf[2 * blockIdx.x];
  if (threadIdx.x < 27) s_nb[threadIdx.x] = table[static_cast<Index>(leaf) * 27 + threadIdx.x];
  __syncthreads();
  const Index tb = tleaf_start[leaf] + static_cast<Index>(chunk_leaf[2 * blockIdx.x + 1]) * kP2PChunk;
  const Index te = min(tleaf_start[leaf + 1], tb + kP2PChunk);
  for (Index i0 = tb; i0 < te; i0 += blockDim.x) {
    const Index i = i0 + threadIdx.x;
    const bool active = i < te;
    const P4<T> t = active ? tpos[i] : P4<T>{T(0), T(0), T(0), T(0)};
    double tot[3] = {0.0, 0.0, 0.0};
    for (int nb = 0; nb < 27; ++nb) {
      const int s = s_nb[nb];
      if (s < 0) continue;
      const T tx = t.x - static_cast<T>(nb / 9 - 1) * wleaf;
      const T ty = t.y - static_cast<T>((nb / 3) % 3 - 1) * wleaf;
      const T tz = t.z - static_cast<T>(nb % 3 - 1) * wleaf;
      const Index sb = sleaf_start[s], se = sleaf_start[s + 1];
      for (Index base = sb; base < se; base += 128) {
        const int cnt = static_cast<int>(min(static_cast<Index>(128), se - base));
        __syncthreads();
        if (threadIdx.x < cnt) {
          s_p[threadIdx.x] = spos[base + threadIdx.x];
          for (int k = 0; k < 3; ++k) s_g[threadIdx.x][k] = sw3[3 * (base + threadIdx.x) + k];
        }
        __syncthreads();
        T a0 = T(0), a1 = T(0), a2 = T(0);
        for (int j = 0; j < cnt; ++j) {
          const P4<T> q = s_p[j];
          if constexpr (GRAD_TARGETS)
            acc_grad_from_grad<KIND>(tx - q.x, ty - q.y, tz - q.z, s_g[j][0], s_g[j][1], s_g[j][2],
                                     kp, a0, a1, a2);
          else
            acc_value_from_grad<KIND>(tx - q.x, ty - q.y, tz - q.z, s_g[j][0], s_g[j][1], s_g[j][2],
                                      kp, a0);
        }
        tot[0] += a0;
        tot[1] += a1;
        tot[2] += a2;
      }
    }
    if (active) {
      if constexpr (GRAD_TARGETS) {
        const Index o = 3 * tperm[i];
        out[o] += tot[0];
        out[o + 1] += tot[1];
        out[o + 2] += tot[2];
      } else {
        out[tperm[i]] += tot[0];
      }
    }
  }
}

// Near field: one block per chunk of a target leaf, each thread one or two targets, source
// tiles in shared memory.

// Chunks of kP2PChunk targets per leaf: count, then (after an exclusive scan) the chunk table
// (leaf, chunk index within the leaf).
__global__ void chunk_count_kernel(const Index* __restrict__ start, Index nleaf,
                                   int* __restrict__ cnt) {
  const Index l = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (l >= nleaf) return;
  const Index n = start[l + 1] - start[l];
  cnt[l] = static_cast<int>((n + kP2PChunk - 1) / kP2PChunk);
}

__global__ void chunk_fill_kernel(const int* __restrict__ cnt, const int* __restrict__ off,
                                  Index nleaf, int* __restrict__ chunk_leaf) {
  const Index l = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (l >= nleaf) return;
  for (int c = 0; c < cnt[l]; ++c) {
    chunk_leaf[2 * (off[l] + c)] = static_cast<int>(l);
    chunk_leaf[2 * (off[l] + c) + 1] = c;
  }
}
template <int KIND, class T>
__global__ void __launch_bounds__(128, 12)
    p2p_kernel(KParams<T> kp, const P4<T>* __restrict__ tpos, const Index* __restrict__ tperm,
               const Index* __restrict__ tleaf_start, const int* __restrict__ chunk_leaf,
               const int* __restrict__ table, const P4<T>* __restrict__ spos,
               const T* __restrict__ sw, const Index* __restrict__ sleaf_start, T wleaf,
               double* __restrict__ out) {
  // Positions are relative to their leaf centres; the neighbour slot nb = 9 (dx+1) + 3 (dy+1) +
  // (dz+1) puts the source leaf centre at the target's + (dx, dy, dz) * wleaf, so
  // d = (t - (dx, dy, dz) wleaf) - s involves only leaf-sized numbers.
  // One block per chunk of at most kP2PChunk targets of one leaf (chunk_leaf: per chunk the
  // leaf and the chunk's index within it), so leaves crowded with targets spread over blocks.
  __shared__ P4<T> s_p[128];
  __shared__ int s_nb[27];
  const int leaf = chunk_leaf[2 * blockIdx.x];
  if (threadIdx.x < 27) s_nb[threadIdx.x] = table[static_cast<Index>(leaf) * 27 + threadIdx.x];
  __syncthreads();
  const Index tb = tleaf_start[leaf] + static_cast<Index>(chunk_leaf[2 * blockIdx.x + 1]) * kP2PChunk;
  const Index te = min(tleaf_start[leaf + 1], tb + kP2PChunk);
  // NT targets per thread (1 or 2, uniform over the block), consecutive: thread t takes targets
  // i0 + NT t .. + NT - 1, so that the threads without targets fill whole warps, which skip the
  // sums. Each source read from shared memory serves NT targets. Weights are staged pre-scaled
  // by the kernel's constant factor where the kernel has one (pair_term).
  const T wscale = pair_weight_scale<KIND>(kp);
  const T c2 = pair_r2_offset<KIND>(kp);
  auto pass = [&]<int NT>(Index i0) {
    P4<T> t[NT];
    bool active[NT];
    bool any = false;
#pragma unroll
    for (int q = 0; q < NT; ++q) {
      const Index i = i0 + NT * threadIdx.x + q;
      active[q] = i < te;
      any |= active[q];
      t[q] = active[q] ? tpos[i] : P4<T>{T(0), T(0), T(0), T(0)};
    }
    const bool warp_busy = __any_sync(0xffffffffu, any);
    double tot[NT];
#pragma unroll
    for (int q = 0; q < NT; ++q) tot[q] = 0;
    for (int nb = 0; nb < 27; ++nb) {
      const int s = s_nb[nb];
      if (s < 0) continue;
      const T ox = static_cast<T>(nb / 9 - 1) * wleaf;
      const T oy = static_cast<T>((nb / 3) % 3 - 1) * wleaf;
      const T oz = static_cast<T>(nb % 3 - 1) * wleaf;
      T tx[NT], ty[NT], tz[NT];
#pragma unroll
      for (int q = 0; q < NT; ++q) {
        tx[q] = t[q].x - ox;
        ty[q] = t[q].y - oy;
        tz[q] = t[q].z - oz;
      }
      const Index sb = sleaf_start[s], se = sleaf_start[s + 1];
      for (Index base = sb; base < se; base += 128) {
        const int cnt = static_cast<int>(min(static_cast<Index>(128), se - base));
        __syncthreads();
        if (threadIdx.x < cnt) {
          P4<T> p = spos[base + threadIdx.x];
          p.w = sw[base + threadIdx.x] * wscale;
          s_p[threadIdx.x] = p;
        }
        __syncthreads();
        if (!warp_busy) continue;
        T acc[NT];
#pragma unroll
        for (int q = 0; q < NT; ++q) acc[q] = T(0);
#pragma unroll 4
        for (int j = 0; j < cnt; ++j) {
          const P4<T> s4 = s_p[j];
#pragma unroll
          for (int q = 0; q < NT; ++q)
            acc[q] = pair_term<KIND>(tx[q] - s4.x, ty[q] - s4.y, tz[q] - s4.z, s4.w, c2, kp, acc[q]);
        }
#pragma unroll
        for (int q = 0; q < NT; ++q) tot[q] += static_cast<double>(acc[q]);
      }
    }
#pragma unroll
    for (int q = 0; q < NT; ++q)
      if (active[q]) out[tperm[i0 + NT * threadIdx.x + q]] += tot[q];
  };
  for (Index i0 = tb; i0 < te;) {
    if (te - i0 > static_cast<Index>(blockDim.x)) {
      pass.template operator()<2>(i0);
      i0 += 2 * blockDim.x;
    } else {
      pass.template operator()<1>(i0);
      i0 += blockDim.x;
    }
  }
}

// Near field of the odd polyharmonic kernels (-p0 rho, p0 rho^3 with rho^2 = r^2 + p1^2) in
// float-float arithmetic: positions, weights and sums carried as unevaluated pairs of floats
// (about 44 significant bits), on the FP32 pipes. Differences use TwoSum, squares and
// products FMA-based TwoProd, the square root one Newton step from rsqrtf. Each 128-source
// tile is summed in float-float and added to an FP64 total.
template <int KIND>
__global__ void __launch_bounds__(128)
    p2p_ff_kernel(KParams<double> kp, const P4<double>* __restrict__ tpos,
                  const Index* __restrict__ tperm, const Index* __restrict__ tleaf_start,
                  const int* __restrict__ table, const P4<double>* __restrict__ spos,
                  const double* __restrict__ sw, const Index* __restrict__ sleaf_start,
                  double wleaf, double* __restrict__ out) {
  // Sources as (x hi, x lo, y hi, y lo) and (z hi, z lo, w hi, w lo): two 16-byte loads a pair.
  __shared__ float4 s_a[128], s_b[128];
  __shared__ int s_nb[27];
  const Index leaf = blockIdx.x;
  if (threadIdx.x < 27) s_nb[threadIdx.x] = table[leaf * 27 + threadIdx.x];
  __syncthreads();
  float c_hi, c_lo;  // p1^2
  ff_split(kp.p1 * kp.p1, c_hi, c_lo);
  const bool reg = kp.p1 != 0.0;
  const Index tb = tleaf_start[leaf], te = tleaf_start[leaf + 1];
  // NT targets per thread (1 or 2), consecutive, so that threads without targets fill whole
  // warps, which only help stage the sources.
  auto pass = [&]<int NT>(Index i0) {
    bool active[NT];
    Index idx[NT];
    P4<double> t[NT];
    bool any = false;
#pragma unroll
    for (int q = 0; q < NT; ++q) {
      idx[q] = i0 + NT * threadIdx.x + q;
      active[q] = idx[q] < te;
      any |= active[q];
      t[q] = active[q] ? tpos[idx[q]] : P4<double>{0.0, 0.0, 0.0, 0.0};
    }
    const bool warp_busy = __any_sync(0xffffffffu, any);
    double tot[NT];
#pragma unroll
    for (int q = 0; q < NT; ++q) tot[q] = 0.0;
    for (int nb = 0; nb < 27; ++nb) {
      const int s = s_nb[nb];
      if (s < 0) continue;
      float txh[NT], txl[NT], tyh[NT], tyl[NT], tzh[NT], tzl[NT];
#pragma unroll
      for (int q = 0; q < NT; ++q) {
        ff_split(t[q].x - static_cast<double>(nb / 9 - 1) * wleaf, txh[q], txl[q]);
        ff_split(t[q].y - static_cast<double>((nb / 3) % 3 - 1) * wleaf, tyh[q], tyl[q]);
        ff_split(t[q].z - static_cast<double>(nb % 3 - 1) * wleaf, tzh[q], tzl[q]);
      }
      const Index sb = sleaf_start[s], se = sleaf_start[s + 1];
      for (Index base = sb; base < se; base += 128) {
        const int cnt = static_cast<int>(min(static_cast<Index>(128), se - base));
        __syncthreads();
        if (threadIdx.x < cnt) {
          const P4<double> p = spos[base + threadIdx.x];
          float4 a, b;
          ff_split(p.x, a.x, a.y);
          ff_split(p.y, a.z, a.w);
          ff_split(p.z, b.x, b.y);
          ff_split(sw[base + threadIdx.x], b.z, b.w);
          s_a[threadIdx.x] = a;
          s_b[threadIdx.x] = b;
        }
        __syncthreads();
        if (!warp_busy) continue;
        float ah[NT], al[NT];
#pragma unroll
        for (int q = 0; q < NT; ++q) ah[q] = al[q] = 0.0f;
#pragma unroll 2
        for (int j = 0; j < cnt; ++j) {
          const float4 a = s_a[j], b = s_b[j];
#pragma unroll
          for (int q = 0; q < NT; ++q)
            ff_poly_accumulate<KIND>(txh[q], txl[q], tyh[q], tyl[q], tzh[q], tzl[q], a.x, a.y, a.z,
                                     a.w, b.x, b.y, b.z, b.w, reg, c_hi, c_lo, ah[q], al[q]);
        }
#pragma unroll
        for (int q = 0; q < NT; ++q) tot[q] += static_cast<double>(ah[q]) + static_cast<double>(al[q]);
      }
    }
    const double scale = KIND == PGPU_RBF_BH3 ? -kp.p0 : kp.p0;
#pragma unroll
    for (int q = 0; q < NT; ++q)
      if (active[q]) out[tperm[idx[q]]] += scale * tot[q];
  };
  for (Index i0 = tb; i0 < te;) {
    if (te - i0 > static_cast<Index>(blockDim.x)) {
      pass.template operator()<2>(i0);
      i0 += 2 * blockDim.x;
    } else {
      pass.template operator()<1>(i0);
      i0 += blockDim.x;
    }
  }
}

// Near field with one thread per target point, for target trees whose leaves hold few points
// (evaluation points spread over a volume while the sources sit on a surface): the block-per-
// leaf kernel above would leave most of its threads idle. Sources are read through the cache;
// threads of one leaf read the same sources (broadcast).
template <int KIND, class T>
__global__ void __launch_bounds__(128)
    p2p_point_kernel(KParams<T> kp, const P4<T>* __restrict__ tpos, const Index* __restrict__ tperm,
                     const int* __restrict__ tleaf, Index nt, const int* __restrict__ table,
                     const P4<T>* __restrict__ spos, const T* __restrict__ sw,
                     const Index* __restrict__ sleaf_start, T wleaf, double* __restrict__ out) {
  const Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= nt) return;
  const P4<T> t = tpos[i];
  const int* nbs = table + static_cast<Index>(tleaf[i]) * 27;
  const T wscale = pair_weight_scale<KIND>(kp);
  const T c2 = pair_r2_offset<KIND>(kp);
  double tot = 0.0;
  for (int nb = 0; nb < 27; ++nb) {
    const int s = nbs[nb];
    if (s < 0) continue;
    const T tx = t.x - static_cast<T>(nb / 9 - 1) * wleaf;
    const T ty = t.y - static_cast<T>((nb / 3) % 3 - 1) * wleaf;
    const T tz = t.z - static_cast<T>(nb % 3 - 1) * wleaf;
    const Index sb = sleaf_start[s], se = sleaf_start[s + 1];
    T acc = T(0);
    for (Index j = sb; j < se; ++j) {
      const P4<T> q = spos[j];
      acc = pair_term<KIND>(tx - q.x, ty - q.y, tz - q.z, sw[j] * wscale, c2, kp, acc);
    }
    tot += static_cast<double>(acc);
  }
  out[tperm[i]] += tot;
}

// Leaf index of every sorted point.
__global__ void leaf_of_kernel(const Index* __restrict__ start, Index nleaf, int* __restrict__ leaf) {
  const Index l = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (l >= nleaf) return;
  for (Index i = start[l]; i < start[l + 1]; ++i) leaf[i] = static_cast<int>(l);
}

template <class T>
__global__ void count_pairs_kernel(const Index* __restrict__ tleaf_start, Index ntl,
                                   const int* __restrict__ table,
                                   const Index* __restrict__ sleaf_start,
                                   unsigned long long* __restrict__ total) {
  Index t = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= ntl) return;
  unsigned long long nt = tleaf_start[t + 1] - tleaf_start[t];
  unsigned long long ns = 0;
  for (int j = 0; j < 27; ++j) {
    int s = table[t * 27 + j];
    if (s >= 0) ns += sleaf_start[s + 1] - sleaf_start[s];
  }
  atomicAdd(total, nt * ns);
}

// ---- host-side structures ------------------------------------------------------------------

template <class T>
struct Tree {
  Index n = 0;
  int lf = 0;
  DevBuf<Index> perm;
  DevBuf<P4<T>> pos;  // sorted
  // FP32 trees only: sorted level-kSortLevel keys, and (built on first use) the leaf-relative
  // positions in FP64 for an FP64 near field.
  DevBuf<uint64_t> skeys;
  DevBuf<P4<double>> pos64;
  // per level k = 0..lf
  std::vector<DevBuf<uint64_t>> keys;
  std::vector<Index> ncell;
  std::vector<DevBuf<Index>> start;   // level lf: point ranges (n_leaf + 1); k < lf: child ranges
  std::vector<DevBuf<Index>> parent;  // level k: parent index (k >= 1)
};

void copy_index(Index* dst, const Index* src, Index n) {
  PGPU_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(Index), cudaMemcpyDeviceToDevice, stream()));
}

// Points sorted once by their Morton key at the deepest candidate level; the key of any
// shallower level is a right shift of it, so the leaf level can be chosen after sorting.
constexpr int kSortLevel = 10;

struct SortedPoints {
  Index n = 0;
  DevBuf<uint64_t> keys;  // level kSortLevel, ascending
  DevBuf<Index> perm;     // sorted position -> input index
};

void sort_points(SortedPoints& sp, const P4<double>* pos, Index n, const Box& box) {
  cudaStream_t st = stream();
  sp.n = n;
  sp.keys.resize(n);
  sp.perm.resize(n);
  if (n == 0) return;
  DevBuf<uint64_t> k_in(n);
  DevBuf<Index> i_in(n);
  keys_kernel<<<blocks_for(n, 256), 256, 0, st>>>(pos, n, box, kSortLevel, k_in.data(), i_in.data());
  PGPU_LAUNCH_CHECK();
  size_t tmp_bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, k_in.data(), sp.keys.data(), i_in.data(),
                                  sp.perm.data(), n, 0, 3 * kSortLevel, st);
  DevBuf<unsigned char> tmp(tmp_bytes);
  PGPU_CUDA(cub::DeviceRadixSort::SortPairs(tmp.data(), tmp_bytes, k_in.data(), sp.keys.data(),
                                            i_in.data(), sp.perm.data(), n, 0, 3 * kSortLevel, st));
}

// hist[d] = number of i with the first level at which key[i] and key[i-1] differ equal to d.
__global__ void occupancy_kernel(const uint64_t* __restrict__ keys, Index n,
                                 unsigned long long* __restrict__ hist) {
  __shared__ unsigned int h[kSortLevel + 1];
  if (threadIdx.x <= kSortLevel) h[threadIdx.x] = 0;
  __syncthreads();
  for (Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x + 1; i < n;
       i += static_cast<Index>(gridDim.x) * blockDim.x) {
    const uint64_t x = keys[i] ^ keys[i - 1];
    if (x == 0) continue;
    const int hb = 63 - __clzll(static_cast<long long>(x));
    atomicAdd(&h[kSortLevel - hb / 3], 1u);
  }
  __syncthreads();
  if (threadIdx.x <= kSortLevel && h[threadIdx.x]) atomicAdd(hist + threadIdx.x, h[threadIdx.x]);
}

// Occupied cells per level 0..kSortLevel.
std::vector<Index> occupancy(const SortedPoints& sp) {
  std::vector<Index> occ(kSortLevel + 1, sp.n > 0 ? 1 : 0);
  if (sp.n < 2) return occ;
  DevBuf<unsigned long long> hist(kSortLevel + 1);
  hist.zero();
  occupancy_kernel<<<std::min<Index>(blocks_for(sp.n, 256), 4 * num_sms()), 256, 0, stream()>>>(
      sp.keys.data(), sp.n, hist.data());
  PGPU_LAUNCH_CHECK();
  auto h = hist.to_host();
  Index run = 1;
  for (int k = 0; k <= kSortLevel; ++k) {
    run += static_cast<Index>(h[k]);
    occ[k] = run;
  }
  return occ;
}

template <class T>
void build_tree(Tree<T>& tr, const SortedPoints& sp, const P4<double>* pos, const Box& box, int lf) {
  cudaStream_t st = stream();
  const Index n = sp.n;
  tr.n = n;
  tr.lf = lf;
  tr.keys.clear();
  tr.keys.resize(lf + 1);
  tr.ncell.assign(lf + 1, 0);
  tr.start.clear();
  tr.start.resize(lf + 1);
  tr.parent.clear();
  tr.parent.resize(lf + 1);
  tr.perm.resize(n);
  tr.pos.resize(n);
  if (n == 0) return;
  copy_index(tr.perm.data(), sp.perm.data(), n);
  const int leaf_shift = 3 * (kSortLevel - lf);
  gather_rel_pos_kernel<T><<<blocks_for(n, 256), 256, 0, st>>>(pos, tr.perm.data(), sp.keys.data(),
                                                                 leaf_shift, n, box, lf,
                                                                 tr.pos.data());
  PGPU_LAUNCH_CHECK();
  tr.pos64.release();
  if constexpr (sizeof(T) == 4) {
    tr.skeys.resize(n);
    PGPU_CUDA(cudaMemcpyAsync(tr.skeys.data(), sp.keys.data(), n * sizeof(uint64_t),
                              cudaMemcpyDeviceToDevice, st));
  }

  // Run-length encode level by level: level lf from the sorted point keys, then parents.
  DevBuf<Index> flags(n), scan(n);
  const uint64_t* src_keys = sp.keys.data();
  Index src_n = n;
  for (int k = lf; k >= 0; --k) {
    const int shift = (k == lf) ? leaf_shift : 3;
    rle_flags_kernel<<<blocks_for(src_n, 256), 256, 0, st>>>(src_keys, src_n, shift, flags.data());
    PGPU_LAUNCH_CHECK();
    size_t sb = 0;
    cub::DeviceScan::InclusiveSum(nullptr, sb, flags.data(), scan.data(), src_n, st);
    DevBuf<unsigned char> stmp(sb);
    PGPU_CUDA(cub::DeviceScan::InclusiveSum(stmp.data(), sb, flags.data(), scan.data(), src_n, st));
    Index nu = 0;
    PGPU_CUDA(cudaMemcpyAsync(&nu, scan.data() + src_n - 1, sizeof(Index), cudaMemcpyDeviceToHost, st));
    sync();
    tr.ncell[k] = nu;
    tr.keys[k].resize(nu);
    tr.start[k].resize(nu + 1);
    if (k < lf) tr.parent[k + 1].resize(src_n);
    rle_scatter_kernel<<<blocks_for(src_n, 256), 256, 0, st>>>(
        src_keys, src_n, shift, scan.data(), tr.keys[k].data(), tr.start[k].data(),
        k < lf ? tr.parent[k + 1].data() : nullptr);
    PGPU_LAUNCH_CHECK();
    PGPU_CUDA(cudaMemcpyAsync(tr.start[k].data() + nu, &src_n, sizeof(Index), cudaMemcpyHostToDevice, st));
    sync();
    src_keys = tr.keys[k].data();
    src_n = nu;
  }
}

// M2L operator matrices K_o (the 7^3 offsets, p^3 x p^3 each) between cells of radius r.
template <class T>
std::shared_ptr<DevBuf<T>> m2l_matrices(int kind, const KParams<T>& kp, double r, int p) {
  const Index p3 = static_cast<Index>(p) * p * p;
  auto buf = std::make_shared<DevBuf<T>>(static_cast<size_t>(kNOff) * p3 * p3);
  std::vector<double> nodes(p);
  for (int m = 0; m < p; ++m) nodes[m] = cheb_node(p, m);
  DevBuf<double> dn;
  dn.upload(nodes);
  dispatch_fmm_kind(kind, [&]<int K>() {
    m2l_matrix_kernel<K, T><<<4 * num_sms(), 256, 0, stream()>>>(kp, p, r, dn.data(), buf->data());
    return 0;
  });
  PGPU_LAUNCH_CHECK();
  sync();
  return buf;
}

// ---- low-rank M2L (SVD compression of the stacked operators) ------------------------------
// With K_o ~ U C_o V^T for all offsets o (U, V: the leading left/right singular vectors of the
// stacked [K_o] matrices), M2L becomes L = U sum_o C_o (V^T M_s): an r x r product per
// interaction instead of p^3 x p^3, plus one projection per cell on each side.

// Cyclic Jacobi eigen-decomposition of a symmetric n x n matrix (row-major). Eigenvalues are
// returned in descending order with the eigenvectors as the columns of vecs (row-major).
void jacobi_eig(int n, std::vector<double> a, std::vector<double>& vals, std::vector<double>& vecs) {
  std::vector<double> v(static_cast<size_t>(n) * n, 0.0);
  for (int i = 0; i < n; ++i) v[static_cast<size_t>(i) * n + i] = 1.0;
  auto A = [&](int i, int j) -> double& { return a[static_cast<size_t>(i) * n + j]; };
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0, diag = 0;
    for (int i = 0; i < n; ++i) {
      diag += A(i, i) * A(i, i);
      for (int j = i + 1; j < n; ++j) off += A(i, j) * A(i, j);
    }
    if (off <= 1e-30 * diag || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A(p, q);
        if (std::fabs(apq) < 1e-300) continue;
        const double theta = (A(q, q) - A(p, p)) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {  // columns p, q
          const double akp = A(k, p), akq = A(k, q);
          A(k, p) = c * akp - s * akq;
          A(k, q) = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {  // rows p, q
          const double apk = A(p, k), aqk = A(q, k);
          A(p, k) = c * apk - s * aqk;
          A(q, k) = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = v[static_cast<size_t>(k) * n + p], vkq = v[static_cast<size_t>(k) * n + q];
          v[static_cast<size_t>(k) * n + p] = c * vkp - s * vkq;
          v[static_cast<size_t>(k) * n + q] = s * vkp + c * vkq;
        }
      }
  }
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](int x, int y) { return A(x, x) > A(y, y); });
  vals.resize(n);
  vecs.assign(static_cast<size_t>(n) * n, 0.0);
  for (int j = 0; j < n; ++j) {
    vals[j] = A(order[j], order[j]);
    for (int i = 0; i < n; ++i) vecs[static_cast<size_t>(i) * n + j] = v[static_cast<size_t>(i) * n + order[j]];
  }
}

__device__ __forceinline__ bool adjacent_offset(int o) {
  const int ox = o / 49 - 3, oy = (o / 7) % 7 - 3, oz = o % 7 - 3;
  return abs(ox) <= 1 && abs(oy) <= 1 && abs(oz) <= 1;
}

// G[i][j] = sum_o sum_k A_o[i][k] A_o[j][k] (rows) or sum_o sum_k A_o[k][i] A_o[k][j] (cols).
__global__ void gram_kernel(const double* __restrict__ K, int n, int cols, double* __restrict__ G) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * n) return;
  const int i = e / n, j = e % n;
  if (j < i) return;
  double s = 0;
  for (int o = 0; o < kNOff; ++o) {
    if (adjacent_offset(o)) continue;
    const double* A = K + static_cast<Index>(o) * n * n;
    if (cols) {
      for (int k = 0; k < n; ++k) s += A[static_cast<Index>(k) * n + i] * A[static_cast<Index>(k) * n + j];
    } else {
      for (int k = 0; k < n; ++k) s += A[static_cast<Index>(i) * n + k] * A[static_cast<Index>(j) * n + k];
    }
  }
  G[static_cast<Index>(i) * n + j] = s;
  G[static_cast<Index>(j) * n + i] = s;
}

// W_o = K_o V (n x r), then C_o = U^T W_o (r x r); U, V row-major n x r.
__global__ void kv_kernel(const double* __restrict__ K, const double* __restrict__ V, int n, int r,
                          double* __restrict__ W) {
  const Index e = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= static_cast<Index>(kNOff) * n * r) return;
  const int o = static_cast<int>(e / (static_cast<Index>(n) * r));
  const int a = static_cast<int>((e / r) % n), j = static_cast<int>(e % r);
  if (adjacent_offset(o)) {
    W[e] = 0.0;
    return;
  }
  const double* A = K + static_cast<Index>(o) * n * n + static_cast<Index>(a) * n;
  double s = 0;
  for (int b = 0; b < n; ++b) s += A[b] * V[static_cast<Index>(b) * r + j];
  W[e] = s;
}

template <class T>
__global__ void ukv_kernel(const double* __restrict__ W, const double* __restrict__ U, int n, int r,
                           double scale, T* __restrict__ C) {
  const Index e = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= static_cast<Index>(kNOff) * r * r) return;
  const int o = static_cast<int>(e / (static_cast<Index>(r) * r));
  const int i = static_cast<int>((e / r) % r), j = static_cast<int>(e % r);
  const double* Wo = W + static_cast<Index>(o) * n * r;
  double s = 0;
  for (int a = 0; a < n; ++a) s += U[static_cast<Index>(a) * r + i] * Wo[static_cast<Index>(a) * r + j];
  C[e] = static_cast<T>(scale * s);
}

// Mt[c][j] = sum_b M[c][b] V[b][j]  (one block per cell, threads over j)
template <class T>
__global__ void compress_kernel(const T* __restrict__ M, const T* __restrict__ V, int n, int r,
                                T* __restrict__ Mt) {
  extern __shared__ unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  const Index c = blockIdx.x;
  for (int b = threadIdx.x; b < n; b += blockDim.x) sm[b] = M[c * n + b];
  __syncthreads();
  for (int j = threadIdx.x; j < r; j += blockDim.x) {
    T s = T(0);
    for (int b = 0; b < n; ++b) s += sm[b] * V[static_cast<Index>(b) * r + j];
    Mt[c * r + j] = s;
  }
}

// L[c][a] += sum_j U[a][j] Lt[c][j]  (one block per cell, threads over a)
template <class T>
__global__ void expand_kernel(const T* __restrict__ Lt, const T* __restrict__ U, int n, int r,
                              T* __restrict__ L) {
  extern __shared__ unsigned char smem_raw[];
  T* sl = reinterpret_cast<T*>(smem_raw);
  const Index c = blockIdx.x;
  for (int j = threadIdx.x; j < r; j += blockDim.x) sl[j] = Lt[c * r + j];
  __syncthreads();
  for (int a = threadIdx.x; a < n; a += blockDim.x) {
    T s = T(0);
    for (int j = 0; j < r; ++j) s += U[static_cast<Index>(a) * r + j] * sl[j];
    L[c * n + a] += s;
  }
}

// Ranks the compressed kernel is instantiated for (multiples of 16; zero-padded bases).
constexpr int kRanks[] = {16, 32, 48, 64, 80, 96, 112, 128};

template <class T>
struct M2LOps {
  int n = 0;  // p^3
  int r = 0;  // padded rank; 0 = dense operators
  // Dense operators; for FP32 at order 6 with the tensor-core M2L on, the head/tail operator
  // blocks in the MMA layout (tc) replace them.
  std::shared_ptr<DevBuf<T>> K;
  std::shared_ptr<M2LTcBlocks> tc;
  DevBuf<T> U, V, C;  // low-rank form: K_o ~ U C_o V^T
  size_t bytes() const {
    size_t b = (U.size() + V.size() + C.size()) * sizeof(T);
    if (K) b += K->size() * sizeof(T);
    if (tc) b += (tc->hi.size() + tc->lo.size()) * sizeof(float);
    return b;
  }
};

struct SvdBasis {
  int r = 0;
  std::vector<double> U, V;  // n x r row-major
};

// Process-wide cache of M2L operators, keyed by (kind, p0, p1, cell radius, order, element
// size, eps). The homogeneous kernels (phi(s d) = s^deg phi(d)) are stored at radius 1 and
// scaled per level by the caller, so one entry serves every box; the others have one entry per
// radius, and the radius follows each point set's bounding box. The cache therefore keeps the
// most recently used entries within a byte budget (PGPU_M2L_CACHE_MB, default 8192). An entry
// dropped from the cache lives on while an FMM holds it; an FMM synchronizes its stream before
// it lets go of its entries, so whichever holder frees an entry last does so after every launch
// that read it has finished.
using OpKey = std::tuple<int, double, double, double, int, int, double>;

struct OpCache {
  std::mutex mu;
  std::list<OpKey> lru;  // most recently used first
  struct Slot {
    std::shared_ptr<void> ops;
    size_t bytes = 0;
    std::list<OpKey>::iterator pos;
  };
  std::map<OpKey, Slot> slots;
  size_t bytes = 0;
  // Bases of the low-rank form (host memory), cleared when they grow past a few dozen.
  std::map<std::tuple<int, double, double, double, int, double>, std::shared_ptr<SvdBasis>> bases;
};

OpCache g_op_cache;

size_t& op_cache_budget_ref() {
  static size_t budget = [] {
    const char* e = std::getenv("PGPU_M2L_CACHE_MB");
    const double mb = e ? std::max(std::atof(e), 0.0) : 8192.0;
    return static_cast<size_t>(mb * 1048576.0);
  }();
  return budget;
}

size_t op_cache_budget() { return op_cache_budget_ref(); }  // g_op_cache.mu held

std::shared_ptr<void> op_cache_find(const OpKey& key) {
  std::lock_guard<std::mutex> lk(g_op_cache.mu);
  auto it = g_op_cache.slots.find(key);
  if (it == g_op_cache.slots.end()) return nullptr;
  g_op_cache.lru.splice(g_op_cache.lru.begin(), g_op_cache.lru, it->second.pos);
  return it->second.ops;
}

// Inserts ops under key (or returns the entry another thread inserted first) and evicts the
// least recently used entries past the budget; the newest entry always stays.
std::shared_ptr<void> op_cache_insert(const OpKey& key, std::shared_ptr<void> ops, size_t bytes) {
  std::vector<std::shared_ptr<void>> evicted;  // released after the lock
  std::shared_ptr<void> out;
  {
    std::lock_guard<std::mutex> lk(g_op_cache.mu);
    auto it = g_op_cache.slots.find(key);
    if (it != g_op_cache.slots.end()) {
      g_op_cache.lru.splice(g_op_cache.lru.begin(), g_op_cache.lru, it->second.pos);
      out = it->second.ops;
    } else {
      g_op_cache.lru.push_front(key);
      g_op_cache.slots[key] = OpCache::Slot{ops, bytes, g_op_cache.lru.begin()};
      g_op_cache.bytes += bytes;
      out = std::move(ops);
      while (g_op_cache.bytes > op_cache_budget() && g_op_cache.slots.size() > 1) {
        auto victim = g_op_cache.slots.find(g_op_cache.lru.back());
        g_op_cache.bytes -= victim->second.bytes;
        evicted.push_back(std::move(victim->second.ops));
        g_op_cache.slots.erase(victim);
        g_op_cache.lru.pop_back();
      }
    }
  }
  return out;
}

}  // namespace

void m2l_cache_stats(int64_t* bytes, int64_t* entries, int64_t* limit) {
  std::lock_guard<std::mutex> lk(g_op_cache.mu);
  if (bytes) *bytes = static_cast<int64_t>(g_op_cache.bytes);
  if (entries) *entries = static_cast<int64_t>(g_op_cache.slots.size());
  if (limit) *limit = static_cast<int64_t>(op_cache_budget());
}

void m2l_cache_set_limit(int64_t bytes) {
  std::vector<std::shared_ptr<void>> evicted;  // released after the lock
  std::lock_guard<std::mutex> lk(g_op_cache.mu);
  op_cache_budget_ref() = static_cast<size_t>(std::max<int64_t>(bytes, 0));
  while (g_op_cache.bytes > op_cache_budget() && !g_op_cache.slots.empty()) {
    auto victim = g_op_cache.slots.find(g_op_cache.lru.back());
    g_op_cache.bytes -= victim->second.bytes;
    evicted.push_back(std::move(victim->second.ops));
    g_op_cache.slots.erase(victim);
    g_op_cache.lru.pop_back();
  }
}

namespace {

// Homogeneous kernels (phi(s d) = s^deg phi(d)): returns deg, or -1.
int homogeneity_degree(int kind, double c) {
  if (c != 0.0) return -1;
  if (kind == PGPU_RBF_BH3) return 1;
  if (kind == PGPU_RBF_TH3) return 3;
  return -1;
}

// The M2L operators for cells of radius r_cell, at radius 1 for homogeneous kernels: the caller
// multiplies the multipole expansions of the level by *scale (r_cell^deg) before the transfer.
template <class T>
std::shared_ptr<M2LOps<T>> m2l_ops(int kind, const KParams<T>& kp, double r_cell, int p, double eps,
                                   double* scale) {
  const int n = p * p * p;
  const double c = static_cast<double>(kp.p1);
  const int deg = homogeneity_degree(kind, c);
  const double r0 = deg >= 0 ? 1.0 : r_cell;
  *scale = deg >= 0 ? std::pow(r_cell, deg) : 1.0;
  const OpKey key = std::make_tuple(kind, static_cast<double>(kp.p0), c, r0, p,
                                    static_cast<int>(sizeof(T)), eps);
  if (auto hit = op_cache_find(key)) return std::static_pointer_cast<M2LOps<T>>(hit);
  auto ops = std::make_shared<M2LOps<T>>();
  ops->n = n;
  if (eps <= 0.0 || p > 6) {
    ops->K = m2l_matrices<T>(kind, kp, r0, p);
  } else {
    KParams<double> kd{static_cast<double>(kp.p0), c};
    auto K64 = m2l_matrices<double>(kind, kd, r0, p);
    auto bkey = std::make_tuple(kind, static_cast<double>(kp.p0), c, r0, p, eps);
    std::shared_ptr<SvdBasis> basis;
    {
      std::lock_guard<std::mutex> lk(g_op_cache.mu);
      auto it = g_op_cache.bases.find(bkey);
      if (it != g_op_cache.bases.end()) basis = it->second;
    }
    if (!basis) {
      basis = std::make_shared<SvdBasis>();
      DevBuf<double> g(static_cast<size_t>(n) * n);
      std::vector<double> gu, gv, vals_u, vals_v, vec_u, vec_v;
      gram_kernel<<<blocks_for(static_cast<Index>(n) * n, 128), 128, 0, stream()>>>(K64->data(), n, 0, g.data());
      PGPU_LAUNCH_CHECK();
      gu = g.to_host();
      gram_kernel<<<blocks_for(static_cast<Index>(n) * n, 128), 128, 0, stream()>>>(K64->data(), n, 1, g.data());
      PGPU_LAUNCH_CHECK();
      gv = g.to_host();
      jacobi_eig(n, gu, vals_u, vec_u);
      jacobi_eig(n, gv, vals_v, vec_v);
      // Smallest rank whose discarded energy is below eps^2 of the total, on both sides.
      auto rank_of = [&](const std::vector<double>& vals) {
        double tot = 0;
        for (double v : vals) tot += std::max(v, 0.0);
        double tail = tot;
        int r = 0;
        while (r < n && tail > eps * eps * tot) tail -= std::max(vals[r++], 0.0);
        return r;
      };
      int r = std::max(rank_of(vals_u), rank_of(vals_v));
      int rp = 0;
      for (int cand : kRanks)
        if (cand >= r) {
          rp = cand;
          break;
        }
      if (rp == 0 || rp >= n) {
        basis->r = 0;  // no useful compression
      } else {
        basis->r = rp;
        basis->U.assign(static_cast<size_t>(n) * rp, 0.0);
        basis->V.assign(static_cast<size_t>(n) * rp, 0.0);
        for (int a = 0; a < n; ++a)
          for (int j = 0; j < std::min(r, rp); ++j) {
            basis->U[static_cast<size_t>(a) * rp + j] = vec_u[static_cast<size_t>(a) * n + j];
            basis->V[static_cast<size_t>(a) * rp + j] = vec_v[static_cast<size_t>(a) * n + j];
          }
      }
      std::lock_guard<std::mutex> lk(g_op_cache.mu);
      if (g_op_cache.bases.size() >= 64) g_op_cache.bases.clear();
      g_op_cache.bases[bkey] = basis;
    }
    if (basis->r == 0) {
      ops->K = m2l_matrices<T>(kind, kp, r0, p);
    } else {
      const int r = basis->r;
      ops->r = r;
      DevBuf<double> du, dv, w(static_cast<size_t>(kNOff) * n * r);
      du.upload(basis->U);
      dv.upload(basis->V);
      const Index nw = static_cast<Index>(kNOff) * n * r;
      kv_kernel<<<blocks_for(nw, 256), 256, 0, stream()>>>(K64->data(), dv.data(), n, r, w.data());
      PGPU_LAUNCH_CHECK();
      ops->C.resize(static_cast<size_t>(kNOff) * r * r);
      const Index nc = static_cast<Index>(kNOff) * r * r;
      ukv_kernel<T><<<blocks_for(nc, 256), 256, 0, stream()>>>(w.data(), du.data(), n, r, 1.0,
                                                                ops->C.data());
      PGPU_LAUNCH_CHECK();
      std::vector<T> hu(basis->U.begin(), basis->U.end()), hv(basis->V.begin(), basis->V.end());
      ops->U.upload(hu);
      ops->V.upload(hv);
    }
  }
  if constexpr (sizeof(T) == 4) {
    if (p == 6 && ops->r == 0 && m2l_tc_enabled()) {
      ops->tc = std::make_shared<M2LTcBlocks>(make_m2l_tc_blocks(ops->K->data()));
      ops->K.reset();
    }
  }
  sync();  // the entry is read from other threads' streams
  const size_t bytes = ops->bytes();
  return std::static_pointer_cast<M2LOps<T>>(op_cache_insert(key, std::move(ops), bytes));
}

int order_for_accuracy(double accuracy) {
  // accuracy = inf: the reference's default order 6 (fmm_accuracy_estimator.hpp:77-79);
  // accuracy = 0: the highest order kept here (the reference interpolates at order 12 on a
  // uniform grid). A finite accuracy has its order chosen by the evaluator's estimate, which
  // sets it explicitly; this fallback maps it by magnitude.
  if (std::isinf(accuracy)) return 6;
  if (accuracy <= 0.0) return 8;
  if (accuracy >= 1e-4) return 6;
  return 8;
}

}  // namespace

template <class T>
struct Fmm<T>::Impl {
  int kind;
  KParams<T> kp;
  Mat3 a;
  Box box;
  double accuracy;
  FarFieldConfig cfg;
  bool cfg_set = false;
  int p = 6;
  Tree<T> src, trg;
  bool symmetric = false;
  const P4<double>* spos_in = nullptr;
  const P4<double>* tpos_in = nullptr;
  Index ns = 0, nt = 0;
  int lf = 2;
  bool near_only = false;  // compact support: near field only (FarFieldConfig::near_only)
  bool grad_out = false;   // gradient targets: three outputs per target (set_gradient_targets)
  bool dipole = false;     // gradient sources: three weights per source (set_gradient_sources)
  DevBuf<T> sw3;           // sorted gradient-source weights
  bool built = false;
  // M2L tables per level (target cells x 343) and P2P table (target leaves x 27).
  std::vector<DevBuf<int>> m2l_table;
  DevBuf<int> p2p_table;
  DevBuf<int> tleaf;  // leaf of each sorted target point (sparse target leaves only)
  DevBuf<int> chunk_leaf;  // P2P chunk -> (target leaf, chunk index within the leaf)
  Index n_chunks = 0;
  // Shared M2L operators per level (cached process-wide) and the factor each level's multipole
  // expansions take before the transfer (r^deg for the homogeneous kernels, else 1).
  std::vector<std::shared_ptr<M2LOps<T>>> kmats;
  std::vector<double> kscale;
  std::vector<DevBuf<T>> M, L, Mt, Lt;  // Mt/Lt: compressed expansions (rank r) when used
  DevBuf<T> sw;
  Index near_pairs = 0;
  std::vector<Index> m2l_pairs;  // interactions per level
  Cheb<T> ch;
  // FP64 near field for an FP32 tree (set_near_fp64).
  bool near64 = false;
  KParams<double> kp64{};
  // Timeout flag of the tensor-core M2L (set on the device, checked after each evaluation).
  DevBuf<int> tc_err;
  bool tc_used = false;

  Tree<T>& ttree() { return symmetric ? src : trg; }

  ~Impl() { release_ops(); }

  // Other threads' FMMs read the shared operators: this stream's launches finish before the
  // references go, so the holder that frees an operator set last frees it unused.
  void release_ops() {
    if (kmats.empty()) return;
    sync_quiet();
    kmats.clear();
  }

  void ensure_pos64(Tree<T>& tr, const P4<double>* pos_in) {
    if (tr.n == 0 || tr.pos64.size() == static_cast<size_t>(tr.n)) return;
    tr.pos64.resize(tr.n);
    gather_rel_pos_kernel<double><<<blocks_for(tr.n, 256), 256, 0, stream()>>>(
        pos_in, tr.perm.data(), tr.skeys.data(), 3 * (kSortLevel - lf), tr.n, box, lf,
        tr.pos64.data());
    PGPU_LAUNCH_CHECK();
  }

  // Leaf level from the measured occupancy: the level whose average number of sources per
  // occupied leaf is closest (in ratio) to the target — surface data fills far fewer cells than
  // uniform data, so a level chosen from the point count alone would overfill the leaves.
  int choose_leaf_level(const std::vector<Index>& occ) const {
    if (cfg_set && cfg.leaf_level >= 0) return std::min(cfg.leaf_level, kSortLevel);
    // PGPU_FMM_LEAF_POINTS overrides the FP32 target (a tuning knob for the benchmark).
    static const double env_target =
        std::getenv("PGPU_FMM_LEAF_POINTS") ? std::atof(std::getenv("PGPU_FMM_LEAF_POINTS")) : 0.0;
    // FP32: 160 (the tensor-core M2L makes cells dearer than near-field pairs; measured on
    // the 3M-point surface fit against 96 and 256).
    const double target = sizeof(T) == 4 ? (env_target > 0 ? env_target : 160.0) : 40.0;
    int best = 2;
    double best_d = INFINITY;
    for (int k = 2; k <= kSortLevel; ++k) {
      const double avg = static_cast<double>(ns) / std::max<Index>(occ[k], 1);
      const double d = std::fabs(std::log(std::max(avg, 1e-9) / target));
      if (d < best_d) {
        best_d = d;
        best = k;
      }
    }
    return best;
  }

  void build() {
    SortedPoints ss, ts;
    sort_points(ss, spos_in, ns, box);
    if (!symmetric) sort_points(ts, tpos_in, nt, box);
    near_only = cfg_set && cfg.near_only;
    if (near_only) {
      // The finest level whose leaves are at least the support radius wide.
      int k = 2;
      while (k < kSortLevel && box.width / static_cast<double>(1 << (k + 1)) >= cfg.near_radius) ++k;
      lf = k;
    } else {
      lf = choose_leaf_level(occupancy(ss));
    }
    p = cfg_set && cfg.order > 0 ? cfg.order : order_for_accuracy(accuracy);
    if (p != 4 && p != 6 && p != 8) p = 6;
    ch = make_cheb<T>(p);
    build_tree(src, ss, spos_in, box, lf);
    if (!symmetric) build_tree(trg, ts, tpos_in, box, lf);
    Tree<T>& tt = ttree();
    cudaStream_t st = stream();
    // Interaction tables.
    m2l_table.clear();
    m2l_table.resize(lf + 1);
    m2l_pairs.assign(lf + 1, 0);
    release_ops();
    kmats.assign(lf + 1, nullptr);
    kscale.assign(lf + 1, 1.0);
    for (int k = 2; k <= (near_only ? 1 : lf); ++k) {
      const Index n_t = tt.ncell[k];
      m2l_table[k].resize(std::max<Index>(n_t, 1) * kNOff);
      PGPU_CUDA(cudaMemsetAsync(m2l_table[k].data(), 0xff, m2l_table[k].size() * sizeof(int), st));
      DevBuf<Index> cnt(std::max<Index>(n_t, 1));
      if (n_t > 0) {
        m2l_table_kernel<<<blocks_for(n_t, 128), 128, 0, st>>>(tt.keys[k].data(), n_t,
                                                               src.keys[k].data(), src.ncell[k], k,
                                                               m2l_table[k].data(), cnt.data());
        PGPU_LAUNCH_CHECK();
        auto hc = cnt.to_host();
        Index s = 0;
        for (Index i = 0; i < n_t; ++i) s += hc[i];
        m2l_pairs[k] = s;
      }
      const double r = box.width / static_cast<double>(1 << k) / 2.0;
      // Dense operators by default. PGPU_M2L_EPS > 0 selects low-rank operators whose discarded
      // singular values carry at most eps^2 of the stacked operators' energy; at the accuracy the
      // fits need (eps <= 1e-8 with order 6) the rank exceeds 128 and nothing is gained.
      static const double env_eps = std::getenv("PGPU_M2L_EPS") ? std::atof(std::getenv("PGPU_M2L_EPS")) : 0.0;
      const double eps = env_eps;
      kmats[k] = m2l_ops<T>(kind, kp, r, p, eps, &kscale[k]);
      if (verbose() && k == lf)
        std::printf("fmm: n %ld -> lf %d, p %d, m2l rank %d\n", static_cast<long>(ns), lf, p,
                    kmats[k]->r);
    }
    const Index ntl = tt.ncell[lf];
    p2p_table.resize(std::max<Index>(ntl, 1) * 27);
    if (ntl > 0) {
      p2p_table_kernel<<<blocks_for(ntl, 128), 128, 0, st>>>(tt.keys[lf].data(), ntl,
                                                             src.keys[lf].data(), src.ncell[lf], lf,
                                                             p2p_table.data());
      PGPU_LAUNCH_CHECK();
      DevBuf<unsigned long long> tot(1);
      PGPU_CUDA(cudaMemsetAsync(tot.data(), 0, sizeof(unsigned long long), st));
      count_pairs_kernel<T><<<blocks_for(ntl, 128), 128, 0, st>>>(
          tt.start[lf].data(), ntl, p2p_table.data(), src.start[lf].data(), tot.data());
      PGPU_LAUNCH_CHECK();
      unsigned long long h = 0;
      PGPU_CUDA(cudaMemcpyAsync(&h, tot.data(), sizeof(h), cudaMemcpyDeviceToHost, st));
      sync();
      near_pairs = static_cast<Index>(h);
      {
        DevBuf<int> cnt(ntl), off(ntl);
        chunk_count_kernel<<<blocks_for(ntl, 128), 128, 0, st>>>(tt.start[lf].data(), ntl,
                                                                 cnt.data());
        PGPU_LAUNCH_CHECK();
        size_t sb = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, sb, cnt.data(), off.data(), ntl, st);
        DevBuf<unsigned char> stmp(sb);
        PGPU_CUDA(cub::DeviceScan::ExclusiveSum(stmp.data(), sb, cnt.data(), off.data(), ntl, st));
        int last_cnt = 0, last_off = 0;
        PGPU_CUDA(cudaMemcpyAsync(&last_cnt, cnt.data() + ntl - 1, sizeof(int),
                                  cudaMemcpyDeviceToHost, st));
        PGPU_CUDA(cudaMemcpyAsync(&last_off, off.data() + ntl - 1, sizeof(int),
                                  cudaMemcpyDeviceToHost, st));
        sync();
        n_chunks = static_cast<Index>(last_off) + last_cnt;
        chunk_leaf.resize(2 * std::max<Index>(n_chunks, 1));
        chunk_fill_kernel<<<blocks_for(ntl, 128), 128, 0, st>>>(cnt.data(), off.data(), ntl,
                                                                chunk_leaf.data());
        PGPU_LAUNCH_CHECK();
      }
      const Index ntp = symmetric ? ns : nt;
      if (!symmetric && ntp < 32 * ntl) {
        tleaf.resize(ntp);
        leaf_of_kernel<<<blocks_for(ntl, 128), 128, 0, st>>>(tt.start[lf].data(), ntl,
                                                             tleaf.data());
        PGPU_LAUNCH_CHECK();
      } else {
        tleaf.release();
      }
    }
    const Index p3 = static_cast<Index>(p) * p * p;
    M.clear();
    L.clear();
    M.resize(lf + 1);
    L.resize(lf + 1);
    Mt.clear();
    Lt.clear();
    Mt.resize(lf + 1);
    Lt.resize(lf + 1);
    for (int k = 2; k <= (near_only ? 1 : lf); ++k) {
      M[k].resize(std::max<Index>(src.ncell[k], 1) * p3);
      L[k].resize(std::max<Index>(tt.ncell[k], 1) * p3);
      if (kmats[k]->r > 0) {
        Mt[k].resize(std::max<Index>(src.ncell[k], 1) * kmats[k]->r);
        Lt[k].resize(std::max<Index>(tt.ncell[k], 1) * kmats[k]->r);
      }
    }
    sw.resize(std::max<Index>(ns, 1));
    built = true;
  }

  // One M2L pass over level k with operators of dimension D (p^3 dense or the compressed rank):
  // tiles of kTT target cells; when the tiles are few, the offsets are split over blockIdx.y and
  // the partial expansions summed in a fixed order.
  template <int D>
  void m2l_apply(const T* K, const T* Min, T* Lout, Index n_t, int k, cudaStream_t st) {
    if constexpr (D == 64 || D == 216) {
      constexpr int TT = 64;
      const Index tiles = (n_t + TT - 1) / TT;
      // Two blocks fit per SM: aim for at least four waves so the last one is a small fraction.
      int groups = static_cast<int>(
          std::min<Index>(16, std::max<Index>(1, (8 * num_sms() + tiles - 1) / tiles)));
      DevBuf<T> part;
      if (groups > 1) part.resize(static_cast<size_t>(groups) * n_t * D);
      m2l_tiled_kernel<D, T><<<dim3(static_cast<unsigned>(tiles), groups), 256, 0, st>>>(
          K, m2l_table[k].data(), n_t, Min, Lout, groups, part.data());
      PGPU_LAUNCH_CHECK();
      if (groups > 1) {
        const Index n = n_t * D;
        m2l_reduce_kernel<T><<<blocks_for(n, 256), 256, 0, st>>>(part.data(), groups, n, Lout);
        PGPU_LAUNCH_CHECK();
      }
      return;
    }
    const size_t smem = (static_cast<size_t>(D) * (kTT + 1) + 8 * D) * sizeof(T);
    auto kern = m2l_kernel<D, T>;
    PGPU_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(smem)));
    const Index tiles = (n_t + kTT - 1) / kTT;
    int groups = static_cast<int>(
        std::min<Index>(16, std::max<Index>(1, (2 * num_sms() + tiles - 1) / tiles)));
    DevBuf<T> part;
    if (groups > 1) part.resize(static_cast<size_t>(groups) * n_t * D);
    kern<<<dim3(static_cast<unsigned>(tiles), groups), 256, smem, st>>>(
        K, m2l_table[k].data(), n_t, Min, Lout, groups, part.data());
    PGPU_LAUNCH_CHECK();
    if (groups > 1) {
      const Index n = n_t * D;
      m2l_reduce_kernel<T><<<blocks_for(n, 256), 256, 0, st>>>(part.data(), groups, n, Lout);
      PGPU_LAUNCH_CHECK();
    }
  }

  template <int P>
  void run_far(cudaStream_t st, double* out) {
    constexpr int P3 = P * P * P;
    Tree<T>& tt = ttree();
    const bool f32 = sizeof(T) == 4;
    // Upward pass.
    if (src.ncell[lf] > 0) {
      ProfScope ps(f32 ? "fmm_p2m_f32" : "fmm_p2m_f64", 4.0 * P3 * static_cast<double>(ns),
                   static_cast<double>(ns) * 5 * sizeof(T));
      if (dipole)
        p2m_dipole_kernel<P, T><<<static_cast<unsigned>(src.ncell[lf]), 256, 0, st>>>(
            ch, src.pos.data(), sw3.data(), src.start[lf].data(), box, lf, M[lf].data());
      else
        p2m_kernel<P, T><<<static_cast<unsigned>(src.ncell[lf]), 256, 0, st>>>(
            ch, src.pos.data(), sw.data(), src.start[lf].data(), src.keys[lf].data(), box, lf,
            M[lf].data());
      PGPU_LAUNCH_CHECK();
    }
    for (int k = lf - 1; k >= 2; --k) {
      if (src.ncell[k] == 0) continue;
      ProfScope ps(f32 ? "fmm_m2m_f32" : "fmm_m2m_f64",
                   static_cast<double>(src.ncell[k + 1]) * 6.0 * P3 * P);
      m2m_kernel<P, T><<<static_cast<unsigned>(src.ncell[k]), ((P3 + 31) / 32) * 32, 0, st>>>(
          ch, src.start[k].data(), src.keys[k + 1].data(), M[k + 1].data(), M[k].data());
      PGPU_LAUNCH_CHECK();
    }
    // Operators of homogeneous kernels are stored at radius 1: the expansions take r^deg.
    for (int k = 2; k <= lf; ++k) {
      const Index n = src.ncell[k] * P3;
      if (n == 0 || tt.ncell[k] == 0 || kscale[k] == 1.0) continue;
      scale_expansions_kernel<T><<<blocks_for(n, 256), 256, 0, st>>>(M[k].data(), n,
                                                                       static_cast<T>(kscale[k]));
      PGPU_LAUNCH_CHECK();
    }
    // Transfer + downward pass.
    const size_t smem = (static_cast<size_t>(P3) * (kTT + 1) + 8 * P3) * sizeof(T);
    for (int k = 2; k <= lf; ++k) {
      const Index n_t = tt.ncell[k];
      if (n_t == 0) continue;
      PGPU_CUDA(cudaMemsetAsync(L[k].data(), 0, n_t * P3 * sizeof(T), st));
      if (k > 2) {
        ProfScope ps(f32 ? "fmm_l2l_f32" : "fmm_l2l_f64", static_cast<double>(n_t) * 6.0 * P3 * P);
        l2l_kernel<P, T><<<static_cast<unsigned>(n_t), ((P3 + 31) / 32) * 32, 0, st>>>(
            ch, tt.parent[k].data(), tt.keys[k].data(), L[k - 1].data(), L[k].data());
        PGPU_LAUNCH_CHECK();
      }
      if (src.ncell[k] > 0) {
        M2LOps<T>& ops = *kmats[k];
        bool tc = false;
        if constexpr (sizeof(T) == 4 && P3 == 216) {
          tc = ops.tc != nullptr;
          if (tc) {
            if (!tc_used) {
              tc_err.resize(1);
              tc_err.zero();
              tc_used = true;
            }
            ProfScope ps("fmm_m2l_tc", 2.0 * P3 * P3 * static_cast<double>(m2l_pairs[k]));
            m2l_tc_apply(*ops.tc, m2l_table[k].data(), n_t, M[k].data(), L[k].data(),
                         tc_err.data(), st);
          }
        }
        if (tc) {
        } else if (ops.r == 0) {
          ProfScope ps(f32 ? "fmm_m2l_f32" : "fmm_m2l_f64",
                       2.0 * P3 * P3 * static_cast<double>(m2l_pairs[k]));
          (void)smem;
          m2l_apply<P3>(ops.K->data(), M[k].data(), L[k].data(), n_t, k, st);
        } else {
          const int r = ops.r;
          const Index ns_k = src.ncell[k];
          {
            ProfScope ps(f32 ? "fmm_m2l_proj_f32" : "fmm_m2l_proj_f64",
                         2.0 * P3 * r * static_cast<double>(ns_k + n_t));
            compress_kernel<T><<<static_cast<unsigned>(ns_k), 128, P3 * sizeof(T), st>>>(
                M[k].data(), ops.V.data(), P3, r, Mt[k].data());
            PGPU_LAUNCH_CHECK();
          }
          {
            ProfScope ps(f32 ? "fmm_m2l_f32" : "fmm_m2l_f64",
                         2.0 * r * r * static_cast<double>(m2l_pairs[k]));
            PGPU_CUDA(cudaMemsetAsync(Lt[k].data(), 0, n_t * r * sizeof(T), st));
            switch (r) {
              case 16: m2l_apply<16>(ops.C.data(), Mt[k].data(), Lt[k].data(), n_t, k, st); break;
              case 32: m2l_apply<32>(ops.C.data(), Mt[k].data(), Lt[k].data(), n_t, k, st); break;
              case 48: m2l_apply<48>(ops.C.data(), Mt[k].data(), Lt[k].data(), n_t, k, st); break;
              case 64: m2l_apply<64>(ops.C.data(), Mt[k].data(), Lt[k].data(), n_t, k, st); break;
              case 80: m2l_apply<80>(ops.C.data(), Mt[k].data(), Lt[k].data(), n_t, k, st); break;
              case 96: m2l_apply<96>(ops.C.data(), Mt[k].data(), Lt[k].data(), n_t, k, st); break;
              case 112: m2l_apply<112>(ops.C.data(), Mt[k].data(), Lt[k].data(), n_t, k, st); break;
              default: m2l_apply<128>(ops.C.data(), Mt[k].data(), Lt[k].data(), n_t, k, st); break;
            }
          }
          {
            ProfScope ps(f32 ? "fmm_m2l_proj_f32" : "fmm_m2l_proj_f64", 0.0);
            expand_kernel<T><<<static_cast<unsigned>(n_t), 128, r * sizeof(T), st>>>(
                Lt[k].data(), ops.U.data(), P3, r, L[k].data());
            PGPU_LAUNCH_CHECK();
          }
        }
      }
    }
    if (tt.ncell[lf] > 0) {
      const double npt = static_cast<double>(symmetric ? ns : nt);
      ProfScope ps(f32 ? "fmm_l2p_f32" : "fmm_l2p_f64", npt * (2.0 * P3 + 6.0 * P * P));
      if (grad_out)
        l2p_grad_kernel<P, T><<<static_cast<unsigned>(n_chunks), 128, 0, st>>>(
            ch, tt.pos.data(), tt.perm.data(), tt.start[lf].data(), chunk_leaf.data(), box, lf,
            L[lf].data(), out);
      else
        l2p_kernel<P, T><<<static_cast<unsigned>(n_chunks), 128, 0, st>>>(
            ch, tt.pos.data(), tt.perm.data(), tt.start[lf].data(), chunk_leaf.data(), box, lf,
            L[lf].data(), out);
      PGPU_LAUNCH_CHECK();
    }
  }

  void evaluate(const T* vw, const T* gg, const double* w64, double* out) {
    if (!built) build();
    cudaStream_t st = stream();
    Tree<T>& tt = ttree();
    if (ns == 0 || (symmetric ? ns : nt) == 0) return;
    // Gradient sources keep their near field in T (their FP64 weights are not at hand here).
    const bool fp64_near = sizeof(T) == 4 && near64 && w64 != nullptr && !dipole;
    if (dipole) {
      sw3.resize(static_cast<size_t>(3 * ns));
      gather_w3_kernel<T><<<blocks_for(ns, 256), 256, 0, st>>>(gg, src.perm.data(), ns, sw3.data());
    } else {
      gather_w_kernel<T><<<blocks_for(ns, 256), 256, 0, st>>>(vw, src.perm.data(), ns, sw.data());
    }
    PGPU_LAUNCH_CHECK();
    if (lf >= 2 && !near_only) {
      switch (p) {
        case 4: run_far<4>(st, out); break;
        case 8: run_far<8>(st, out); break;
        default: run_far<6>(st, out); break;
      }
      if (tc_used) {
        int e = 0;
        PGPU_CUDA(cudaMemcpyAsync(&e, tc_err.data(), sizeof(int), cudaMemcpyDeviceToHost, st));
        sync();
        if (e != 0) {
          tc_err.zero();  // the next evaluation starts with a clear flag
          throw Error(PGPU_TIMEOUT, "tensor-core M2L: a bounded wait ran out");
        }
      }
    }
    const Index ntl = tt.ncell[lf];
    if (ntl > 0 && dipole) {
      ProfScope ps(sizeof(T) == 4 ? "fmm_p2p_dipole_f32" : "fmm_p2p_dipole_f64",
                   (grad_out ? 9.0 : 3.0) * pair_flops(kind) * static_cast<double>(near_pairs));
      const T wl = static_cast<T>(box.width / static_cast<double>(1 << lf));
      dispatch_kind(kind, [&]<int K>() {
        if (grad_out)
          p2p_dipole_kernel<K, T, true><<<static_cast<unsigned>(n_chunks), 128, 0, st>>>(
              kp, tt.pos.data(), tt.perm.data(), tt.start[lf].data(), chunk_leaf.data(),
              p2p_table.data(), src.pos.data(), sw3.data(), src.start[lf].data(), wl, out);
        else
          p2p_dipole_kernel<K, T, false><<<static_cast<unsigned>(n_chunks), 128, 0, st>>>(
              kp, tt.pos.data(), tt.perm.data(), tt.start[lf].data(), chunk_leaf.data(),
              p2p_table.data(), src.pos.data(), sw3.data(), src.start[lf].data(), wl, out);
        return 0;
      });
      PGPU_LAUNCH_CHECK();
    } else if (ntl > 0 && grad_out) {
      // Gradient targets (3 outputs per target), public smooth kinds only.
      ProfScope ps(sizeof(T) == 4 && !fp64_near ? "fmm_p2p_grad_f32" : "fmm_p2p_grad_f64",
                   3.0 * pair_flops(kind) * static_cast<double>(near_pairs));
      if (fp64_near) {
        ensure_pos64(src, spos_in);
        if (!symmetric) ensure_pos64(trg, tpos_in);
        DevBuf<double> sw64(ns);
        gather_w_kernel<double><<<blocks_for(ns, 256), 256, 0, st>>>(w64, src.perm.data(), ns,
                                                                     sw64.data());
        PGPU_LAUNCH_CHECK();
        const double wl = box.width / static_cast<double>(1 << lf);
        dispatch_kind(kind, [&]<int K>() {
          p2p_grad_kernel<K, double><<<static_cast<unsigned>(n_chunks), 128, 0, st>>>(
              kp64, tt.pos64.data(), tt.perm.data(), tt.start[lf].data(), chunk_leaf.data(),
              p2p_table.data(), src.pos64.data(), sw64.data(), src.start[lf].data(), wl, out);
          return 0;
        });
      } else {
        const T wl = static_cast<T>(box.width / static_cast<double>(1 << lf));
        dispatch_kind(kind, [&]<int K>() {
          p2p_grad_kernel<K, T><<<static_cast<unsigned>(n_chunks), 128, 0, st>>>(
              kp, tt.pos.data(), tt.perm.data(), tt.start[lf].data(), chunk_leaf.data(),
              p2p_table.data(), src.pos.data(), sw.data(), src.start[lf].data(), wl, out);
          return 0;
        });
      }
      PGPU_LAUNCH_CHECK();
    } else if (ntl > 0 && fp64_near) {
      ensure_pos64(src, spos_in);
      if (!symmetric) ensure_pos64(trg, tpos_in);
      DevBuf<double> sw64(ns);
      gather_w_kernel<double><<<blocks_for(ns, 256), 256, 0, st>>>(w64, src.perm.data(), ns,
                                                                   sw64.data());
      PGPU_LAUNCH_CHECK();
      const double wl = box.width / static_cast<double>(1 << lf);
      if (kind == PGPU_RBF_BH3 || kind == PGPU_RBF_TH3) {
        ProfScope ps("fmm_p2p_ff", pair_flops(kind) * static_cast<double>(near_pairs));
        if (kind == PGPU_RBF_BH3)
          p2p_ff_kernel<PGPU_RBF_BH3><<<static_cast<unsigned>(ntl), 128, 0, st>>>(
              kp64, tt.pos64.data(), tt.perm.data(), tt.start[lf].data(), p2p_table.data(),
              src.pos64.data(), sw64.data(), src.start[lf].data(), wl, out);
        else
          p2p_ff_kernel<PGPU_RBF_TH3><<<static_cast<unsigned>(ntl), 128, 0, st>>>(
              kp64, tt.pos64.data(), tt.perm.data(), tt.start[lf].data(), p2p_table.data(),
              src.pos64.data(), sw64.data(), src.start[lf].data(), wl, out);
        PGPU_LAUNCH_CHECK();
      } else {
        ProfScope ps("fmm_p2p_f64", pair_flops(kind) * static_cast<double>(near_pairs));
        dispatch_fmm_kind(kind, [&]<int K>() {
          p2p_kernel<K, double><<<static_cast<unsigned>(n_chunks), 128, 0, st>>>(
              kp64, tt.pos64.data(), tt.perm.data(), tt.start[lf].data(), chunk_leaf.data(),
              p2p_table.data(), src.pos64.data(), sw64.data(), src.start[lf].data(), wl, out);
          return 0;
        });
        PGPU_LAUNCH_CHECK();
      }
    } else if (ntl > 0) {
      ProfScope ps(symmetric ? (sizeof(T) == 4 ? "fmm_p2p_f32" : "fmm_p2p_f64")
                             : (sizeof(T) == 4 ? "fmm_p2p_f32_st" : "fmm_p2p_f64_st"),
                   pair_flops(kind) * static_cast<double>(near_pairs));
      const T wl = static_cast<T>(box.width / static_cast<double>(1 << lf));
      if (tleaf.size() > 0) {
        dispatch_fmm_kind(kind, [&]<int K>() {
          p2p_point_kernel<K, T><<<blocks_for(nt, 128), 128, 0, st>>>(
              kp, tt.pos.data(), tt.perm.data(), tleaf.data(), nt, p2p_table.data(),
              src.pos.data(), sw.data(), src.start[lf].data(), wl, out);
          return 0;
        });
      } else {
        dispatch_fmm_kind(kind, [&]<int K>() {
          p2p_kernel<K, T><<<static_cast<unsigned>(n_chunks), 128, 0, st>>>(
              kp, tt.pos.data(), tt.perm.data(), tt.start[lf].data(), chunk_leaf.data(),
              p2p_table.data(), src.pos.data(), sw.data(), src.start[lf].data(), wl, out);
          return 0;
        });
      }
      PGPU_LAUNCH_CHECK();
    }
  }
};

template <class T>
bool Fmm<T>::near_only_supported(int kind) {
  return kind == PGPU_RBF_CUB || kind == PGPU_RBF_SPH ||
         (kind >= kKindSpDirect && kind < kKindSpDirect + 4);
}

template <class T>
bool Fmm<T>::supported(int kind) {
  // Compactly supported and piecewise kernels are not smooth enough for interpolation: they run
  // near-field-only trees (near_only_supported), and the spheroidal family is split into a
  // compact direct part and a smooth fast part (src/fmm/spheroidal_evaluator.hpp), as the
  // evaluator arranges.
  if (kind >= kKindSpDirect) return false;
  if (kind >= kKindSpFast) return true;
  switch (kind) {
    case PGPU_RBF_CUB:
    case PGPU_RBF_SPH:
    case PGPU_RBF_SP3:
    case PGPU_RBF_SP5:
    case PGPU_RBF_SP7:
    case PGPU_RBF_SP9:
      return false;
    default:
      return true;
  }
}

template <class T>
Fmm<T>::Fmm(int kind, const KParams<T>& kp, const Mat3& a, const double box_min[3],
            double box_width, double accuracy)
    : impl_(new Impl) {
  impl_->kind = kind;
  impl_->kp = kp;
  impl_->a = a;
  for (int k = 0; k < 3; ++k) impl_->box.min[k] = box_min[k];
  impl_->box.width = box_width;
  impl_->accuracy = accuracy;
}

template <class T>
Fmm<T>::~Fmm() {
  delete impl_;
}

template <class T>
void Fmm<T>::set_config(const FarFieldConfig& c) {
  impl_->cfg = c;
  impl_->cfg_set = true;
  impl_->built = false;
}

template <class T>
void Fmm<T>::set_points(const P4<double>* pos, Index n) {
  impl_->symmetric = true;
  impl_->spos_in = impl_->tpos_in = pos;
  impl_->ns = impl_->nt = n;
  impl_->built = false;
}

template <class T>
void Fmm<T>::set_sources(const P4<double>* pos, Index n) {
  impl_->symmetric = false;
  impl_->spos_in = pos;
  impl_->ns = n;
  impl_->built = false;
}

template <class T>
void Fmm<T>::set_targets(const P4<double>* pos, Index n) {
  impl_->symmetric = false;
  impl_->tpos_in = pos;
  impl_->nt = n;
  impl_->built = false;
}

template <class T>
void Fmm<T>::set_gradient_targets(bool on) {
  impl_->grad_out = on;
}

template <class T>
void Fmm<T>::set_near_fp64(bool on, const KParams<double>& kp64) {
  impl_->near64 = on;
  impl_->kp64 = kp64;
}

template <class T>
void Fmm<T>::evaluate(const T* vw, const T* gg, const double* w64, double* out_v, double*) {
  impl_->evaluate(vw, gg, w64, out_v);
}

template <class T>
void Fmm<T>::set_gradient_sources(bool on) {
  impl_->dipole = on;
}

template <class T>
Index Fmm<T>::near_pairs() const {
  return impl_->near_pairs;
}

template class Fmm<double>;
template class Fmm<float>;

}  // namespace pgpu
