// Tiled O(N*M) direct sums on the device: the GPU form of src/fmm/full_direct.hpp:7-52 and
// of interpolation/direct_evaluator.hpp:38-88 (value and gradient sources, value and
// gradient targets). Sources are staged in shared memory one tile at a time; each thread owns
// one target. Large source sets are split across blockIdx.y into partial sums that are reduced
// in a fixed order, so results are deterministic.
#include "common.hpp"
#include "direct.hpp"
#include "kernels.cuh"
#include "profile.hpp"

namespace pgpu {

namespace {

constexpr int kThreads = 128;
constexpr int kTile = 128;

template <class T, int KIND, bool TGRAD>
__global__ void __launch_bounds__(kThreads)
    direct_kernel(KParams<T> kp, Mat3 a, const P4<T>* __restrict__ vpos,
                  const T* __restrict__ vw, Index nv, const P4<T>* __restrict__ gpos,
                  const T* __restrict__ gg, Index ng, const P4<T>* __restrict__ tpos, Index nt,
                  double* __restrict__ out, double* __restrict__ part, Index chunk) {
  __shared__ P4<T> s_pos[kTile];
  __shared__ T s_g[3 * kTile];

  const Index i = static_cast<Index>(blockIdx.x) * kThreads + threadIdx.x;
  const bool active = i < nt;
  P4<T> t = active ? tpos[i] : P4<T>{T(0), T(0), T(0), T(0)};

  // Accumulators: per-tile partials in T, running totals in double.
  double tot0 = 0, tot1 = 0, tot2 = 0;

  const Index vbeg = static_cast<Index>(blockIdx.y) * chunk;
  const Index vend = min(nv, vbeg + chunk);
  for (Index base = vbeg; base < vend; base += kTile) {
    const int cnt = static_cast<int>(min(static_cast<Index>(kTile), vend - base));
    __syncthreads();
    if (threadIdx.x < cnt) {
      P4<T> p = vpos[base + threadIdx.x];
      p.w = vw[base + threadIdx.x];
      s_pos[threadIdx.x] = p;
    }
    __syncthreads();
    if (active) {
      if constexpr (!TGRAD) {
        T acc = T(0);
#pragma unroll 4
        for (int j = 0; j < cnt; ++j) {
          P4<T> s = s_pos[j];
          acc_value_from_value<KIND>(t.x - s.x, t.y - s.y, t.z - s.z, s.w, kp, acc);
        }
        tot0 += static_cast<double>(acc);
      } else {
        T ax = T(0), ay = T(0), az = T(0);
#pragma unroll 4
        for (int j = 0; j < cnt; ++j) {
          P4<T> s = s_pos[j];
          acc_grad_from_value<KIND>(t.x - s.x, t.y - s.y, t.z - s.z, s.w, kp, ax, ay, az);
        }
        tot0 += static_cast<double>(ax);
        tot1 += static_cast<double>(ay);
        tot2 += static_cast<double>(az);
      }
    }
  }

  const Index gbeg = static_cast<Index>(blockIdx.y) * chunk;
  const Index gend = min(ng, gbeg + chunk);
  for (Index base = gbeg; base < gend; base += kTile) {
    const int cnt = static_cast<int>(min(static_cast<Index>(kTile), gend - base));
    __syncthreads();
    if (threadIdx.x < cnt) {
      s_pos[threadIdx.x] = gpos[base + threadIdx.x];
      s_g[3 * threadIdx.x + 0] = gg[3 * (base + threadIdx.x) + 0];
      s_g[3 * threadIdx.x + 1] = gg[3 * (base + threadIdx.x) + 1];
      s_g[3 * threadIdx.x + 2] = gg[3 * (base + threadIdx.x) + 2];
    }
    __syncthreads();
    if (active) {
      if constexpr (!TGRAD) {
        T acc = T(0);
        for (int j = 0; j < cnt; ++j) {
          P4<T> s = s_pos[j];
          acc_value_from_grad<KIND>(t.x - s.x, t.y - s.y, t.z - s.z, s_g[3 * j], s_g[3 * j + 1],
                                    s_g[3 * j + 2], kp, acc);
        }
        tot0 += static_cast<double>(acc);
      } else {
        T ax = T(0), ay = T(0), az = T(0);
        for (int j = 0; j < cnt; ++j) {
          P4<T> s = s_pos[j];
          acc_grad_from_grad<KIND>(t.x - s.x, t.y - s.y, t.z - s.z, s_g[3 * j], s_g[3 * j + 1],
                                   s_g[3 * j + 2], kp, ax, ay, az);
        }
        tot0 += static_cast<double>(ax);
        tot1 += static_cast<double>(ay);
        tot2 += static_cast<double>(az);
      }
    }
  }

  if (!active) return;
  if constexpr (!TGRAD) {
    if (part) {
      part[static_cast<Index>(blockIdx.y) * nt + i] = tot0;
    } else {
      out[i] += tot0;
    }
  } else {
    double ox, oy, oz;
    mat3_tvec(a.a, tot0, tot1, tot2, ox, oy, oz);
    if (part) {
      double* p = part + static_cast<Index>(blockIdx.y) * nt * 3;
      p[3 * i] = ox;
      p[3 * i + 1] = oy;
      p[3 * i + 2] = oz;
    } else {
      out[3 * i] += ox;
      out[3 * i + 1] += oy;
      out[3 * i + 2] += oz;
    }
  }
}

__global__ void reduce_parts_kernel(const double* __restrict__ part, int nparts, Index n,
                                    double* __restrict__ out) {
  Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0;
  for (int c = 0; c < nparts; ++c) s += part[static_cast<Index>(c) * n + i];
  out[i] += s;
}

template <class T, bool TGRAD>
void launch_direct(int kind, const KParams<T>& kp, const Mat3& a, const DirectSources<T>& src,
                   const P4<T>* tpos, Index nt, double* out, cudaStream_t st) {
  if (nt == 0 || (src.nv == 0 && src.ng == 0)) return;
  const int bx = blocks_for(nt, kThreads);
  // Split the sources so that the grid covers the machine about four times.
  const Index nsrc = src.nv > src.ng ? src.nv : src.ng;
  const int want = 4 * num_sms();
  int chunks = 1;
  if (bx < want) {
    chunks = (want + bx - 1) / bx;
    Index max_chunks = (nsrc + 4 * kTile - 1) / (4 * kTile);
    if (chunks > max_chunks) chunks = static_cast<int>(max_chunks < 1 ? 1 : max_chunks);
    if (chunks > 65535) chunks = 65535;
  }
  Index chunk = (nsrc + chunks - 1) / chunks;
  chunk = ((chunk + kTile - 1) / kTile) * kTile;
  if (chunk == 0) chunk = kTile;
  chunks = static_cast<int>((nsrc + chunk - 1) / chunk);
  if (chunks < 1) chunks = 1;

  const int comps = TGRAD ? 3 : 1;
  ProfScope ps(sizeof(T) == 4 ? "direct_f32" : "direct_f64",
               pair_flops(kind) * static_cast<double>(nt) * static_cast<double>(src.nv + src.ng));
  DevBuf<double> part;
  if (chunks > 1) part.resize(static_cast<size_t>(chunks) * nt * comps);
  dim3 grid(bx, chunks);
  dispatch_kind(kind, [&]<int K>() {
    direct_kernel<T, K, TGRAD><<<grid, kThreads, 0, st>>>(
        kp, a, src.vpos, src.vw, src.nv, src.gpos, src.gg, src.ng, tpos, nt, out,
        chunks > 1 ? part.data() : nullptr, chunk);
    return 0;
  });
  PGPU_LAUNCH_CHECK();
  if (chunks > 1) {
    Index n = nt * comps;
    reduce_parts_kernel<<<blocks_for(n, 256), 256, 0, st>>>(part.data(), chunks, n, out);
    PGPU_LAUNCH_CHECK();
  }
}

// Value sources to value targets for the odd polyharmonic kernels in float-float arithmetic
// (about 44 significant bits on the FP32 pipes): FP64-class sums at a fraction of the FP64
// cost. Positions are the FP64 frame coordinates; same tiling and source split as above.
template <int KIND>
__global__ void __launch_bounds__(kThreads)
    direct_ff_kernel(KParams<double> kp, const P4<double>* __restrict__ vpos,
                     const double* __restrict__ vw, Index nv, const P4<double>* __restrict__ tpos,
                     Index nt, double* __restrict__ out, double* __restrict__ part, Index chunk) {
  __shared__ float s_p[8][kTile];
  const Index i = static_cast<Index>(blockIdx.x) * kThreads + threadIdx.x;
  const bool active = i < nt;
  const P4<double> t = active ? tpos[i] : P4<double>{0.0, 0.0, 0.0, 0.0};
  float txh, txl, tyh, tyl, tzh, tzl;
  ff_split(t.x, txh, txl);
  ff_split(t.y, tyh, tyl);
  ff_split(t.z, tzh, tzl);
  float c_hi, c_lo;
  ff_split(kp.p1 * kp.p1, c_hi, c_lo);
  const bool reg = kp.p1 != 0.0;
  const Index s0 = static_cast<Index>(blockIdx.y) * chunk;
  const Index s1 = min(nv, s0 + chunk);
  double tot = 0.0;
  for (Index base = s0; base < s1; base += kTile) {
    const int cnt = static_cast<int>(min(static_cast<Index>(kTile), s1 - base));
    __syncthreads();
    if (threadIdx.x < cnt) {
      const P4<double> p = vpos[base + threadIdx.x];
      ff_split(p.x, s_p[0][threadIdx.x], s_p[1][threadIdx.x]);
      ff_split(p.y, s_p[2][threadIdx.x], s_p[3][threadIdx.x]);
      ff_split(p.z, s_p[4][threadIdx.x], s_p[5][threadIdx.x]);
      ff_split(vw[base + threadIdx.x], s_p[6][threadIdx.x], s_p[7][threadIdx.x]);
    }
    __syncthreads();
    float ah = 0.0f, al = 0.0f;
#pragma unroll 2
    for (int j = 0; j < cnt; ++j)
      ff_poly_accumulate<KIND>(txh, txl, tyh, tyl, tzh, tzl, s_p[0][j], s_p[1][j], s_p[2][j],
                               s_p[3][j], s_p[4][j], s_p[5][j], s_p[6][j], s_p[7][j], reg, c_hi,
                               c_lo, ah, al);
    tot += static_cast<double>(ah) + static_cast<double>(al);
  }
  if (!active) return;
  const double v = (KIND == PGPU_RBF_BH3 ? -kp.p0 : kp.p0) * tot;
  if (part) part[static_cast<Index>(blockIdx.y) * nt + i] = v;
  else out[i] += v;
}

}  // namespace

bool direct_evaluate_ff(int kind, const KParams<double>& kp, const P4<double>* spos,
                        const double* w, Index ns, const P4<double>* tpos, Index nt, double* out,
                        cudaStream_t st) {
  if (kind != PGPU_RBF_BH3 && kind != PGPU_RBF_TH3) return false;
  if (nt == 0 || ns == 0) return true;
  const int bx = blocks_for(nt, kThreads);
  const int want = 4 * num_sms();
  int chunks = 1;
  if (bx < want) {
    chunks = (want + bx - 1) / bx;
    const Index max_chunks = (ns + 4 * kTile - 1) / (4 * kTile);
    if (chunks > max_chunks) chunks = static_cast<int>(max_chunks < 1 ? 1 : max_chunks);
    if (chunks > 65535) chunks = 65535;
  }
  Index chunk = (ns + chunks - 1) / chunks;
  chunk = ((chunk + kTile - 1) / kTile) * kTile;
  chunks = static_cast<int>((ns + chunk - 1) / chunk);
  ProfScope ps("direct_ff", pair_flops(kind) * static_cast<double>(nt) * static_cast<double>(ns));
  DevBuf<double> part;
  if (chunks > 1) part.resize(static_cast<size_t>(chunks) * nt);
  dim3 grid(bx, chunks);
  if (kind == PGPU_RBF_BH3)
    direct_ff_kernel<PGPU_RBF_BH3><<<grid, kThreads, 0, st>>>(kp, spos, w, ns, tpos, nt, out,
                                                              chunks > 1 ? part.data() : nullptr, chunk);
  else
    direct_ff_kernel<PGPU_RBF_TH3><<<grid, kThreads, 0, st>>>(kp, spos, w, ns, tpos, nt, out,
                                                              chunks > 1 ? part.data() : nullptr, chunk);
  PGPU_LAUNCH_CHECK();
  if (chunks > 1) {
    reduce_parts_kernel<<<blocks_for(nt, 256), 256, 0, st>>>(part.data(), chunks, nt, out);
    PGPU_LAUNCH_CHECK();
  }
  return true;
}

template <class T>
void direct_evaluate(int kind, const KParams<T>& kp, const Mat3& a, const DirectSources<T>& src,
                     const DirectTargets<T>& trg, cudaStream_t st) {
  launch_direct<T, false>(kind, kp, a, src, trg.vpos, trg.nv, trg.out_v, st);
  launch_direct<T, true>(kind, kp, a, src, trg.gpos, trg.ng, trg.out_g, st);
}

template void direct_evaluate<double>(int, const KParams<double>&, const Mat3&,
                                      const DirectSources<double>&, const DirectTargets<double>&,
                                      cudaStream_t);
template void direct_evaluate<float>(int, const KParams<float>&, const Mat3&,
                                     const DirectSources<float>&, const DirectTargets<float>&,
                                     cudaStream_t);

}  // namespace pgpu
