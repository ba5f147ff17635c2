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

}  // namespace

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
