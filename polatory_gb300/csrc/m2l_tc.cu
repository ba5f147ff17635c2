// Tensor-core M2L for the FP32 far field at order 6 (p^3 = 216 interpolation nodes per cell).
//
// One CTA owns 128 target cells of a level (one M = 128 tile). For every offset o present
// among its cells and every 16-node chunk of the source nodes it forms
//   D_o[cell][a] = sum_b M_{s(cell, o)}[b] * K_o[a][b]
// with tcgen05.mma (kind::tf32, M = 128, N = 224, K = 8) into one of two TMEM accumulators
// (offsets alternate between them). While the tensor core fills one, the CTA adds the other,
// complete, offset into per-thread FP32 running sums (round-to-nearest): the tensor core's own
// accumulation then spans 81 products only, which keeps its rounding from building up over the
// ~300 offsets of a cell. Nothing leaves the SM but the final sums; the result is
// deterministic. FP32 accuracy comes from splitting both operands into a TF32 head and tail:
//   A B ~ A_hi B_hi + A_hi B_lo + A_lo B_hi   (relative error about 2^-22 per product).
// The operator chunks (head and tail, 224 x 16 each, already in the canonical no-swizzle
// K-major core-matrix layout) arrive by bulk TMA copies completing on an mbarrier; the gathered
// multipole rows arrive by cp.async, and their head/tail split is computed in shared memory.
// Five pipeline stages, filled and drained by separate warp roles (below).
//
// Layout of one operand chunk in shared memory (no swizzle, K-major): core matrices of 8 rows x
// 16 bytes (4 TF32 values) stored contiguously (128 B); the 4 core matrices of one 8-row group
// along K are adjacent (leading-dimension byte offset 128 B) and consecutive 8-row groups are
// 512 B apart (stride-dimension byte offset).
//
// Every wait on an mbarrier is bounded; a wait that runs out sets *err, the CTA waits for its
// copies and MMAs in flight, frees its TMEM and returns.
#include <algorithm>
#include <cstdint>
#include <mutex>

#include "common.hpp"
#include "m2l_tc.hpp"
#include "tcgen05.cuh"
#include "profile.hpp"

namespace pgpu {

namespace {

constexpr int kD = 216;           // p^3 at order 6
constexpr int kN = 224;           // MMA N (target nodes, padded)
constexpr int kChunk = 16;        // source nodes per pipeline step
constexpr int kChunks = 14;       // ceil(216 / 16)
constexpr int kCells = 128;       // target cells per CTA (one M = 128 tile)
constexpr int kStages = 5;
constexpr int kLookahead = 2;  // gather steps in flight ahead of the split
constexpr int kNOffsets = 343;
constexpr int kAFloats = kCells * kChunk;  // 2048
constexpr int kBFloats = kN * kChunk;      // 3584
constexpr int kStageFloats = 2 * kAFloats + 2 * kBFloats;
constexpr uint32_t kBBytes = kBFloats * 4;  // 14336
constexpr int kTmemCols = 512;
constexpr int kBars = 3 * kStages + 5;  // operator bytes, gathers, stage releases, accumulators full/free, final

// Shared-memory layout (bytes from a 1024-aligned base).
constexpr int kSmemStages = kStages * kStageFloats * 4;        // 225,280
constexpr int kSmemBars = kSmemStages;
constexpr int kSmemMisc = kSmemBars + 8 * kBars;               // tmem address, flags
constexpr int kSmemList = kSmemMisc + 32;                      // offset list (343 ints)
constexpr int kSmemMask = kSmemList + 4 * kNOffsets;           // offset bitmask (11 words)
constexpr int kSmemTotal = kSmemMask + 4 * 12;
constexpr int kSmemLaunch = kSmemTotal + 1024;                 // room to align the base

using namespace tc;

constexpr uint32_t kIdesc = idesc_tf32(128, kN);  // M = 128, N = 224

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t acc) {
  tc::mma_tf32(tmem_d, a, b, kIdesc, acc);
}

// Warp roles (384 threads, 12 warps: three per SM sub-partition, which leaves each thread up to
// 168 registers):
//   warps 0-1   gather: thread t owns target cells t and t + 64 of the tile; for each pipeline
//               step it loads their 16 multipole values of the offset's source cells
//               (cp.async), splits them into TF32 head and tail in the MMA layout and arrives on
//               the stage's producer barrier (kLookahead steps in flight inside the thread; the
//               source cells of the next offset are looked up one offset ahead);
//   warps 2-9   drain: warp w reads TMEM lanes 32 (w % 4) .. + 31 (its cells; a warp reaches
//               the lanes of its position in its warpgroup) and columns 112 ((w - 2) / 4) .. +
//               111 of a finished accumulator into FP32 running sums, then frees the accumulator;
//   warp 10     MMA issue (one thread) and TMEM allocation;
//   warp 11     operator copies (one thread): bulk copies of the head and tail chunks.
// Hand-offs are mbarriers only: stage s is full when its operator bytes have landed (tma_bar)
// and the 64 gather threads have arrived (prod_bar); the MMAs of a stage release it through
// tcgen05.commit (free_bar); an accumulator is full after the last chunk of its offset
// (acc_bar) and empty again once the 256 drain threads have read it (acc_free_bar).
// Every wait is bounded and gives up early when another role has aborted.
constexpr int kThreads = 384;
constexpr int kGatherWarps = 2, kDrainWarp0 = 2, kMmaWarp = 10, kTmaWarp = 11;
constexpr int kGatherThreads = kGatherWarps * 32;  // 64: two rows each

__global__ void __launch_bounds__(kThreads, 1)
    m2l_tc_kernel(const float* __restrict__ kb_hi, const float* __restrict__ kb_lo,
                  const int* __restrict__ table, Index nt, const float* __restrict__ Ms,
                  float* __restrict__ L, float* __restrict__ part, int* __restrict__ err,
                  int stall_polls) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  float* stage_f = reinterpret_cast<float*>(smem);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kSmemBars);
  // misc: [0] TMEM address, [1] abort flag, [2] offsets present, [3] last step whose operator
  // bytes the MMA thread saw land, [4] last step whose operator copies were issued.
  uint32_t* misc = reinterpret_cast<uint32_t*>(smem + kSmemMisc);
  int* olist = reinterpret_cast<int*>(smem + kSmemList);
  uint32_t* omask = reinterpret_cast<uint32_t*>(smem + kSmemMask);
  auto tma_bar = [&](int s) { return smem_u32(&bars[s]); };
  auto prod_bar = [&](int s) { return smem_u32(&bars[kStages + s]); };
  auto free_bar = [&](int s) { return smem_u32(&bars[2 * kStages + s]); };
  auto acc_bar = [&](int b) { return smem_u32(&bars[3 * kStages + b]); };
  auto acc_free_bar = [&](int b) { return smem_u32(&bars[3 * kStages + 2 + b]); };
  const uint32_t final_bar = smem_u32(&bars[3 * kStages + 4]);
  volatile uint32_t* abort_flag = &misc[1];

  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int lane = tid & 31;
  // Fault injection (host knob): the first CTA leaves the operator copy of its first stage
  // unissued and gives up on its waits after stall_polls polls.
  const bool stall = stall_polls > 0 && blockIdx.x == 0 && blockIdx.y == 0;
  const int limit = stall ? stall_polls : kWaitPolls;
  const Index t0 = static_cast<Index>(blockIdx.x) * kCells;
  // Waits that give up when another role has aborted.
  auto wait = [&](uint32_t bar, uint32_t parity) {
    for (int it = 0; it < limit; ++it) {
      if (mbar_try(bar, parity)) return true;
      if (*abort_flag != 0) return false;
      if (it >= 1024) __nanosleep(128);
    }
    atomicExch(const_cast<uint32_t*>(abort_flag), 1u);
    return false;
  };

  // Offsets present among the CTA's cells.
  if (tid < 12) omask[tid] = 0;
  __syncthreads();
  if (tid < kCells && t0 + tid < nt) {
    const int* row = table + (t0 + tid) * kNOffsets;
    for (int o = 0; o < kNOffsets; ++o)
      if (row[o] >= 0) atomicOr(&omask[o >> 5], 1u << (o & 31));
  }
  __syncthreads();
  if (tid == 0) {
    int n = 0;
    for (int o = 0; o < kNOffsets; ++o)
      if (omask[o >> 5] & (1u << (o & 31))) olist[n++] = o;
    misc[2] = static_cast<uint32_t>(n);
    misc[1] = 0;
    misc[3] = 0xFFFFFFFFu;
    misc[4] = 0xFFFFFFFFu;
    for (int s = 0; s < kStages; ++s) {
      mbar_init(tma_bar(s), 1);
      mbar_init(prod_bar(s), kGatherThreads);
      mbar_init(free_bar(s), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(acc_bar(b), 1);
      mbar_init(acc_free_bar(b), (kMmaWarp - kDrainWarp0) * 32);
    }
    mbar_init(final_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  // Group blockIdx.y of gridDim.y takes a contiguous share of the offsets; with several groups
  // each writes its partial sums to part (summed afterwards in group order).
  const int n_all = static_cast<int>(misc[2]);
  const int groups = static_cast<int>(gridDim.y);
  const int q_beg = static_cast<int>((static_cast<long>(blockIdx.y) * n_all) / groups);
  const int q_end = static_cast<int>((static_cast<long>(blockIdx.y + 1) * n_all) / groups);
  const int n_off = q_end - q_beg;
  float* out_base = groups == 1 ? L : part + static_cast<Index>(blockIdx.y) * nt * kD;
  // Drain role geometry.
  const bool is_drain = warp >= kDrainWarp0 && warp < kMmaWarp;
  const int dw = warp - kDrainWarp0;
  const int lane_base = 32 * (warp & 3);
  const int col_base = 112 * (dw >> 2);
  const Index d_cell = t0 + lane_base + lane;
  if (n_off == 0) {
    if (groups > 1 && is_drain && d_cell < nt) {
      float* dst = out_base + d_cell * kD + col_base;
      for (int j = 0; j < 112 && col_base + j < kD; ++j) dst[j] = 0.0f;
    }
    return;
  }

  // TMEM: two accumulators of 224 columns (columns 0 and 256), one per offset in turn.
  if (warp == kMmaWarp) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&misc[0])),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = misc[0];

  const int n_iter = n_off * kChunks;
  auto a_hi = [&](int s) { return stage_f + s * kStageFloats; };
  auto a_lo = [&](int s) { return stage_f + s * kStageFloats + kAFloats; };
  auto b_hi = [&](int s) { return stage_f + s * kStageFloats + 2 * kAFloats; };
  auto b_lo = [&](int s) { return stage_f + s * kStageFloats + 2 * kAFloats + kBFloats; };

  float sum[112];
#pragma unroll
  for (int j = 0; j < 112; ++j) sum[j] = 0.0f;

  if (warp < kGatherWarps) {
    // Gather: rows tid and tid + 64 of every stage. The loads of step i are issued kLookahead
    // steps before their split. Steps past the end commit empty copy groups so that the group
    // count stays uniform.
    int src[2] = {-1, -1}, nsrc[2] = {-1, -1};
    auto lookup = [&](int q, int* out) {
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        const Index cell = t0 + tid + kGatherThreads * r;
        out[r] = cell < nt ? table[cell * kNOffsets + olist[q_beg + q]] : -1;
      }
    };
    lookup(0, nsrc);
    for (int i = 0; i < n_iter + kLookahead; ++i) {
      if (i < n_iter) {
        const int s = i % kStages;
        const int c = i % kChunks;
        if (i >= kStages && !wait(free_bar(s), ((i / kStages) - 1) & 1)) break;
        if (c == 0) {
          const int q = i / kChunks;
          src[0] = nsrc[0];
          src[1] = nsrc[1];
          if (q + 1 < n_off) lookup(q + 1, nsrc);
        }
        float* dst = a_hi(s);
#pragma unroll
        for (int r = 0; r < 2; ++r) {
          const int row = tid + kGatherThreads * r;
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int k = c * kChunk + 4 * j;
            const bool have = src[r] >= 0 && k < kD;
            const float* g = have ? Ms + static_cast<Index>(src[r]) * kD + k : Ms;
            cp_async16(smem_u32(dst + core_off(row, 4 * j)), g, have ? 16u : 0u);
          }
        }
      }
      cp_async_commit();
      if (i >= kLookahead) {
        cp_async_wait<kLookahead>();
        const int sp = (i - kLookahead) % kStages;
#pragma unroll
        for (int jj = 0; jj < 8; ++jj) {
          const int row = tid + kGatherThreads * (jj >> 2), j = jj & 3;
          const int off = core_off(row, 4 * j);
          float4* ph = reinterpret_cast<float4*>(a_hi(sp) + off);
          float4* pl = reinterpret_cast<float4*>(a_lo(sp) + off);
          const float4 x = *ph;
          const float4 h{tf32_round(x.x), tf32_round(x.y), tf32_round(x.z), tf32_round(x.w)};
          *ph = h;
          *pl = float4{x.x - h.x, x.y - h.y, x.z - h.z, x.w - h.w};
        }
        fence_proxy_async();
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(prod_bar(sp)) : "memory");
      }
      if (*abort_flag != 0) break;
    }
    cp_async_wait<0>();
  } else if (is_drain) {
    for (int q = 0; q < n_off; ++q) {
      const int b = q & 1;
      if (!wait(acc_bar(b), (q >> 1) & 1)) break;
      tc_fence_after();
      const uint32_t base = tmem + (static_cast<uint32_t>(lane_base) << 16) +
                            static_cast<uint32_t>(b * 256 + col_base);
#pragma unroll
      for (int u = 0; u < 7; ++u) {
        float v[16];
        tmem_ld16(base + static_cast<uint32_t>(16 * u), v);
#pragma unroll
        for (int j = 0; j < 16; ++j) sum[16 * u + j] += v[j];
      }
      tc_fence_before();
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(acc_free_bar(b)) : "memory");
    }
  } else if (warp == kMmaWarp) {
    if (lane == 0) {
      for (int i = 0; i < n_iter; ++i) {
        const int s = i % kStages;
        const int q = i / kChunks;
        const int c = i % kChunks;
        const uint32_t ph = (i / kStages) & 1;
        if (!wait(tma_bar(s), ph)) break;
        misc[3] = static_cast<uint32_t>(i);
        if (!wait(prod_bar(s), ph)) break;
        if (c == 0 && q >= 2 && !wait(acc_free_bar(q & 1), ((q >> 1) - 1) & 1)) break;
        tc_fence_after();
        const uint32_t d = tmem + static_cast<uint32_t>((q & 1) * 256);
        const uint32_t ah = smem_u32(a_hi(s)), al = smem_u32(a_lo(s));
        const uint32_t bh = smem_u32(b_hi(s)), bl = smem_u32(b_lo(s));
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) {
          const uint32_t ko = static_cast<uint32_t>(ks * 256);
          // The first product of an offset overwrites its accumulator.
          mma_tf32(d, make_desc(ah + ko), make_desc(bh + ko), (c == 0 && ks == 0) ? 0u : 1u);
          mma_tf32(d, make_desc(ah + ko), make_desc(bl + ko), 1u);
          mma_tf32(d, make_desc(al + ko), make_desc(bh + ko), 1u);
        }
        mma_commit(free_bar(s));
        if (c == kChunks - 1) mma_commit(acc_bar(q & 1));
      }
    }
    __syncwarp();
  } else if (warp == kTmaWarp) {
    if (lane == 0) {
      for (int i = 0; i < n_iter; ++i) {
        const int s = i % kStages;
        if (i >= kStages && !wait(free_bar(s), ((i / kStages) - 1) & 1)) break;
        if (!(stall && i == 0)) {
          const int o = olist[q_beg + i / kChunks];
          const int c = i % kChunks;
          mbar_expect_tx(tma_bar(s), 2 * kBBytes);
          const size_t blk = (static_cast<size_t>(o) * kChunks + c) * kBFloats;
          bulk_g2s(smem_u32(b_hi(s)), kb_hi + blk, kBBytes, tma_bar(s));
          bulk_g2s(smem_u32(b_lo(s)), kb_lo + blk, kBBytes, tma_bar(s));
        }
        misc[4] = static_cast<uint32_t>(i);
      }
    }
    __syncwarp();
  }
  __syncthreads();
  bool aborted = *abort_flag != 0;
  if (aborted && warp == kTmaWarp && lane == 0) {
    // Operator copies still in flight land before the CTA's shared memory is released.
    const int seen = static_cast<int>(misc[3]);
    const int issued = static_cast<int>(misc[4]);
    for (int j = seen + 1; j <= issued; ++j)
      if (!(stall && j == 0)) mbar_wait(tma_bar(j % kStages), (j / kStages) & 1, kWaitPolls);
  }
  // Every MMA still in flight completes before TMEM is freed.
  if (warp == kMmaWarp && lane == 0) mma_commit(final_bar);
  const bool drained = mbar_wait(final_bar, 0, kWaitPolls);
  __syncthreads();
  aborted = *abort_flag != 0 || !drained;
  if (tid == 0 && aborted) atomicExch(err, 1);
  if (!aborted && is_drain && d_cell < nt) {
    float* dst = out_base + d_cell * kD + col_base;
    if (groups == 1) {
#pragma unroll
      for (int j = 0; j < 112; ++j)
        if (col_base + j < kD) dst[j] += sum[j];
    } else {
#pragma unroll
      for (int j = 0; j < 112; ++j)
        if (col_base + j < kD) dst[j] = sum[j];
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == kMmaWarp) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols)
                 : "memory");
  }
}

// Operator chunks in the core-matrix layout: for offset o and chunk c, the 224 x 16 block
// B[a][b'] = K_o[a][16 c + b'] (zero outside 216 x 216), head and tail.
__global__ void m2l_tc_blocks_kernel(const float* __restrict__ K, float* __restrict__ hi,
                                     float* __restrict__ lo) {
  const Index total = static_cast<Index>(kNOffsets) * kChunks * kBFloats;
  for (Index e = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x; e < total;
       e += static_cast<Index>(gridDim.x) * blockDim.x) {
    const Index blk = e / kBFloats;
    const int o = static_cast<int>(blk / kChunks), c = static_cast<int>(blk % kChunks);
    const int w = static_cast<int>(e % kBFloats);
    // Invert core_off: w = (a / 8) * 128 + (kk / 4) * 32 + (a % 8) * 4 + kk % 4.
    const int a = (w / 128) * 8 + (w % 32) / 4;
    const int kk = ((w % 128) / 32) * 4 + (w % 4);
    const int b = c * kChunk + kk;
    const float v = (a < kD && b < kD) ? K[(static_cast<Index>(o) * kD + a) * kD + b] : 0.0f;
    const float h = tf32_round(v);
    hi[e] = h;
    lo[e] = tf32_round(v - h);
  }
}

}  // namespace

bool m2l_tc_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("PGPU_M2L_TC");
    return e == nullptr || std::atoi(e) != 0;
  }();
  return on;
}

M2LTcBlocks make_m2l_tc_blocks(const float* K) {
  M2LTcBlocks b;
  const size_t n = static_cast<size_t>(kNOffsets) * kChunks * kBFloats;
  b.hi.resize(n);
  b.lo.resize(n);
  m2l_tc_blocks_kernel<<<8 * num_sms(), 256, 0, stream()>>>(K, b.hi.data(), b.lo.data());
  PGPU_LAUNCH_CHECK();
  sync();  // the blocks are shared with other threads' streams
  return b;
}

__global__ void m2l_tc_reduce_kernel(const float* __restrict__ part, int groups, Index n,
                                     float* __restrict__ L) {
  const Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float s = 0.0f;
  for (int g = 0; g < groups; ++g) s += part[static_cast<Index>(g) * n + i];
  L[i] += s;
}

void m2l_tc_apply(const M2LTcBlocks& b, const int* table, Index nt, const float* Ms, float* L,
                  int* err, cudaStream_t st) {
  if (nt <= 0) return;
  static std::once_flag attr_flag;
  std::call_once(attr_flag, [] {
    PGPU_CUDA(cudaFuncSetAttribute(m2l_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   kSmemLaunch));
  });
  const Index tiles = (nt + kCells - 1) / kCells;
  // Small levels split each tile's offsets over several CTAs so that about two waves run.
  const int groups = static_cast<int>(
      std::min<Index>(16, std::max<Index>(1, (2 * num_sms() + tiles - 1) / tiles)));
  DevBuf<float> part;
  if (groups > 1) part.resize(static_cast<size_t>(groups) * nt * kD);
  const int stall_polls = static_cast<int>(std::min<int64_t>(take_m2l_stall(), kWaitPolls));
  m2l_tc_kernel<<<dim3(static_cast<unsigned>(tiles), groups), kThreads, kSmemLaunch, st>>>(
      b.hi.data(), b.lo.data(), table, nt, Ms, L, part.data(), err, stall_polls);
  PGPU_LAUNCH_CHECK();
  if (groups > 1) {
    const Index n = nt * kD;
    m2l_tc_reduce_kernel<<<blocks_for(n, 256), 256, 0, st>>>(part.data(), groups, n, L);
    PGPU_LAUNCH_CHECK();
  }
}

}  // namespace pgpu
