// pgpu_direct_evaluate_noalloc: a variant of the direct-sum evaluation that allocates no memory.
//
// The regular direct path (direct.cu) stages transformed positions in temporary device buffers
// and, when the targets are few, splits the sources over several blocks whose partial sums go
// to a scratch buffer obtained from the library's memory pool. Callers that cannot let the
// library allocate — a host application whose device memory is owned and budgeted by its own
// allocator, or a caller that has already reserved every byte it is allowed to use — need an
// entry point that touches only the memory they pass in. This variant reads the caller's raw
// point and weight arrays directly and keeps its partial sums in a fixed, file-scope device
// array instead.
//
// Scratch: kNoAllocScratch doubles (16 MiB) in a static __device__ array. Every GPU that loads
// the library holds it until the process exits. The number of targets per call is limited to
// kNoAllocScratch (one partial per target is always needed); larger calls are rejected.
// All calls share the array and each call overwrites it, so calls whose kernels may overlap on
// the GPU (different streams, or different host threads on one device) race: callers must
// serialise them. The device address of the array is looked up once per device on the first
// call made with that device current (make that first call before any stream capture) and kept
// for the life of the process: after cudaDeviceReset, or any teardown of the device's primary
// context, the kept address is stale and the entry point must not be called again.
// The entry point works on the caller's current device (cudaGetDevice), not on the device that
// pgpu_set_device selected for the library's other calls, and every pointer must be device memory
// of that device (or managed memory).
#include <mutex>

#include "common.hpp"
#include "kernels.cuh"

namespace pgpu {

constexpr Index kNoAllocScratch = Index{1} << 21;  // doubles: 16 MiB

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratch];

namespace {

constexpr int kThreads = 128;
constexpr int kTile = 128;
constexpr int kMaxDevices = 64;

std::mutex g_setup_mu;
double* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array for the current device (looked up once per device).
double* scratch_for_current_device(int* err) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    *err = 1;
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (g_scratch_ptr[dev] == nullptr) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) {
      *err = 2;
      return nullptr;
    }
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  return g_scratch_ptr[dev];
}

// Same arithmetic as direct_kernel<double, KIND, false>: each block sums one source chunk for
// kThreads targets; positions are transformed by A on the fly, in FP64.
template <int KIND>
__global__ void __launch_bounds__(kThreads)
    noalloc_direct_kernel(KParams<double> kp, Mat3 a, const double* __restrict__ src, Index ns,
                          const double* __restrict__ w, const double* __restrict__ trg, Index nt,
                          Index chunk, double* __restrict__ part) {
  __shared__ P4<double> s_pos[kTile];
  const Index i = static_cast<Index>(blockIdx.x) * kThreads + threadIdx.x;
  const bool active = i < nt;
  double tx = 0, ty = 0, tz = 0;
  if (active) mat3_vec(a.a, trg[3 * i], trg[3 * i + 1], trg[3 * i + 2], tx, ty, tz);
  double tot = 0;
  const Index beg = static_cast<Index>(blockIdx.y) * chunk;
  const Index end = min(ns, beg + chunk);
  for (Index base = beg; base < end; base += kTile) {
    const int cnt = static_cast<int>(min(static_cast<Index>(kTile), end - base));
    __syncthreads();
    if (threadIdx.x < cnt) {
      const Index j = base + threadIdx.x;
      double x, y, z;
      mat3_vec(a.a, src[3 * j], src[3 * j + 1], src[3 * j + 2], x, y, z);
      s_pos[threadIdx.x] = P4<double>{x, y, z, w[j]};
    }
    __syncthreads();
    if (active) {
      double acc = 0;
      for (int j = 0; j < cnt; ++j) {
        const P4<double> s = s_pos[j];
        acc_value_from_value<KIND>(tx - s.x, ty - s.y, tz - s.z, s.w, kp, acc);
      }
      tot += acc;
    }
  }
  if (active) part[static_cast<Index>(blockIdx.y) * nt + i] = tot;
}

__global__ void noalloc_reduce_kernel(const double* __restrict__ part, int nparts, Index n,
                                      double* __restrict__ out) {
  const Index i = static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0;
  for (int c = 0; c < nparts; ++c) s += part[static_cast<Index>(c) * n + i];
  out[i] = s;
}

// Device memory of device `dev`, or managed memory.
bool device_ptr(const void* p, int dev) {
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (attr.type == cudaMemoryTypeManaged) return true;
  return attr.type == cudaMemoryTypeDevice && attr.device == dev;
}

}  // namespace

// Returns 0 on success or a PGPU_* status; msg receives a static description on failure.
int direct_evaluate_noalloc(const pgpu_rbf* rbf, const double* src, int64_t ns,
                            const double* weights, const double* trg, int64_t nt, double* out,
                            cudaStream_t st, const char** msg) {
  if (rbf == nullptr || rbf->kind < 0 || rbf->kind >= PGPU_RBF_COUNT) {
    *msg = "rbf must be a valid kernel description";
    return PGPU_INVALID_ARGUMENT;
  }
  if (ns < 0 || nt < 0) {
    *msg = "point counts must be non-negative";
    return PGPU_INVALID_ARGUMENT;
  }
  if (nt > kNoAllocScratch) {
    *msg = "too many targets for the allocation-free entry point (limit 2097152 per call)";
    return PGPU_INVALID_ARGUMENT;
  }
  if (nt == 0) return PGPU_OK;
  if (out == nullptr || trg == nullptr || (ns > 0 && (src == nullptr || weights == nullptr))) {
    *msg = "points, weights and out must not be null";
    return PGPU_INVALID_ARGUMENT;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    *msg = "cudaGetDevice failed";
    return PGPU_CUDA_ERROR;
  }
  if (!device_ptr(out, dev) || !device_ptr(trg, dev) ||
      (ns > 0 && (!device_ptr(src, dev) || !device_ptr(weights, dev)))) {
    *msg = "the allocation-free entry point takes device pointers of the current device only";
    return PGPU_INVALID_ARGUMENT;
  }
  int err = 0;
  double* scratch = scratch_for_current_device(&err);
  if (scratch == nullptr) {
    *msg = "cudaGetSymbolAddress failed for the scratch array";
    return PGPU_CUDA_ERROR;
  }
  // Source chunks: as many as the scratch holds (and the GPU needs), at most 1024.
  const int bx = blocks_for(nt, kThreads);
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    *msg = "cudaDeviceGetAttribute failed";
    return PGPU_CUDA_ERROR;
  }
  Index chunks = 1;
  if (bx < 4 * sms && ns > 0) chunks = (4 * sms + bx - 1) / bx;
  chunks = std::min<Index>(chunks, std::max<Index>(1, kNoAllocScratch / nt));
  chunks = std::min<Index>(chunks, std::max<Index>(1, (ns + 4 * kTile - 1) / (4 * kTile)));
  chunks = std::min<Index>(chunks, 1024);
  Index chunk = (ns + chunks - 1) / chunks;
  chunk = std::max<Index>(kTile, ((chunk + kTile - 1) / kTile) * kTile);
  chunks = std::max<Index>(1, (ns + chunk - 1) / chunk);
  Mat3 a;
  for (int k = 0; k < 9; ++k) a.a[k] = rbf->aniso[k];
  KParams<double> kp{rbf->params[0], rbf->params[1]};
  dim3 grid(bx, static_cast<unsigned>(chunks));
  dispatch_kind(rbf->kind, [&]<int K>() {
    noalloc_direct_kernel<K><<<grid, kThreads, 0, st>>>(kp, a, src, ns, weights, trg, nt, chunk,
                                                          scratch);
    return 0;
  });
  noalloc_reduce_kernel<<<blocks_for(nt, 256), 256, 0, st>>>(scratch, static_cast<int>(chunks), nt,
                                                            out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    *msg = "kernel launch failed in the allocation-free entry point";
    return PGPU_CUDA_ERROR;
  }
  return PGPU_OK;
}

}  // namespace pgpu
