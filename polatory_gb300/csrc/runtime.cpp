// Library context: per-thread device and stream, the stream-ordered memory pool, pointer
// classification and the host<->device copy helpers.
#include <atomic>
#include <chrono>
#include <cstdlib>
#include <mutex>

#include "common.hpp"

namespace pgpu {

namespace {

struct ThreadCtx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool stream_owned = false;
  bool initialized = false;
};

thread_local ThreadCtx g_ctx;
std::once_flag g_pool_flags[64];

void configure_pool(int device) {
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    // Keep freed blocks cached in the pool instead of returning them to the driver at every
    // synchronization: fits allocate and free the same sizes every iteration.
    uint64_t threshold = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
  }
}

ThreadCtx& ctx() {
  if (!g_ctx.initialized) {
    PGPU_CUDA(cudaSetDevice(g_ctx.device));
    std::call_once(g_pool_flags[g_ctx.device & 63], configure_pool, g_ctx.device);
    PGPU_CUDA(cudaStreamCreateWithFlags(&g_ctx.stream, cudaStreamNonBlocking));
    g_ctx.stream_owned = true;
    g_ctx.initialized = true;
  }
  return g_ctx;
}

}  // namespace

cudaStream_t stream() { return ctx().stream; }

void set_stream(cudaStream_t s) {
  ctx();
  g_ctx.stream = s;
}

void set_device(int device) {
  if (g_ctx.initialized) {
    if (g_ctx.device == device) return;
    if (g_ctx.stream_owned) cudaStreamDestroy(g_ctx.stream);
    g_ctx = ThreadCtx{};
  }
  g_ctx.device = device;
  ctx();
}

namespace {
thread_local int64_t g_thread_bytes = 0;
thread_local int64_t g_thread_peak = 0;
// Host-side fault injection (pgpu_debug_inject): countdowns, 0 = off.
thread_local int64_t g_fail_alloc_in = 0;
thread_local int64_t g_m2l_stall_polls = 0;
}  // namespace

void inject_alloc_failure(int64_t after) { g_fail_alloc_in = after > 0 ? after : 0; }
void inject_m2l_stall(int64_t polls) { g_m2l_stall_polls = polls > 0 ? polls : 0; }
int64_t take_m2l_stall() {
  const int64_t p = g_m2l_stall_polls;
  g_m2l_stall_polls = 0;
  return p;
}

void* dev_alloc(size_t bytes) {
  void* p = nullptr;
  if (bytes == 0) return nullptr;
  if (g_fail_alloc_in > 0 && --g_fail_alloc_in == 0)
    throw Error(PGPU_OUT_OF_MEMORY, "out of device memory (injected allocation failure)");
  PGPU_CUDA(cudaMallocAsync(&p, bytes, stream()));
  g_thread_bytes += static_cast<int64_t>(bytes);
  if (g_thread_bytes > g_thread_peak) g_thread_peak = g_thread_bytes;
  return p;
}

// Never throws: it runs in destructors, including those of process-wide caches at exit, on
// threads that may never have used the library (their context is not created for a free).
void dev_free(void* p, size_t bytes) {
  if (!p) return;
  g_thread_bytes -= static_cast<int64_t>(bytes);
  cudaStream_t s = g_ctx.initialized ? g_ctx.stream : nullptr;
  if (cudaFreeAsync(p, s) != cudaSuccess) cudaGetLastError();
}

void sync_quiet() noexcept {
  if (g_ctx.initialized) cudaStreamSynchronize(g_ctx.stream);
}

int64_t thread_device_bytes() { return g_thread_bytes; }
int64_t thread_device_peak() { return g_thread_peak; }
void reset_thread_device_peak() { g_thread_peak = g_thread_bytes; }

void release_cached_memory() {
  cudaMemPool_t pool;
  PGPU_CUDA(cudaStreamSynchronize(stream()));
  PGPU_CUDA(cudaDeviceGetDefaultMemPool(&pool, g_ctx.device));
  PGPU_CUDA(cudaMemPoolTrimTo(pool, 0));
}

bool is_device_pointer(const void* p) {
  if (p == nullptr) return false;
  cudaPointerAttributes attr;
  cudaError_t e = cudaPointerGetAttributes(&attr, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

void copy_in(DevBuf<double>& dst, const double* src, size_t n) {
  dst.resize(n);
  if (n == 0) return;
  auto kind = is_device_pointer(src) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  PGPU_CUDA(cudaMemcpyAsync(dst.data(), src, n * sizeof(double), kind, stream()));
  if (kind == cudaMemcpyHostToDevice) {
    // The caller may free or reuse its host buffer as soon as we return.
    PGPU_CUDA(cudaStreamSynchronize(stream()));
  }
}

void copy_out(double* dst, const double* src_dev, size_t n) {
  if (n == 0) return;
  auto kind = is_device_pointer(dst) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  PGPU_CUDA(cudaMemcpyAsync(dst, src_dev, n * sizeof(double), kind, stream()));
  PGPU_CUDA(cudaStreamSynchronize(stream()));
}

int num_sms() {
  static thread_local int sms = -1;
  if (sms < 0) {
    int dev = 0;
    PGPU_CUDA(cudaGetDevice(&dev));
    PGPU_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  }
  return sms;
}

bool verbose() {
  static const bool v = std::getenv("PGPU_VERBOSE") != nullptr;
  return v;
}

namespace {
std::atomic<int64_t> g_launches{0};
}

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
int64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }

double wall_seconds() {
  using clock = std::chrono::steady_clock;
  return std::chrono::duration<double>(clock::now().time_since_epoch()).count();
}

}  // namespace pgpu
