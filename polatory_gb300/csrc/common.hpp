// Internal infrastructure of libpolatory_gpu: error type, CUDA checks, device buffers and the
// per-thread library context (device, stream). Host-only header (also included by .cu files).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "polatory_gpu.h"

namespace pgpu {

using Index = int64_t;

// Internal exception; converted to a status code at the C ABI.
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& msg) : std::runtime_error(msg), code(c) {}
};

[[noreturn]] inline void throw_invalid(const std::string& msg) {
  throw Error(PGPU_INVALID_ARGUMENT, msg);
}
[[noreturn]] inline void throw_runtime(const std::string& msg) {
  throw Error(PGPU_RUNTIME_ERROR, msg);
}

#define PGPU_CUDA(expr)                                                                    \
  do {                                                                                     \
    cudaError_t e_ = (expr);                                                               \
    if (e_ != cudaSuccess) {                                                               \
      throw ::pgpu::Error(e_ == cudaErrorMemoryAllocation ? PGPU_OUT_OF_MEMORY             \
                                                          : PGPU_CUDA_ERROR,               \
                          std::string(#expr) + ": " + cudaGetErrorString(e_) + " at " +    \
                              __FILE__ + ":" + std::to_string(__LINE__));                  \
    }                                                                                      \
  } while (0)

#define PGPU_LAUNCH_CHECK()      \
  do {                           \
    ::pgpu::count_launch();      \
    PGPU_CUDA(cudaGetLastError()); \
  } while (0)

// Library stream (one per host thread; the reference's evaluators are single-thread-affine).
cudaStream_t stream();
void set_stream(cudaStream_t s);

// Host-side fault injection of this thread (pgpu_debug_inject): the after-th next dev_alloc
// throws PGPU_OUT_OF_MEMORY; the next tensor-core M2L launch stalls one stage and polls its wait
// at most `polls` times (take_m2l_stall returns and clears the count).
void inject_alloc_failure(int64_t after);
void inject_m2l_stall(int64_t polls);
int64_t take_m2l_stall();
// Device memory from the stream-ordered pool of the current device.
void* dev_alloc(size_t bytes);
void dev_free(void* p, size_t bytes);
// Device bytes this thread holds through DevBuf now, and the peak since the last reset.
int64_t thread_device_bytes();
int64_t thread_device_peak();
void reset_thread_device_peak();

template <class T>
class DevBuf {
 public:
  DevBuf() = default;
  explicit DevBuf(size_t n) { resize(n); }
  ~DevBuf() { release(); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p_(o.p_), n_(o.n_) {
    o.p_ = nullptr;
    o.n_ = 0;
  }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      p_ = o.p_;
      n_ = o.n_;
      o.p_ = nullptr;
      o.n_ = 0;
    }
    return *this;
  }
  void resize(size_t n) {
    if (n == n_) return;
    release();
    if (n > 0) p_ = static_cast<T*>(dev_alloc(n * sizeof(T)));
    n_ = n;
  }
  void release() {
    if (p_) dev_free(p_, n_ * sizeof(T));
    p_ = nullptr;
    n_ = 0;
  }
  void zero() {
    if (n_) PGPU_CUDA(cudaMemsetAsync(p_, 0, n_ * sizeof(T), stream()));
  }
  void upload(const T* h, size_t n) {
    resize(n);
    if (n) PGPU_CUDA(cudaMemcpyAsync(p_, h, n * sizeof(T), cudaMemcpyHostToDevice, stream()));
  }
  void upload(const std::vector<T>& v) { upload(v.data(), v.size()); }
  void download(T* h, size_t n) const {
    if (n) PGPU_CUDA(cudaMemcpyAsync(h, p_, n * sizeof(T), cudaMemcpyDeviceToHost, stream()));
  }
  std::vector<T> to_host() const {
    std::vector<T> v(n_);
    download(v.data(), n_);
    PGPU_CUDA(cudaStreamSynchronize(stream()));
    return v;
  }
  T* data() { return p_; }
  const T* data() const { return p_; }
  size_t size() const { return n_; }

 private:
  T* p_ = nullptr;
  size_t n_ = 0;
};

// True when p is a device (or managed) pointer.
bool is_device_pointer(const void* p);

// Copies n doubles from a host-or-device pointer into a device buffer.
void copy_in(DevBuf<double>& dst, const double* src, size_t n);
// Copies n doubles from a device buffer to a host-or-device pointer (synchronizes).
void copy_out(double* dst, const double* src_dev, size_t n);

inline void sync() { PGPU_CUDA(cudaStreamSynchronize(stream())); }
// Waits for this thread's stream without throwing (destructors): errors are left for the next
// checked call.
void sync_quiet() noexcept;

inline int blocks_for(Index n, int threads) {
  Index b = (n + threads - 1) / threads;
  return static_cast<int>(b < 1 ? 1 : b);
}

int num_sms();

// Monotonic host clock in seconds.
double wall_seconds();

// PGPU_VERBOSE set in the environment: progress and phase timings on stdout.
bool verbose();

// Counts kernel launches (every launch site is followed by PGPU_LAUNCH_CHECK).
void count_launch();
int64_t launch_count();

}  // namespace pgpu
