// Device-side building blocks shared by the direct, near-field (P2P) and assembly kernels.
#pragma once

#include <cuda_runtime.h>

#include "rbf.cuh"

namespace pgpu {

// Packed point: position in the anisotropy-transformed frame, relative to a frame origin
// (so that FP32 copies keep their precision), plus one payload slot.
template <class T>
struct alignas(4 * sizeof(T)) P4 {
  T x, y, z, w;
};

// Interaction of one source with one target, summed into value or gradient accumulators.
//   value target  <- value source : phi(d) w
//   value target  <- grad source  : -gcoef(d) (G . d)          (= G . grad_y phi)
//   grad target   <- value source : gcoef(d) d w               (A-frame gradient)
//   grad target   <- grad source  : -(ha G + hb d (d . G))     (= -H G)
// with d = X_target - Y_source, matching interpolation/direct_evaluator.hpp:45-79 once the
// A-frame gradient is mapped back with A^T and G = A g.
template <int KIND, class T>
__device__ __forceinline__ void acc_value_from_value(T dx, T dy, T dz, T w, const KParams<T>& kp,
                                                     T& acc) {
  T r2 = dx * dx + dy * dy + dz * dz;
  acc += rbf_value<KIND>(r2, kp) * w;
}

template <int KIND, class T>
__device__ __forceinline__ void acc_value_from_grad(T dx, T dy, T dz, T gx, T gy, T gz,
                                                    const KParams<T>& kp, T& acc) {
  T r2 = dx * dx + dy * dy + dz * dz;
  T c = rbf_gcoef<KIND>(r2, kp);
  acc -= c * (gx * dx + gy * dy + gz * dz);
}

template <int KIND, class T>
__device__ __forceinline__ void acc_grad_from_value(T dx, T dy, T dz, T w, const KParams<T>& kp,
                                                    T& ax, T& ay, T& az) {
  T r2 = dx * dx + dy * dy + dz * dz;
  T c = rbf_gcoef<KIND>(r2, kp) * w;
  ax += c * dx;
  ay += c * dy;
  az += c * dz;
}

template <int KIND, class T>
__device__ __forceinline__ void acc_grad_from_grad(T dx, T dy, T dz, T gx, T gy, T gz,
                                                   const KParams<T>& kp, T& ax, T& ay, T& az) {
  T r2 = dx * dx + dy * dy + dz * dz;
  T ha, hb;
  rbf_hess<KIND>(r2, kp, ha, hb);
  T dg = dx * gx + dy * gy + dz * gz;
  ax -= ha * gx + hb * dx * dg;
  ay -= ha * gy + hb * dy * dg;
  az -= ha * gz + hb * dz * dg;
}

// 3x3 row-major matrix-vector products for the A-frame <-> original-frame maps.
__device__ __forceinline__ void mat3_tvec(const double* a, double x, double y, double z,
                                          double& ox, double& oy, double& oz) {
  // A^T v
  ox = a[0] * x + a[3] * y + a[6] * z;
  oy = a[1] * x + a[4] * y + a[7] * z;
  oz = a[2] * x + a[5] * y + a[8] * z;
}

__device__ __forceinline__ void mat3_vec(const double* a, double x, double y, double z,
                                         double& ox, double& oy, double& oz) {
  // A v
  ox = a[0] * x + a[1] * y + a[2] * z;
  oy = a[3] * x + a[4] * y + a[5] * z;
  oz = a[6] * x + a[7] * y + a[8] * z;
}

struct Mat3 {
  double a[9];
};

// Algorithmic flops of one value-value pair interaction (3 subtractions, 5 for r^2, the kernel,
// 2 for the multiply-add into the accumulator; sqrt/exp/log/div count 1): biharmonic 11,
// triharmonic 13, exponential 14; the other kernels are counted like the exponential.
inline double pair_flops(int kind) {
  switch (kind) {
    case PGPU_RBF_BH3: return 11.0;
    case PGPU_RBF_TH3: return 13.0;
    default: return 14.0;
  }
}

}  // namespace pgpu
