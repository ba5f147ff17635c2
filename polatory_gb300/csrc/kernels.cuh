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

#ifdef __CUDACC__
// ---- float-float arithmetic for the odd polyharmonic kernels ---------------------------------
// Values carried as unevaluated pairs of floats (about 44 significant bits) on the FP32 pipes:
// differences by TwoSum, squares and products by FMA-based TwoProd, the square root one Newton
// step from rsqrtf.
__device__ __forceinline__ void ff_split(double x, float& hi, float& lo) {
  hi = static_cast<float>(x);
  lo = static_cast<float>(x - static_cast<double>(hi));
}

__device__ __forceinline__ void ff_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float v = s - a;
  e = (a - (s - v)) + (b - v);
}

// Adds w * phi(|t - s|) / p0 to the float-float accumulator (ah, al) for -p0 rho (bh3) or
// p0 rho^3 (th3), rho^2 = r^2 + p1^2 with (c_hi, c_lo) = p1^2 (reg: p1 != 0).
template <int KIND>
__device__ __forceinline__ void ff_poly_accumulate(float txh, float txl, float tyh, float tyl,
                                                   float tzh, float tzl, float sxh, float sxl,
                                                   float syh, float syl, float szh, float szl,
                                                   float wh, float wl, bool reg, float c_hi,
                                                   float c_lo, float& ah, float& al) {
  float dxh, dxe, dyh, dye, dzh, dze;
  ff_two_sum(txh, -sxh, dxh, dxe);
  ff_two_sum(tyh, -syh, dyh, dye);
  ff_two_sum(tzh, -szh, dzh, dze);
  dxe += txl - sxl;
  dye += tyl - syl;
  dze += tzl - szl;
  // r^2 = sum (h + e)^2 ~ h^2 + 2 h e.
  const float px = dxh * dxh, py = dyh * dyh, pz = dzh * dzh;
  const float pxe = fmaf(2.0f * dxh, dxe, fmaf(dxh, dxh, -px));
  const float pye = fmaf(2.0f * dyh, dye, fmaf(dyh, dyh, -py));
  const float pze = fmaf(2.0f * dzh, dze, fmaf(dzh, dzh, -pz));
  float a, ea, r2h, eb;
  ff_two_sum(px, py, a, ea);
  ff_two_sum(a, pz, r2h, eb);
  float r2l = ea + eb + pxe + pye + pze;
  if (reg) {
    float sh, se2;
    ff_two_sum(r2h, c_hi, sh, se2);
    r2h = sh;
    r2l += se2 + c_lo;
  }
  {
    const float nh = r2h + r2l;
    r2l = r2l - (nh - r2h);
    r2h = nh;
  }
  const float rinv = rsqrtf(fmaxf(r2h, 1e-30f));
  const float rh = r2h * rinv;
  const float rl = (fmaf(-rh, rh, r2h) + r2l) * (0.5f * rinv);
  float ph, pl;
  if constexpr (KIND == PGPU_RBF_BH3) {
    ph = rh;
    pl = rl;
  } else {
    ph = rh * r2h;
    pl = fmaf(rh, r2h, -ph) + fmaf(rh, r2l, rl * r2h);
  }
  const float th = wh * ph;
  const float tl = fmaf(wh, ph, -th) + fmaf(wh, pl, wl * ph);
  float sh, e2;
  ff_two_sum(ah, th, sh, e2);
  al += e2 + tl;
  ah = sh;
}
#endif

}  // namespace pgpu
