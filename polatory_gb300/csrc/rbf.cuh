// RBF kernel formulas, shared by host and device code, templated on the arithmetic type.
//
// Every kernel is isotropic in the anisotropy-transformed space: with d = A (x - y) and
// r2 = |d|^2 the value is phi(r2), the gradient is gcoef(r2) * d and the Hessian is
// ha(r2) * I + hb(r2) * d d^T. The formulas follow the reference kernels one by one:
//   polyharmonic odd   include/polatory/rbf/polyharmonic_odd.hpp:21-67
//   polyharmonic even  include/polatory/rbf/polyharmonic_even.hpp:22-73
//   cov_cubic          include/polatory/rbf/cov_cubic.hpp:33-58
//   cov_exponential    include/polatory/rbf/cov_exponential.hpp:33-61
//   cov_gaussian       include/polatory/rbf/cov_gaussian.hpp:33-61
//   cov_generalized_cauchy{3,5,7,9}  rbf/cov_generalized_cauchy*.hpp:33-66
//   cov_spherical      include/polatory/rbf/cov_spherical.hpp:33-58
//   cov_spheroidal{3,5,7,9}          rbf/cov_spheroidal*.hpp:43-112
// Parameters: p0 = scale (polyharmonic) or psill (covariance); p1 = c or range.
#pragma once

#include <math.h>

#include "polatory_gpu.h"

#if defined(__CUDACC__)
#define PG_HD __host__ __device__ __forceinline__
#else
#define PG_HD inline
#endif

namespace pgpu {

template <class T>
struct M;

template <>
struct M<double> {
  static PG_HD double sqrt(double x) { return ::sqrt(x); }
  static PG_HD double exp(double x) { return ::exp(x); }
  static PG_HD double log(double x) { return ::log(x); }
};

template <>
struct M<float> {
  static PG_HD float sqrt(float x) { return ::sqrtf(x); }
  static PG_HD float exp(float x) { return ::expf(x); }
  static PG_HD float log(float x) { return ::logf(x); }
};

// x^(n/2) for odd n, as rbf_base.hpp:125-147 (sqrt_pow).
template <int N, class T>
PG_HD T sqrt_pow(T x) {
  T s = M<T>::sqrt(x);
  if constexpr (N == 3) return x * s;
  if constexpr (N == 5) return x * x * s;
  if constexpr (N == 7) return x * x * x * s;
  if constexpr (N == 9) {
    T x2 = x * x;
    return x2 * x2 * s;
  }
  if constexpr (N == 11) {
    T x2 = x * x;
    return x2 * x2 * x * s;
  }
  return T(0);
}

// Which kernels have a Hessian (cov_cubic and cov_spherical throw in the reference).
PG_HD bool kind_has_hessian(int kind) { return kind != PGPU_RBF_CUB && kind != PGPU_RBF_SPH; }

PG_HD int kind_cpd_order(int kind) {
  switch (kind) {
    case PGPU_RBF_BH3: return 1;  // (K+1)/2, K=1
    case PGPU_RBF_TH3: return 2;  // K=3
    case PGPU_RBF_BH2: return 2;  // K/2+1, K=2
    case PGPU_RBF_TH2: return 3;  // K=4
    default: return 0;            // covariance functions
  }
}

PG_HD bool kind_is_covariance(int kind) { return kind_cpd_order(kind) == 0; }

// Spheroidal constants (rho0, A, B, C, D, E), cov_spheroidal{3,5,7,9}.hpp:27-32.
struct SpheroidalConst {
  double rho0, a, b, c, d, e;
};

PG_HD SpheroidalConst spheroidal_const(int kind) {
  switch (kind) {
    case PGPU_RBF_SP3:
      return {0.18657871684006438, 2.009875543958482, 0.8734640537108553, 7.181510581693163,
              18.81837403335934, 0.1392464703107397};
    case PGPU_RBF_SP5:
      return {0.2580127411803573, 1.6149073288415876, 0.8575980168032007, 2.5036086535164204,
              10.735449080535068, 0.39942344766841226};
    case PGPU_RBF_SP7:
      return {0.2944149476843637, 1.4859979204216045, 0.8494862533016855, 1.44208314742683,
              8.57520866899984, 0.6934412913598931};
    default:  // SP9: C = E = 1
      return {0.31622776601683794, 1.4230249470757708, 0.8445585690332554, 1.0,
              7.601027121299299, 1.0};
  }
}

PG_HD double support_radius_isotropic(int kind, const double* p) {
  if (kind == PGPU_RBF_CUB || kind == PGPU_RBF_SPH) return p[1];
  return INFINITY;
}

// Internal kinds of the split spheroidal kernels (src/fmm/spheroidal_evaluator.hpp:8-62 with
// rbf/cov_spheroidal{3,5,7,9}.hpp direct_part / fast_part): the smooth fast part is the inverse
// multiquadric tail over all distances, the compact direct part the linear head minus that tail
// inside rho0 (zero beyond). They only reach the FMM's near and far fields (value kernels).
constexpr int kKindSpFast = 16;    // 16..19: fast parts of sp3, sp5, sp7, sp9
constexpr int kKindSpDirect = 20;  // 20..23: direct parts of sp3, sp5, sp7, sp9
PG_HD constexpr int sp_base_kind(int k) {
  return k >= kKindSpDirect ? PGPU_RBF_SP3 + (k - kKindSpDirect) : PGPU_RBF_SP3 + (k - kKindSpFast);
}

// Generalized Cauchy "A" constants, cov_generalized_cauchy{3,5,7}.hpp:24 (gc9 has none: 1).
PG_HD double cauchy_a(int kind) {
  switch (kind) {
    case PGPU_RBF_GC3: return 7.0;
    case PGPU_RBF_GC5: return 2.4822022531844965;
    case PGPU_RBF_GC7: return 1.438027308408951;
    default: return 1.0;
  }
}

// Kernel parameters in the working precision, with derived constants.
template <class T>
struct KParams {
  T p0, p1;
};

// ---- value -----------------------------------------------------------------------------
template <int KIND, class T>
PG_HD T rbf_value(T r2, const KParams<T>& kp) {
  const T p = kp.p0;
  if constexpr (KIND == PGPU_RBF_BH3 || KIND == PGPU_RBF_TH3) {
    T rho2 = r2 + kp.p1 * kp.p1;
    T rho = M<T>::sqrt(rho2);
    if constexpr (KIND == PGPU_RBF_BH3) return -p * rho;
    else return p * rho2 * rho;
  } else if constexpr (KIND == PGPU_RBF_BH2 || KIND == PGPU_RBF_TH2) {
    T rho2 = r2 + kp.p1 * kp.p1;
    T rho = M<T>::sqrt(rho2);
    if (rho == T(0)) return T(0);
    if constexpr (KIND == PGPU_RBF_BH2) return p * rho2 * M<T>::log(rho);
    else return -p * rho2 * rho2 * M<T>::log(rho);
  } else {
    const T range = kp.p1;
    T r = M<T>::sqrt(r2);
    T rho = r / range;
    if constexpr (KIND == PGPU_RBF_CUB) {
      T rho2 = rho * rho;
      return r < range
                 ? p * (T(1) + rho2 * (T(-7) + rho * (T(8.75) + rho2 * (T(-3.5) + T(0.75) * rho2))))
                 : T(0);
    } else if constexpr (KIND == PGPU_RBF_EXP) {
      return p * M<T>::exp(T(-3) * rho);
    } else if constexpr (KIND == PGPU_RBF_GAU) {
      return p * M<T>::exp(T(-3) * rho * rho);
    } else if constexpr (KIND == PGPU_RBF_GC3) {
      return p / sqrt_pow<3>(T(1) + T(cauchy_a(KIND)) * rho * rho);
    } else if constexpr (KIND == PGPU_RBF_GC5) {
      return p / sqrt_pow<5>(T(1) + T(cauchy_a(KIND)) * rho * rho);
    } else if constexpr (KIND == PGPU_RBF_GC7) {
      return p / sqrt_pow<7>(T(1) + T(cauchy_a(KIND)) * rho * rho);
    } else if constexpr (KIND == PGPU_RBF_GC9) {
      return p / sqrt_pow<9>(T(1) + rho * rho);
    } else if constexpr (KIND == PGPU_RBF_SPH) {
      return r < range ? p * (T(1) + rho * (T(-1.5) + T(0.5) * rho * rho)) : T(0);
    } else if constexpr (KIND >= kKindSpFast) {  // split spheroidal parts
      constexpr int base = sp_base_kind(KIND);
      const SpheroidalConst s = spheroidal_const(base);
      const T q = T(1) + T(s.c) * rho * rho;
      T den;
      if constexpr (base == PGPU_RBF_SP3) den = sqrt_pow<3>(q);
      else if constexpr (base == PGPU_RBF_SP5) den = sqrt_pow<5>(q);
      else if constexpr (base == PGPU_RBF_SP7) den = sqrt_pow<7>(q);
      else den = sqrt_pow<9>(q);
      const T imq = p * T(s.b) / den;
      if constexpr (KIND < kKindSpDirect) return imq;
      else return rho < T(s.rho0) ? p * (T(1) - T(s.a) * rho) - imq : T(0);
    } else {  // spheroidal
      const SpheroidalConst s = spheroidal_const(KIND);
      if (rho < T(s.rho0)) return p * (T(1) - T(s.a) * rho);
      T q = T(1) + T(s.c) * rho * rho;
      T den;
      if constexpr (KIND == PGPU_RBF_SP3) den = sqrt_pow<3>(q);
      else if constexpr (KIND == PGPU_RBF_SP5) den = sqrt_pow<5>(q);
      else if constexpr (KIND == PGPU_RBF_SP7) den = sqrt_pow<7>(q);
      else den = sqrt_pow<9>(q);
      return p * T(s.b) / den;
    }
  }
}

#if defined(__CUDACC__)
// FP32 near-field value with fewer instructions for the odd polyharmonic kernels: rho as
// rho2 * rsqrt(rho2) (MUFU.RSQ, ~2 ulp) with rho2 clamped away from zero, which changes the
// value at coincident points by less than 1e-14 relative to the kernel scale.
template <int KIND>
__device__ __forceinline__ float rbf_value_fast(float r2, const KParams<float>& kp) {
  if constexpr (KIND == PGPU_RBF_BH3 || KIND == PGPU_RBF_TH3) {
    const float rho2 = fmaxf(r2 + kp.p1 * kp.p1, 1e-30f);
    const float rho = rho2 * rsqrtf(rho2);
    if constexpr (KIND == PGPU_RBF_BH3) return -kp.p0 * rho;
    else return kp.p0 * rho2 * rho;
  } else {
    return rbf_value<KIND>(r2, kp);
  }
}
template <int KIND>
__device__ __forceinline__ double rbf_value_fast(double r2, const KParams<double>& kp) {
  return rbf_value<KIND>(r2, kp);
}

// Near-field pair term acc + w' phi(d) with the kernel's constant factor folded into the staged
// weight w' = w * pair_weight_scale and, for the odd polyharmonic kernels in FP32, the
// regularisation p1^2 (plus 1e-30, which keeps rsqrt finite at d = 0 and is below the rounding
// of any nonzero squared distance of leaf-sized coordinates) folded into the first FMA of r^2:
//   bh3: -p0 rho = w' rho with w' = -p0 w;  th3: p0 rho^3 = w' rho^3 with w' = p0 w,
// rho = rho2 * rsqrt(rho2). Other kernels: rbf_value_fast(r^2) * w.
template <int KIND, class T>
__device__ __forceinline__ T pair_weight_scale(const KParams<T>& kp) {
  if constexpr (sizeof(T) == 4 && KIND == PGPU_RBF_BH3) return -kp.p0;
  else if constexpr (sizeof(T) == 4 && KIND == PGPU_RBF_TH3) return kp.p0;
  else return T(1);
}
template <int KIND, class T>
__device__ __forceinline__ T pair_r2_offset(const KParams<T>& kp) {
  if constexpr (sizeof(T) == 4 && (KIND == PGPU_RBF_BH3 || KIND == PGPU_RBF_TH3))
    return kp.p1 * kp.p1 + 1e-30f;
  else return T(0);
}
template <int KIND, class T>
__device__ __forceinline__ T pair_term(T dx, T dy, T dz, T w, T c2, const KParams<T>& kp, T acc) {
  if constexpr (sizeof(T) == 4 && (KIND == PGPU_RBF_BH3 || KIND == PGPU_RBF_TH3)) {
    const T rho2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, c2)));
    const T rho = rho2 * rsqrtf(rho2);
    if constexpr (KIND == PGPU_RBF_BH3) return fmaf(w, rho, acc);
    else return fmaf(w, rho2 * rho, acc);
  } else {
    return acc + rbf_value_fast<KIND>(dx * dx + dy * dy + dz * dz, kp) * w;
  }
}
#endif

// ---- gradient coefficient: grad = gcoef * d ---------------------------------------------
template <int KIND, class T>
PG_HD T rbf_gcoef(T r2, const KParams<T>& kp) {
  const T p = kp.p0;
  if constexpr (KIND == PGPU_RBF_BH3 || KIND == PGPU_RBF_TH3) {
    T rho2 = r2 + kp.p1 * kp.p1;
    T rho = M<T>::sqrt(rho2);
    if (rho == T(0)) return T(0);
    if constexpr (KIND == PGPU_RBF_BH3) return -p / rho;
    else return T(3) * p * rho;
  } else if constexpr (KIND == PGPU_RBF_BH2 || KIND == PGPU_RBF_TH2) {
    T rho2 = r2 + kp.p1 * kp.p1;
    T rho = M<T>::sqrt(rho2);
    if (rho == T(0)) return T(0);
    if constexpr (KIND == PGPU_RBF_BH2) return p * (T(1) + T(2) * M<T>::log(rho));
    else return -p * rho2 * (T(1) + T(4) * M<T>::log(rho));
  } else {
    const T range = kp.p1;
    T r = M<T>::sqrt(r2);
    T rho = r / range;
    if constexpr (KIND == PGPU_RBF_CUB) {
      T rho2 = rho * rho;
      return r < range ? p * (T(-14) + rho * (T(26.25) + rho2 * (T(-17.5) + T(5.25) * rho2))) /
                             (range * range)
                       : T(0);
    } else if constexpr (KIND == PGPU_RBF_EXP) {
      return T(-3) * p * M<T>::exp(T(-3) * rho) / (range * r);
    } else if constexpr (KIND == PGPU_RBF_GAU) {
      return T(-6) * p * M<T>::exp(T(-3) * rho * rho) / (range * range);
    } else if constexpr (KIND == PGPU_RBF_GC3) {
      const T ka = T(cauchy_a(KIND));
      return -ka * T(3) * p / (sqrt_pow<5>(T(1) + ka * rho * rho) * range * range);
    } else if constexpr (KIND == PGPU_RBF_GC5) {
      const T ka = T(cauchy_a(KIND));
      return -ka * T(5) * p / (sqrt_pow<7>(T(1) + ka * rho * rho) * range * range);
    } else if constexpr (KIND == PGPU_RBF_GC7) {
      const T ka = T(cauchy_a(KIND));
      return -ka * T(7) * p / (sqrt_pow<9>(T(1) + ka * rho * rho) * range * range);
    } else if constexpr (KIND == PGPU_RBF_GC9) {
      return T(-9) * p / (sqrt_pow<11>(T(1) + rho * rho) * range * range);
    } else if constexpr (KIND == PGPU_RBF_SPH) {
      return r < range ? p * (T(-1.5) / rho + T(1.5) * rho) / (range * range) : T(0);
    } else {
      const SpheroidalConst s = spheroidal_const(KIND);
      if (rho < T(s.rho0)) return -p * T(s.a) / (r * range);
      T q = T(1) + T(s.c) * rho * rho;
      T den;
      if constexpr (KIND == PGPU_RBF_SP3) den = sqrt_pow<5>(q);
      else if constexpr (KIND == PGPU_RBF_SP5) den = sqrt_pow<7>(q);
      else if constexpr (KIND == PGPU_RBF_SP7) den = sqrt_pow<9>(q);
      else den = sqrt_pow<11>(q);
      return -p * T(s.d) / (den * range * range);
    }
  }
}

// ---- Hessian: H = ha * I + hb * d d^T ------------------------------------------------------
// Kernels without a Hessian (cub, sph) return zeros here; the host rejects them before any
// launch that needs a Hessian.
template <int KIND, class T>
PG_HD void rbf_hess(T r2, const KParams<T>& kp, T& ha, T& hb) {
  const T p = kp.p0;
  if constexpr (KIND == PGPU_RBF_BH3 || KIND == PGPU_RBF_TH3) {
    T rho2 = r2 + kp.p1 * kp.p1;
    T rho = M<T>::sqrt(rho2);
    if (rho == T(0)) {
      ha = hb = T(0);
      return;
    }
    if constexpr (KIND == PGPU_RBF_BH3) {
      T c = -p / rho;
      ha = c;
      hb = -c / rho2;  // (K - 2) / rho2 with K = 1
    } else {
      T c = T(3) * p * rho;
      ha = c;
      hb = c / rho2;  // K - 2 = 1
    }
  } else if constexpr (KIND == PGPU_RBF_BH2 || KIND == PGPU_RBF_TH2) {
    T rho2 = r2 + kp.p1 * kp.p1;
    T rho = M<T>::sqrt(rho2);
    if (rho == T(0)) {
      ha = hb = T(0);
      return;
    }
    T lg = M<T>::log(rho);
    if constexpr (KIND == PGPU_RBF_BH2) {
      T c = p * (T(1) + T(2) * lg);
      ha = c;
      hb = c * (T(2) / (T(1) + T(2) * lg)) / rho2;  // K - 2 + K / (1 + K log rho), K = 2
    } else {
      T c = -p * rho2 * (T(1) + T(4) * lg);
      ha = c;
      hb = c * (T(2) + T(4) / (T(1) + T(4) * lg)) / rho2;
    }
  } else if constexpr (KIND == PGPU_RBF_CUB || KIND == PGPU_RBF_SPH) {
    ha = hb = T(0);
  } else {
    const T range = kp.p1;
    T r = M<T>::sqrt(r2);
    T rho = r / range;
    if constexpr (KIND == PGPU_RBF_EXP) {
      T c = T(-3) * p * M<T>::exp(T(-3) * rho) / (range * r);
      ha = c;
      hb = -c * (T(1) / (r * r) + T(3) / (range * r));
    } else if constexpr (KIND == PGPU_RBF_GAU) {
      T c = T(-6) * p * M<T>::exp(T(-3) * rho * rho) / (range * range);
      ha = c;
      hb = -c * T(6) / (range * range);
    } else if constexpr (KIND == PGPU_RBF_GC3 || KIND == PGPU_RBF_GC5 || KIND == PGPU_RBF_GC7) {
      const T ka = T(cauchy_a(KIND));
      T q = T(1) + ka * rho * rho;
      T c;
      T f;
      if constexpr (KIND == PGPU_RBF_GC3) {
        c = -ka * T(3) * p / (sqrt_pow<5>(q) * range * range);
        f = ka * T(5);
      } else if constexpr (KIND == PGPU_RBF_GC5) {
        c = -ka * T(5) * p / (sqrt_pow<7>(q) * range * range);
        f = ka * T(7);
      } else {
        c = -ka * T(7) * p / (sqrt_pow<9>(q) * range * range);
        f = ka * T(9);
      }
      ha = c;
      hb = -c * f / (ka * r * r + range * range);
    } else if constexpr (KIND == PGPU_RBF_GC9) {
      T c = T(-9) * p / (sqrt_pow<11>(T(1) + rho * rho) * range * range);
      ha = c;
      hb = -c * T(11) / (r * r + range * range);
    } else {
      const SpheroidalConst s = spheroidal_const(KIND);
      if (rho < T(s.rho0)) {
        T c = -p * T(s.a) / (r * range);
        ha = c;
        hb = -c / (r * r);
      } else {
        T q = T(1) + T(s.c) * rho * rho;
        T den;
        T f;
        if constexpr (KIND == PGPU_RBF_SP3) {
          den = sqrt_pow<5>(q);
          f = T(5);
        } else if constexpr (KIND == PGPU_RBF_SP5) {
          den = sqrt_pow<7>(q);
          f = T(7);
        } else if constexpr (KIND == PGPU_RBF_SP7) {
          den = sqrt_pow<9>(q);
          f = T(9);
        } else {
          den = sqrt_pow<11>(q);
          f = T(11);
        }
        T c = -p * T(s.d) / (den * range * range);
        ha = c;
        hb = -c * f / (r * r + T(s.e) * range * range);
      }
    }
  }
}

// Runtime dispatch over the 16 kinds: calls f.template operator()<KIND>().
template <class F>
PG_HD auto dispatch_kind(int kind, F&& f) {
  switch (kind) {
    case PGPU_RBF_BH2: return f.template operator()<PGPU_RBF_BH2>();
    case PGPU_RBF_BH3: return f.template operator()<PGPU_RBF_BH3>();
    case PGPU_RBF_CUB: return f.template operator()<PGPU_RBF_CUB>();
    case PGPU_RBF_EXP: return f.template operator()<PGPU_RBF_EXP>();
    case PGPU_RBF_GAU: return f.template operator()<PGPU_RBF_GAU>();
    case PGPU_RBF_GC3: return f.template operator()<PGPU_RBF_GC3>();
    case PGPU_RBF_GC5: return f.template operator()<PGPU_RBF_GC5>();
    case PGPU_RBF_GC7: return f.template operator()<PGPU_RBF_GC7>();
    case PGPU_RBF_GC9: return f.template operator()<PGPU_RBF_GC9>();
    case PGPU_RBF_SPH: return f.template operator()<PGPU_RBF_SPH>();
    case PGPU_RBF_SP3: return f.template operator()<PGPU_RBF_SP3>();
    case PGPU_RBF_SP5: return f.template operator()<PGPU_RBF_SP5>();
    case PGPU_RBF_SP7: return f.template operator()<PGPU_RBF_SP7>();
    case PGPU_RBF_SP9: return f.template operator()<PGPU_RBF_SP9>();
    case PGPU_RBF_TH2: return f.template operator()<PGPU_RBF_TH2>();
    default: return f.template operator()<PGPU_RBF_TH3>();
  }
}

// The FMM's dispatch: the 16 public kinds and the split spheroidal parts.
template <class F>
PG_HD auto dispatch_fmm_kind(int kind, F&& f) {
  switch (kind) {
    case kKindSpFast + 0: return f.template operator()<kKindSpFast + 0>();
    case kKindSpFast + 1: return f.template operator()<kKindSpFast + 1>();
    case kKindSpFast + 2: return f.template operator()<kKindSpFast + 2>();
    case kKindSpFast + 3: return f.template operator()<kKindSpFast + 3>();
    case kKindSpDirect + 0: return f.template operator()<kKindSpDirect + 0>();
    case kKindSpDirect + 1: return f.template operator()<kKindSpDirect + 1>();
    case kKindSpDirect + 2: return f.template operator()<kKindSpDirect + 2>();
    case kKindSpDirect + 3: return f.template operator()<kKindSpDirect + 3>();
    default: return dispatch_kind(kind, f);
  }
}

}  // namespace pgpu
