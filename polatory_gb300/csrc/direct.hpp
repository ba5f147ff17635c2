// Host interface of the direct-sum kernels.
#pragma once

#include "common.hpp"
#include "kernels.cuh"

namespace pgpu {

// Sources in the anisotropy frame: value sources (position + weight) and gradient sources
// (position + A g, three entries per source).
template <class T>
struct DirectSources {
  const P4<T>* vpos = nullptr;
  const T* vw = nullptr;
  Index nv = 0;
  const P4<T>* gpos = nullptr;
  const T* gg = nullptr;
  Index ng = 0;
};

// Targets: value targets add into out_v[i]; gradient targets add A^T (A-frame gradient) into
// out_g[3 i + k].
template <class T>
struct DirectTargets {
  const P4<T>* vpos = nullptr;
  Index nv = 0;
  double* out_v = nullptr;
  const P4<T>* gpos = nullptr;
  Index ng = 0;
  double* out_g = nullptr;
};

template <class T>
void direct_evaluate(int kind, const KParams<T>& kp, const Mat3& a, const DirectSources<T>& src,
                     const DirectTargets<T>& trg, cudaStream_t st);

// Value sources to value targets of the odd polyharmonic kernels (bh3, th3) in float-float
// arithmetic: FP64-class accuracy on the FP32 pipes. Returns false for other kernels (the
// caller then uses the FP64 kernel). Positions: FP64 frame coordinates; out is added to.
bool direct_evaluate_ff(int kind, const KParams<double>& kp, const P4<double>* spos,
                        const double* w, Index ns, const P4<double>* tpos, Index nt, double* out,
                        cudaStream_t st);

}  // namespace pgpu
