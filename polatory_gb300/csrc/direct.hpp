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

}  // namespace pgpu
