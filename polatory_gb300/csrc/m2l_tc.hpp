// Tensor-core M2L (tcgen05, TF32 head/tail split) for the FP32 far field at order 6.
#pragma once

#include "common.hpp"

namespace pgpu {

// The 343 operators of one level in the MMA's shared-memory layout, head and tail.
struct M2LTcBlocks {
  DevBuf<float> hi, lo;
};

// PGPU_M2L_TC=0 in the environment selects the CUDA-core M2L everywhere.
bool m2l_tc_enabled();
// K: 343 x 216 x 216 row-major (target node, source node) operators of one level.
M2LTcBlocks make_m2l_tc_blocks(const float* K);
// L[t] += sum_o K_o M[table[t][o]] for the nt target cells; *err is set if a wait timed out.
void m2l_tc_apply(const M2LTcBlocks& b, const int* table, Index nt, const float* Ms, float* L,
                  int* err, cudaStream_t st);

}  // namespace pgpu
