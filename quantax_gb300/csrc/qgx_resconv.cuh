// ResConv parameter-table layout shared by the CUDA-core and the tensor-core kernels.
// Per layer l (two per block): W'[i][tap][o] (cin x 9 x C floats; tap = 3 (dy+1) + (dx+1))
// followed by bias[o] (C floats, zero for the last block's second convolution).
#pragma once

#include <cstdint>

namespace qgx {
namespace {

__host__ __device__ inline int layer_cin(int l, int C) { return l == 0 ? 1 : C; }
__host__ __device__ inline int64_t layer_floats(int l, int C) { return (int64_t)layer_cin(l, C) * 9 * C + C; }
__host__ __device__ inline int64_t layer_offset(int l, int C) {
  int64_t off = 0;
  for (int k = 0; k < l; ++k) off += layer_floats(k, C);
  return off;
}

__device__ inline float gelu_tanh(float x) {
  const float k0 = 0.7978845608028654f;  // sqrt(2 / pi)
  return 0.5f * x * (1.0f + tanhf(k0 * fmaf(0.044715f * x, x * x, x)));
}

}  // namespace

// tensor-core forward (resconv_tc.cu); kind 0: TF32 operands, 1: BF16 operands
int rc_launch_forward_tc(const float* table, int L, int B, int C, bool cplx, const uint32_t* cfg, int64_t ncfg,
                         const int64_t* n_live, float2* out, int kind, cudaStream_t st);

}  // namespace qgx
