// Column-statistics kernels shared by the centring paths (generic dense O and the RBM
// Obar writer). Each translation unit that includes this header gets its own copy.
#pragma once

#include "qgx_common.cuh"

namespace qgx {
namespace {

// mean_u[col] = sum_k part_u[k, col] / ns, omean[col] = sum_k part_w[k, col] / ns,
// mean_f = float copy of mean_u (may be NULL).
__global__ void col_reduce_kernel(const double* __restrict__ part_u, const double* __restrict__ part_w,
                                  int64_t nchunk, int64_t np, int64_t ns, double* __restrict__ mean_u,
                                  double* __restrict__ omean, float* __restrict__ mean_f) {
  const int64_t col = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (col >= np) return;
  KahanD su, sw;
  for (int64_t k = 0; k < nchunk; ++k) {
    su.add(part_u[k * np + col]);
    sw.add(part_w[k * np + col]);
  }
  const double mu = su.value() / (double)ns;
  if (mean_u) mean_u[col] = mu;
  if (mean_f) mean_f[col] = (float)mu;
  if (omean) omean[col] = sw.value() / (double)ns;
}

}  // namespace
}  // namespace qgx
