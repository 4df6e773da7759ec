// Gram matrices of the SR / MinSR solve (quantax/optimizer/solver.py:139 T = A A^T and
// :157 S = A^T A), FP32 operands, written as FP64 for the solver.
//
// This file holds the SIMT paths: QGX_GRAM_FP32 (FP32 accumulation) and QGX_GRAM_FP64, the
// Gram of the FP32 matrix to about 48 bits: every product is formed exactly as a float pair
// (TwoProd by FMA) and summed into a float-pair accumulator (TwoSum). FP64 arithmetic runs at
// a small fraction of the FP32 rate on this GPU, and this keeps the work on the FP32 pipe.
// 128 x 128 output tiles, 256
// threads with 8 x 8 register micro-tiles, K staged through shared memory in chunks of
// 16 with a register prefetch of the next chunk. Only tiles on or below the diagonal
// are computed; each off-diagonal tile is written twice (itself and its mirror). The
// tensor-core paths (TF32 / BF16 / split TF32) live in gram_tc.cu.
#include <algorithm>

#include "qgx_common.cuh"

namespace qgx {

int gram_tc(const float* A, int64_t rows, int64_t k, int64_t lda, double* T, int64_t ldt, int mode, cudaStream_t st);

namespace {

constexpr int BM = 128;
constexpr int BK = 16;
constexpr int NT = 256;
constexpr int PAD = 4;

// TRANS = false: vectors are rows of A (T = A A^T, vector length k, count rows)
// TRANS = true : vectors are columns of A (S = A^T A, vector length rows, count k)
template <bool TRANS>
__device__ inline float load_elem(const float* __restrict__ A, int64_t lda, int64_t vec, int64_t kk, int64_t nvec,
                                  int64_t klen) {
  if (vec >= nvec || kk >= klen) return 0.0f;
  return TRANS ? __ldg(A + kk * lda + vec) : __ldg(A + vec * lda + kk);
}

// (h, l) += a * b exactly rounded to a float pair; the _rn intrinsics are never contracted
__device__ inline void ds_fma(float a, float b, float& h, float& l) {
  const float p = __fmul_rn(a, b);
  const float e = fmaf(a, b, -p);
  const float t = __fadd_rn(h, p);
  const float z = __fsub_rn(t, h);
  l = __fadd_rn(l, __fadd_rn(__fadd_rn(__fsub_rn(h, __fsub_rn(t, z)), __fsub_rn(p, z)), e));
  h = t;
}

template <bool TRANS, bool DS>
__global__ void __launch_bounds__(NT, 1)
    gram_simt_kernel(const float* __restrict__ A, int64_t nvec, int64_t klen, int64_t lda, double* __restrict__ T,
                     int64_t ldt) {
  __shared__ __align__(16) float As[2][BK][BM + PAD];
  __shared__ __align__(16) float Bs[2][BK][BM + PAD];

  // lower-triangular tile index -> (bi, bj), bi >= bj
  const int64_t tile = blockIdx.x;
  int64_t bi = (int64_t)((sqrt(8.0 * (double)tile + 1.0) - 1.0) * 0.5);
  while ((bi + 1) * (bi + 2) / 2 <= tile) ++bi;
  while (bi * (bi + 1) / 2 > tile) --bi;
  const int64_t bj = tile - bi * (bi + 1) / 2;
  const int64_t row0 = bi * BM, col0 = bj * BM;

  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;  // 16 x 16 thread grid, 8 x 8 each

  // loader mapping: 2048 elements per operand tile per chunk, 8 per thread
  float ra[8], rb[8];
  auto gload = [&](int64_t k0) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int e = tid + q * NT;  // 0..2047
      int v, kk;
      if (TRANS) {  // contiguous along vectors
        v = e % BM;
        kk = e / BM;
      } else {  // contiguous along k
        v = e / BK;
        kk = e % BK;
      }
      ra[q] = load_elem<TRANS>(A, lda, row0 + v, k0 + kk, nvec, klen);
      rb[q] = load_elem<TRANS>(A, lda, col0 + v, k0 + kk, nvec, klen);
    }
  };
  auto sstore = [&](int buf) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int e = tid + q * NT;
      int v, kk;
      if (TRANS) {
        v = e % BM;
        kk = e / BM;
      } else {
        v = e / BK;
        kk = e % BK;
      }
      As[buf][kk][v] = ra[q];
      Bs[buf][kk][v] = rb[q];
    }
  };

  float acc[8][8], accl[DS ? 8 : 1][DS ? 8 : 1];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;
#pragma unroll
  for (int i = 0; i < (DS ? 8 : 1); ++i)
#pragma unroll
    for (int j = 0; j < (DS ? 8 : 1); ++j) accl[i][j] = 0.0f;

  const int64_t nk = (klen + BK - 1) / BK;
  gload(0);
  sstore(0);
  __syncthreads();
  for (int64_t kc = 0; kc < nk; ++kc) {
    const int buf = (int)(kc & 1);
    if (kc + 1 < nk) gload((kc + 1) * BK);
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      float a[8], b[8];
      const float4 a0 = *reinterpret_cast<const float4*>(&As[buf][kk][ty * 4]);
      const float4 a1 = *reinterpret_cast<const float4*>(&As[buf][kk][64 + ty * 4]);
      const float4 b0 = *reinterpret_cast<const float4*>(&Bs[buf][kk][tx * 4]);
      const float4 b1 = *reinterpret_cast<const float4*>(&Bs[buf][kk][64 + tx * 4]);
      a[0] = a0.x; a[1] = a0.y; a[2] = a0.z; a[3] = a0.w;
      a[4] = a1.x; a[5] = a1.y; a[6] = a1.z; a[7] = a1.w;
      b[0] = b0.x; b[1] = b0.y; b[2] = b0.z; b[3] = b0.w;
      b[4] = b1.x; b[5] = b1.y; b[6] = b1.z; b[7] = b1.w;
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          if constexpr (DS) {
            ds_fma(a[i], b[j], acc[i][j], accl[i & (DS ? 7 : 0)][j & (DS ? 7 : 0)]);
          } else {
            acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
          }
        }
    }
    if constexpr (DS) {
      // renormalise each pair (FastTwoSum, |h| >= |l|) once per chunk: the low word stays
      // below half an ulp of the high word, which keeps its own rounding negligible (about
      // 1e-13 relative at K = 8192, against 3e-12 without)
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          float& h = acc[i][j];
          float& l = accl[i & (DS ? 7 : 0)][j & (DS ? 7 : 0)];
          const float t = __fadd_rn(h, l);
          l = __fsub_rn(l, __fsub_rn(t, h));
          h = t;
        }
    }
    if (kc + 1 < nk) sstore(buf ^ 1);
    __syncthreads();
  }

  // write the tile and, off the diagonal, its mirror
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int64_t r = row0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + (i - 4));
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int64_t c = col0 + (j < 4 ? tx * 4 + j : 64 + tx * 4 + (j - 4));
      if (r < nvec && c < nvec) {
        double v = (double)acc[i][j];
        if constexpr (DS) v += (double)accl[i & (DS ? 7 : 0)][j & (DS ? 7 : 0)];
        T[r * ldt + c] = v;
        if (bi != bj) T[c * ldt + r] = v;
      }
    }
  }
}

template <bool TRANS, bool DS = false>
int launch_gram_simt(const float* A, int64_t nvec, int64_t klen, int64_t lda, double* T, int64_t ldt, cudaStream_t st) {
  const int64_t nb = (nvec + BM - 1) / BM;
  const int64_t tiles = nb * (nb + 1) / 2;
  if (tiles > 0x7fffffff) return QGX_ERR_UNSUPPORTED;
  gram_simt_kernel<TRANS, DS><<<(unsigned)tiles, NT, 0, st>>>(A, nvec, klen, lda, T, ldt);
  return launch_status();
}

}  // namespace
}  // namespace qgx

using namespace qgx;

extern "C" {

int qgx_gram(const float* A, int64_t rows, int64_t k, int64_t lda, double* T, int64_t ldt, int32_t mode,
             qgx_stream_t stream) {
  QGX_CHECK_ARG(rows >= 0 && k >= 0 && lda >= k && ldt >= rows);
  if (rows == 0) return QGX_OK;
  QGX_CHECK_ARG(A && T);
  if (mode == QGX_GRAM_FP32) return launch_gram_simt<false>(A, rows, k, lda, T, ldt, as_cuda(stream));
  if (mode == QGX_GRAM_FP64) return launch_gram_simt<false, true>(A, rows, k, lda, T, ldt, as_cuda(stream));
  if (mode == QGX_GRAM_TF32 || mode == QGX_GRAM_BF16 || mode == QGX_GRAM_3XTF32)
    return gram_tc(A, rows, k, lda, T, ldt, mode, as_cuda(stream));
  return QGX_ERR_ARG;
}

int qgx_gram_t(const float* A, int64_t rows, int64_t k, int64_t lda, double* S, int64_t lds, qgx_stream_t stream) {
  QGX_CHECK_ARG(rows >= 0 && k >= 0 && lda >= k && lds >= k);
  if (k == 0) return QGX_OK;
  QGX_CHECK_ARG(A && S);
  return launch_gram_simt<true>(A, k, rows, lda, S, lds, as_cuda(stream));
}

}  // extern "C"
