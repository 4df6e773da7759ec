// Shared device helpers of the qgx library: status plumbing, Philox4x32-10, bit-packed
// spin access and warp reductions.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/qgx.h"

namespace qgx {

// ---- status ---------------------------------------------------------------------------
void set_last_error(cudaError_t e);
void set_last_message(const char* msg);
int launch_status();  // QGX_OK or QGX_ERR_CUDA after a kernel launch

#define QGX_CHECK_ARG(cond)            \
  do {                                 \
    if (!(cond)) return QGX_ERR_ARG;   \
  } while (0)

#define QGX_CHECK_CUDA(expr)                 \
  do {                                       \
    cudaError_t e_ = (expr);                 \
    if (e_ != cudaSuccess) {                 \
      ::qgx::set_last_error(e_);             \
      return QGX_ERR_CUDA;                   \
    }                                        \
  } while (0)

inline cudaStream_t as_cuda(qgx_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

constexpr int kNumSMs = 152;  // GB300: 2 dies x 76 SMs (queried at run time where it matters)
int device_sm_count();
int device_max_smem_optin();

// ---- Philox4x32-10 (Salmon et al., SC'11) -----------------------------------------------
struct u32x4 {
  uint32_t x, y, z, w;
};

__host__ __device__ inline uint32_t mulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

__host__ __device__ inline u32x4 philox4x32_10(u32x4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = mulhi32(0xD2511F53u, c.x);
    const uint32_t lo0 = 0xD2511F53u * c.x;
    const uint32_t hi1 = mulhi32(0xCD9E8D57u, c.z);
    const uint32_t lo1 = 0xCD9E8D57u * c.z;
    c = u32x4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

// Stream tags (counter word 3, bits 24..31).
constexpr uint32_t kTagPropose = 1;
constexpr uint32_t kTagInit = 2;
constexpr uint32_t kTagInitPerm = 3;
constexpr uint32_t kTagExact = 4;  // draws of the exact sampler

__host__ __device__ inline u32x4 draw(uint64_t seed, uint64_t chain, uint64_t step, uint32_t tag,
                                      uint32_t substream = 0) {
  u32x4 c{(uint32_t)chain, (uint32_t)step, (uint32_t)(step >> 32), (tag << 24) | (substream & 0xFFFFFFu)};
  return philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}

// (w * n) >> 32: uniform word -> {0..n-1}
__host__ __device__ inline uint32_t bounded(uint32_t w, uint32_t n) {
  return (uint32_t)(((uint64_t)w * n) >> 32);
}

// (w >> 8) * 2^-24: uniform in [0, 1), exact in fp32
__host__ __device__ inline float unit_float(uint32_t w) { return (float)(w >> 8) * (1.0f / 16777216.0f); }

// ((x >> 5) 2^26 + (y >> 6)) 2^-53: uniform in [0, 1) with 53 random bits, exact in fp64
__host__ __device__ inline double unit_double(uint32_t x, uint32_t y) {
  return ((double)(x >> 5) * 67108864.0 + (double)(y >> 6)) * (1.0 / 9007199254740992.0);
}

// ---- packed spins ----------------------------------------------------------------------
__host__ __device__ inline int words_for(int n) { return (n + 31) >> 5; }

// ---- warp helpers ----------------------------------------------------------------------
// A sum kept as an unevaluated pair of floats (h + l), about 48 bits: exact FP32 products
// (TwoProd by FMA) and TwoSum accumulation on the FP32 pipe, where FP64 arithmetic runs at a
// small fraction of the FP32 rate. The _rn intrinsics are never contracted into FMAs, which
// would void the error terms.
struct DSum {
  float h = 0.0f, l = 0.0f;
  __device__ inline void add2(float p, float e) {  // (h, l) += p + e, |e| small
    const float t = __fadd_rn(h, p);
    const float z = __fsub_rn(t, h);
    l = __fadd_rn(l, __fadd_rn(__fadd_rn(__fsub_rn(h, __fsub_rn(t, z)), __fsub_rn(p, z)), e));
    h = t;
  }
  __device__ inline void add(float v) { add2(v, 0.0f); }
  // += a * (yh + yl), the product formed exactly
  __device__ inline void add_prod(float a, float yh, float yl) {
    const float p = __fmul_rn(a, yh);
    float e = fmaf(a, yh, -p);
    e = fmaf(a, yl, e);
    add2(p, e);
  }
  __device__ inline double value() const { return (double)h + (double)l; }
};

// a double as two floats, hi + lo
__device__ inline float2 split_double(double v) {
  const float hi = (float)v;
  return make_float2(hi, (float)(v - (double)hi));
}

__device__ inline float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ inline double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ inline float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Neumaier-compensated double accumulator
struct KahanD {
  double s = 0.0, c = 0.0;
  __device__ inline void add(double x) {
    double t = s + x;
    if (fabs(s) >= fabs(x))
      c += (s - t) + x;
    else
      c += (x - t) + s;
    s = t;
  }
  __device__ inline double value() const { return s + c; }
};

// log cosh(x) = |x| + log1p(exp(-2|x|)) - log 2, accurate for all finite x
__device__ inline float logcoshf(float x) {
  const float ax = fabsf(x);
  return ax + log1pf(expf(-2.0f * ax)) - 0.69314718055994531f;
}

}  // namespace qgx
