// ResConv parameter-table layout shared by the CUDA-core and the tensor-core kernels.
// FP32 part, per layer l (two per block): W'[i][tap][o] (cin x 9 x C floats; tap =
// 3 (dy+1) + (dx+1)) followed by bias[o] (C floats, zero for the last block's second
// convolution). Then, 256-byte aligned, the tensor-core weight images: per layer the smem
// image of the MMA B operand for 16 channels (zero-padded), [tap][chunk][o][e] with 16-byte
// chunks of e = 8 bf16 / 4 tf32 input channels, followed by 16 FP32 biases; first the BF16
// image of all layers, then the TF32 one (values rounded to nearest).
#pragma once

#include <cstdint>

#include "qgx_common.cuh"

namespace qgx {
namespace {

__host__ __device__ inline int layer_cin(int l, int C) { return l == 0 ? 1 : C; }
__host__ __device__ inline int64_t layer_floats(int l, int C) { return (int64_t)layer_cin(l, C) * 9 * C + C; }
__host__ __device__ inline int64_t layer_offset(int l, int C) {
  int64_t off = 0;
  for (int k = 0; k < l; ++k) off += layer_floats(k, C);
  return off;
}

inline int64_t table_floats_fp32(int B, int C) { return layer_offset(2 * B, C); }

constexpr int kTcCh = 16;  // channel width of the tensor-core tiles
// bytes of one layer's weight image; esz: operand bytes (2 bf16, 4 tf32)
__host__ __device__ inline int64_t tc_layer_bytes(int esz) { return 9LL * (kTcCh * esz / 16) * 256 + 64; }
__host__ __device__ inline int64_t al256_i64(int64_t b) { return (b + 255) / 256 * 256; }
// byte offset of an image from the table start; kind 1: BF16, 0: TF32
__host__ __device__ inline int64_t tc_image_offset(int B, int C, int kind) {
  int64_t off = al256_i64(layer_offset(2 * B, C) * 4);
  if (kind == 0) off += al256_i64(2LL * B * tc_layer_bytes(2));
  return off;
}
inline int64_t table_floats_rc(int B, int C) { return (tc_image_offset(B, C, 0) + 2LL * B * tc_layer_bytes(4)) / 4; }

// TF32 operand value: round to nearest (ties away) on 10 mantissa bits; the MMA itself
// would drop the low 13 bits, a bias that accumulates through the residual stack
__device__ inline float to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ inline float gelu_tanh(float x) {
  const float k0 = 0.7978845608028654f;  // sqrt(2 / pi)
  return 0.5f * x * (1.0f + tanhf(k0 * fmaf(0.044715f * x, x * x, x)));
}

// the same function as 0.5 x (1 + tanh u) = x / (1 + exp(-2u)), with the fast exponential;
// exp overflow gives x / inf = 0, the limit of gelu at -inf
__device__ inline float gelu_fast(float x) {
  const float k0 = 0.7978845608028654f;
  const float u = k0 * fmaf(0.044715f * x, x * x, x);
  return __fdividef(x, 1.0f + __expf(-2.0f * u));
}

// SpinExchange proposal of one chain (common_samplers.py:58-162) on its packed words w
// (nw <= 8, updated in place): site i uniform among the hopping spins (w0 of the draw), j
// uniform in the padded neighbour row of i (w2; -1: no move); returns whether the swap
// changed the configuration
__device__ inline bool propose_exchange(uint32_t (&w)[8], int n, int nw, const u32x4& r, const int32_t* __restrict__ nbr,
                                        int z, int hop) {
  int total = 0;
  for (int k = 0; k < nw; ++k) {
    const uint32_t valid = (32 * k + 32 <= n) ? 0xffffffffu : ((1u << (n - 32 * k)) - 1u);
    total += __popc((hop > 0 ? w[k] : ~w[k]) & valid);
  }
  if (total == 0) return false;
  int pick = (int)bounded(r.x, (uint32_t)total);
  int i = -1;
  for (int k = 0; k < nw && i < 0; ++k) {
    const uint32_t valid = (32 * k + 32 <= n) ? 0xffffffffu : ((1u << (n - 32 * k)) - 1u);
    uint32_t m = (hop > 0 ? w[k] : ~w[k]) & valid;
    const int cnt = __popc(m);
    if (pick < cnt) {
      for (int q = 0; q < pick; ++q) m &= m - 1u;
      i = 32 * k + __ffs(m) - 1;
    } else {
      pick -= cnt;
    }
  }
  int j = nbr[(int64_t)i * z + (int)bounded(r.z, (uint32_t)z)];
  if (j < 0) j = i;
  const uint32_t bi = (w[i >> 5] >> (i & 31)) & 1u, bj = (w[j >> 5] >> (j & 31)) & 1u;
  if (bi == bj) return false;
  w[i >> 5] ^= 1u << (i & 31);
  w[j >> 5] ^= 1u << (j & 31);
  return true;
}

// sinhp1_by_scale (nn/activation.py:7-15) on one final feature z = a + i b, shifted by e^-m:
// f = (sinh z + 1) e^-m and g = f'(z) e^-m = cosh z e^-m, as (re, im) pairs
__device__ inline void sinhp1_shifted(float a, float b, float m, bool cplx, float* fr, float* fi, float* gr, float* gi) {
  float sn = 0.0f, cs = 1.0f;
  if (cplx) sincosf(b, &sn, &cs);
  const float ep = expf(a - m), em = expf(-a - m);
  const float sh = 0.5f * (ep - em), ch = 0.5f * (ep + em);
  *fr = fmaf(sh, cs, expf(-m));
  *fi = ch * sn;
  *gr = ch * cs;
  *gi = sh * sn;
}

// log psi = log mean_e f(z_e) of one configuration, one warp: z_e = scale * za[at(e)] for
// e < cpN (real parts), imaginary parts at za[cpN + at(e)] when cplx; at maps an element of the
// site order to its place in storage (the identity, or a permutation within each channel plane).
// The terms are summed in the order of e whatever the storage. exp_by_scale
// (nn/activation.py:26-32) shifts by max Re z, sinhp1_by_scale by max |Re z|. (re, im) of log psi.
template <class At>
__device__ inline float2 rc_warp_log_psi_at(const float* za, int cpN, float scale, bool cplx, bool sinhp1, int lane,
                                            At at) {
  float m = -INFINITY;
  for (int e = lane; e < cpN; e += 32) {
    const float a = za[at(e)] * scale;
    m = fmaxf(m, sinhp1 ? fabsf(a) : a);
  }
  m = warp_max(m);
  float sr = 0.0f, si = 0.0f;
  for (int e = lane; e < cpN; e += 32) {
    const int k = at(e);
    if (sinhp1) {
      float fr, fi, gr, gi;
      sinhp1_shifted(za[k] * scale, cplx ? za[cpN + k] * scale : 0.0f, m, cplx, &fr, &fi, &gr, &gi);
      sr += fr;
      si += fi;
    } else {
      const float ex = expf(za[k] * scale - m);
      float sn = 0.0f, cs = 1.0f;
      if (cplx) sincosf(za[cpN + k] * scale, &sn, &cs);
      sr = fmaf(ex, cs, sr);
      si = fmaf(ex, sn, si);
    }
  }
  sr = warp_sum(sr);
  si = warp_sum(si);
  return make_float2(m + 0.5f * logf(sr * sr + si * si) - logf((float)cpN), atan2f(si, sr));
}

struct RcSiteOrder {
  __device__ int operator()(int e) const { return e; }
};

__device__ inline float2 rc_warp_log_psi(const float* za, int cpN, float scale, bool cplx, bool sinhp1, int lane) {
  return rc_warp_log_psi_at(za, cpN, scale, cplx, sinhp1, lane, RcSiteOrder{});
}

}  // namespace

// writes both tensor-core weight images from the FP32 part of the table (resconv_tc.cu)
int rc_prepare_tc_images(float* table, int B, int C, cudaStream_t st);

// RBM_Dense on the images of a projected RBM (rbm.cu): log psi as (log psi, 0) pairs of ncfg
// configurations (n_live: device run-time cap, may be NULL), and the uncentred O rows
int rbm_log_psi_pairs(const float* table, int n, int m, const uint32_t* cfg, int64_t ncfg, const int64_t* n_live,
                      float2* out, cudaStream_t st);
int rbm_jacobian_rows(const float* table, int n, int m, int has_vbias, const uint32_t* cfg, int64_t rows, float* O,
                      int64_t ldo, cudaStream_t st);

// tensor-core forward (resconv_tc.cu); kind 0: TF32 operands, 1: BF16 operands (grouped: the
// warp-specialised kernel, where its shape fits)
int rc_launch_forward_tc(const float* table, int L, int B, int C, bool cplx, bool sinhp1, const uint32_t* cfg,
                         int64_t ncfg, const int64_t* n_live, float2* out, int kind, bool grouped,
                         cudaStream_t st);

}  // namespace qgx
