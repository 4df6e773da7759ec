// ResConv forward on the tcgen05 tensor cores (TF32 or BF16 operands, FP32 accumulation
// in TMEM), the precision form of quantax/model/conv_nets.py:26-183.
//
// A CTA holds S samples. Conv inputs are stored chunk-major over a halo-padded grid:
// every sample occupies (L+2)^2 rows, row (y+1)(L+2) + (x+1) holds site (y, x) and the
// halo rows repeat the periodic neighbours. A chunk is 16 bytes of channels (8 bf16 or
// 4 tf32) and chunk c of every row is contiguous (row stride 16 bytes). Then the 3x3
// circular convolution for 128 output rows is, for each tap (dy, dx), one MMA (two for
// TF32) whose A operand starts dy (L+2) + dx rows further: D[128 x 16] += A_tap[128 x 16]
// W_tap[16 x 16]. No im2col tile is built; the descriptor (no swizzle, K-major: 16-byte
// core-matrix rows, leading offset = one chunk plane, stride offset = 8 rows) points into
// the activation buffer directly. All tiles of a layer accumulate in TMEM at once (16
// columns each); one commit, then the epilogue applies bias, GELU / the residual add and
// refills the halo. The residual stream x stays in FP32; the one-channel first convolution
// runs on the CUDA cores.
#include <cuda_bf16.h>

#include <algorithm>

#include "qgx_common.cuh"
#include "qgx_resconv.cuh"
#include "qgx_tc.cuh"

namespace qgx {
namespace {

constexpr int kThreadsTc = 128;
constexpr int kCh = 16;  // channel width of the tiles; C < 16 runs zero-padded
constexpr int kGuard = 32;

template <int KIND>  // 1: bf16, 0: tf32
struct TcCfg {
  static constexpr int esz = KIND == 1 ? 2 : 4;
  static constexpr int epc = 16 / esz;           // elements per 16-byte chunk
  static constexpr int chunks = kCh / epc;       // chunk planes of the 16 channels
  static constexpr int mma_per_tap = chunks / 2; // an MMA covers 32 bytes of K
  static constexpr uint32_t fmt = KIND == 1 ? 1u : 2u;
  static constexpr uint32_t idesc = (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(kCh >> 3) << 17) |
                                    ((uint32_t)(128 >> 4) << 24);
};

struct TcShape {
  int L, N, Lp, NP, B, C, S, ntiles, rows_tot;
  bool cplx;
  // byte offsets in shared memory
  int oX, oP, oQ, oW, oBias, oW0, oHalo, oNbr, oBar;
  int smem;
  uint32_t tmem_cols;
};

// samples per CTA: enough padded rows for nine 128-row tiles at L = 10
inline int tc_samples_per_cta(int L) { return std::max(1, std::min(32, 1152 / ((L + 2) * (L + 2)))); }

inline TcShape tc_shape(int L, int B, int C, bool cplx, int esz, int S) {
  TcShape s;
  s.L = L;
  s.C = C;
  s.N = L * L;
  s.Lp = L + 2;
  s.NP = s.Lp * s.Lp;
  s.B = B;
  s.cplx = cplx;
  s.S = S;
  const int rows = s.S * s.NP;
  s.ntiles = (rows + 127) / 128;
  s.rows_tot = kGuard + s.ntiles * 128 + kGuard;
  auto al = [](int x, int a) { return (x + a - 1) / a * a; };
  int o = 0;
  s.oX = o;
  o = al(o + s.S * kCh * s.N * 4, 128);
  const int plane = s.rows_tot * 16;
  const int chunks = kCh * esz / 16;
  s.oP = o;
  o = al(o + chunks * plane, 128);
  s.oQ = o;
  o = al(o + chunks * plane, 128);
  s.oW = o;
  o = al(o + 9 * chunks * 256, 128);
  s.oBias = o;
  o += kCh * 4;
  s.oW0 = o;
  o += (9 * kCh + kCh) * 4;
  s.oHalo = o;
  o = al(o + s.NP * 2, 16);
  s.oNbr = o;
  o = al(o + s.N * 9 * 2, 16);
  s.oBar = o;
  o += 16;
  s.smem = o + 1024;  // slack for aligning the base to 1024 bytes
  uint32_t cols = 32;
  while (cols < (uint32_t)(s.ntiles * 16)) cols <<= 1;
  s.tmem_cols = cols;
  return s;
}

__device__ inline uint64_t desc_noswizzle(uint32_t saddr, uint32_t lbo_bytes, uint32_t sbo_bytes) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo_bytes >> 4) & 0x3FFFu) << 16;  // K-adjacent core matrices: one chunk plane apart
  d |= (uint64_t)((sbo_bytes >> 4) & 0x3FFFu) << 32;  // M/N-adjacent core matrices: 8 rows apart
  d |= (uint64_t)1 << 46;                             // descriptor version of tcgen05; layout 0 = no swizzle
  return d;
}

template <int KIND>
__device__ inline void mma_tc(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t accumulate) {
  if (KIND == 1) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(TcCfg<KIND>::idesc), "r"(accumulate));
  } else {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(TcCfg<KIND>::idesc), "r"(accumulate));
  }
}

__device__ inline void tmem_ld_16cols(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// TF32 operand value: round to nearest (ties away) on 10 mantissa bits; the MMA itself
// would drop the low 13 bits, a bias that accumulates through the residual stack
__device__ inline float to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// store one channel value of padded row m (absolute row index incl. guard) into a chunk-major buffer
template <int KIND>
__device__ inline void put(uint8_t* buf, int rows_tot, int m, int ch, float v) {
  using Cfg = TcCfg<KIND>;
  uint8_t* p = buf + (ch / Cfg::epc) * rows_tot * 16 + m * 16 + (ch % Cfg::epc) * Cfg::esz;
  if (KIND == 1)
    *reinterpret_cast<__nv_bfloat16*>(p) = __float2bfloat16_rn(v);
  else
    *reinterpret_cast<float*>(p) = to_tf32(v);
}

// halo rows of every sample repeat their periodic interior rows (all chunk planes)
template <int KIND>
__device__ inline void fill_halo(uint8_t* buf, const TcShape& sh, const int16_t* halo, int s_here) {
  using Cfg = TcCfg<KIND>;
  const int per = sh.NP * Cfg::chunks;
  for (int e = threadIdx.x; e < s_here * per; e += blockDim.x) {
    const int a = e / per, rem = e % per;
    const int p = rem / Cfg::chunks, c = rem % Cfg::chunks;
    const int src = halo[p];
    if (src == p) continue;
    const int base = kGuard + a * sh.NP;
    uint8_t* plane = buf + c * sh.rows_tot * 16;
    *reinterpret_cast<uint4*>(plane + (base + p) * 16) = *reinterpret_cast<const uint4*>(plane + (base + src) * 16);
  }
}

// W_smem[tap][chunk][n][epc] from the FP32 table slice [i][tap][o] (+ bias); channels >= C are zero
template <int KIND>
__device__ inline void stage_weights(uint8_t* wsm, float* bias, const float* tl, int C) {
  using Cfg = TcCfg<KIND>;
  const int total = 9 * Cfg::chunks * kCh * Cfg::epc;
  for (int e = threadIdx.x; e < total; e += blockDim.x) {
    const int tap = e / (Cfg::chunks * kCh * Cfg::epc);
    const int rem = e % (Cfg::chunks * kCh * Cfg::epc);
    const int c = rem / (kCh * Cfg::epc);
    const int n = (rem / Cfg::epc) % kCh;
    const int k = rem % Cfg::epc;
    const int i = c * Cfg::epc + k;
    const float w = (i < C && n < C) ? __ldg(tl + (i * 9 + tap) * C + n) : 0.0f;
    uint8_t* dst = wsm + ((tap * Cfg::chunks + c) * kCh + n) * 16 + k * Cfg::esz;
    if (KIND == 1)
      *reinterpret_cast<__nv_bfloat16*>(dst) = __float2bfloat16_rn(w);
    else
      *reinterpret_cast<float*>(dst) = to_tf32(w);
  }
  for (int o = threadIdx.x; o < kCh; o += blockDim.x) bias[o] = o < C ? __ldg(tl + C * 9 * C + o) : 0.0f;
}

__device__ inline int padded_row(int r, int L) { return (r / L + 1) * (L + 2) + (r % L) + 1; }

template <int KIND>
__global__ void __launch_bounds__(kThreadsTc, 1)
    rc_forward_tc_kernel(const float* __restrict__ table, TcShape sh, const uint32_t* __restrict__ cfg, int64_t ncfg,
                         const int64_t* __restrict__ n_live, float2* __restrict__ out, int32_t* __restrict__ status) {
  using Cfg = TcCfg<KIND>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  float* X = reinterpret_cast<float*>(sm + sh.oX);
  uint8_t* P = sm + sh.oP;
  uint8_t* Q = sm + sh.oQ;
  uint8_t* W = sm + sh.oW;
  float* bias = reinterpret_cast<float*>(sm + sh.oBias);
  float* W0 = reinterpret_cast<float*>(sm + sh.oW0);
  int16_t* halo = reinterpret_cast<int16_t*>(sm + sh.oHalo);
  int16_t* nbr = reinterpret_cast<int16_t*>(sm + sh.oNbr);
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + sh.oBar);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + sh.oBar + 8);
  __shared__ int fail;

  const int L = sh.L, N = sh.N, Lp = sh.Lp, NP = sh.NP, S = sh.S, nw = words_for(N);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int plane = sh.rows_tot * 16;

  for (int p = threadIdx.x; p < NP; p += blockDim.x) {
    const int py = p / Lp, px = p % Lp;
    const int sy = (py - 1 + L) % L, sx = (px - 1 + L) % L;
    halo[p] = (int16_t)((sy + 1) * Lp + sx + 1);
  }
  for (int e = threadIdx.x; e < N * 9; e += blockDim.x) {
    const int r = e / 9, t = e % 9, y = r / L, x = r % L;
    nbr[e] = (int16_t)(((y + t / 3 - 1 + L) % L) * L + (x + t % 3 - 1 + L) % L);
  }
  // guard rows and both buffers start zeroed (rows outside any sample stay finite)
  for (int e = threadIdx.x; e < Cfg::chunks * plane / 16; e += blockDim.x) {
    reinterpret_cast<uint4*>(P)[e] = make_uint4(0, 0, 0, 0);
    reinterpret_cast<uint4*>(Q)[e] = make_uint4(0, 0, 0, 0);
  }
  for (int e = threadIdx.x; e < 10 * kCh; e += blockDim.x) {
    const int t = e / kCh, o = e % kCh;  // t = 9: bias
    W0[e] = o < sh.C ? __ldg(table + t * sh.C + o) : 0.0f;
  }
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(sh.tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  uint32_t phase = 0;

  // one convolution with C input channels from buffer `in`: accumulate every tile in TMEM
  auto conv_tc = [&](const uint8_t* in) -> bool {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x == 0) {
      const uint32_t ib = smem_u32(in), wb = smem_u32(W);
      for (int j = 0; j < sh.ntiles; ++j) {
        const int row0 = kGuard + j * 128;
        for (int t = 0; t < 9; ++t) {
          const int off = (t / 3 - 1) * Lp + (t % 3 - 1);
#pragma unroll
          for (int q = 0; q < Cfg::mma_per_tap; ++q) {
            const uint64_t da = desc_noswizzle(ib + (uint32_t)((row0 + off) * 16 + 2 * q * plane), (uint32_t)plane, 128);
            const uint64_t db = desc_noswizzle(wb + (uint32_t)((t * Cfg::chunks + 2 * q) * 256), 256, 128);
            mma_tc<KIND>(tmem + (uint32_t)(16 * j), da, db, (t > 0 || q > 0) ? 1u : 0u);
          }
        }
      }
      mma_commit(bar);
    }
    const bool ok = mbar_wait(bar, phase & 1u);
    phase++;
    if (!ok) fail = 1;
    __syncthreads();
    tc_fence_after();
    return fail == 0;
  };

  const int64_t total = n_live ? min(ncfg, *n_live) : ncfg;
  for (int64_t base = (int64_t)blockIdx.x * S; base < total && !fail; base += (int64_t)gridDim.x * S) {
    const int s_here = (int)(total - base < S ? total - base : S);
    __syncthreads();
    for (int e = threadIdx.x; e < S * N; e += blockDim.x) {
      const int a = e / N, r = e % N;
      float v = 0.0f;
      if (a < s_here) v = ((cfg[(base + a) * nw + (r >> 5)] >> (r & 31)) & 1u) ? 1.0f : -1.0f;
      for (int c = 0; c < kCh; ++c) X[(a * kCh + c) * N + r] = c < sh.C ? v : 0.0f;
    }
    __syncthreads();
    // block 0, conv1 (one input channel) on the CUDA cores: Q = gelu(conv(s / sqrt 2) + b1)
    for (int e = threadIdx.x; e < s_here * N; e += blockDim.x) {
      const int a = e / N, r = e % N;
      float acc[kCh];
#pragma unroll
      for (int o = 0; o < kCh; ++o) acc[o] = W0[9 * kCh + o];
#pragma unroll
      for (int t = 0; t < 9; ++t) {
        const float v = X[(a * kCh) * N + nbr[r * 9 + t]] * 0.70710678118654752f;
#pragma unroll
        for (int o = 0; o < kCh; ++o) acc[o] = fmaf(v, W0[t * kCh + o], acc[o]);
      }
      const int m = kGuard + a * NP + padded_row(r, L);
#pragma unroll
      for (int o = 0; o < kCh; ++o) put<KIND>(Q, sh.rows_tot, m, o, gelu_tanh(acc[o]));
    }
    __syncthreads();
    fill_halo<KIND>(Q, sh, halo, s_here);
    for (int b = 0; b < sh.B; ++b) {
      if (b > 0) {
        // P = gelu(x / sqrt(b + 1)), conv1 on the tensor cores, Q = gelu(acc + b1)
        const float scale = rsqrtf((float)(b + 1));
        __syncthreads();
        for (int e = threadIdx.x; e < s_here * kCh * N; e += blockDim.x) {
          const int a = e / (kCh * N), rem = e % (kCh * N), c = rem / N, r = rem % N;
          put<KIND>(P, sh.rows_tot, kGuard + a * NP + padded_row(r, L), c, gelu_tanh(X[e] * scale));
        }
        __syncthreads();
        fill_halo<KIND>(P, sh, halo, s_here);
        stage_weights<KIND>(W, bias, table + layer_offset(2 * b, sh.C), sh.C);
        if (!conv_tc(P)) break;
        for (int j = 0; j < sh.ntiles; ++j) {
          float v[16];
          tmem_ld_16cols(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(16 * j), v);
          const int m = j * 128 + threadIdx.x, a = m / NP, p = m % NP, py = p / Lp, px = p % Lp;
          if (a < s_here && py >= 1 && py <= L && px >= 1 && px <= L) {
#pragma unroll
            for (int o = 0; o < kCh; ++o) put<KIND>(Q, sh.rows_tot, kGuard + m, o, gelu_tanh(v[o] + bias[o]));
          }
        }
        tc_fence_before();
        __syncthreads();
        fill_halo<KIND>(Q, sh, halo, s_here);
      }
      // conv2 on the tensor cores, x += acc + b2
      stage_weights<KIND>(W, bias, table + layer_offset(2 * b + 1, sh.C), sh.C);
      if (!conv_tc(Q)) break;
      for (int j = 0; j < sh.ntiles; ++j) {
        float v[16];
        tmem_ld_16cols(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(16 * j), v);
        const int m = j * 128 + threadIdx.x, a = m / NP, p = m % NP, py = p / Lp, px = p % Lp;
        if (a < s_here && py >= 1 && py <= L && px >= 1 && px <= L) {
          const int r = (py - 1) * L + (px - 1);
#pragma unroll
          for (int o = 0; o < kCh; ++o) X[(a * kCh + o) * N + r] += v[o] + bias[o];
        }
      }
      tc_fence_before();
      __syncthreads();
    }
    if (fail) break;
    // log sum exp over (channel, site) per sample, one warp per sample
    const float fs = rsqrtf((float)(sh.B + 1));
    const int cp = sh.cplx ? sh.C / 2 : sh.C;
    for (int a = warp; a < s_here; a += kThreadsTc / 32) {
      const float* xa = X + a * kCh * N;
      float mx = -INFINITY;
      for (int e = lane; e < cp * N; e += 32) mx = fmaxf(mx, xa[e] * fs);
      mx = warp_max(mx);
      float sr = 0.0f, si = 0.0f;
      for (int e = lane; e < cp * N; e += 32) {
        const float ex = expf(xa[e] * fs - mx);
        float sn = 0.0f, cs = 1.0f;
        if (sh.cplx) sincosf(xa[cp * N + e] * fs, &sn, &cs);
        sr = fmaf(ex, cs, sr);
        si = fmaf(ex, sn, si);
      }
      sr = warp_sum(sr);
      si = warp_sum(si);
      if (lane == 0)
        out[base + a] = make_float2(mx + 0.5f * logf(sr * sr + si * si) - logf((float)(cp * N)), atan2f(si, sr));
    }
  }
  if (fail && threadIdx.x == 0 && status) atomicExch(status, QGX_ERR_TIMEOUT);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(sh.tmem_cols) : "memory");
  }
}

}  // namespace

int rc_launch_forward_tc(const float* table, int L, int B, int C, bool cplx, const uint32_t* cfg, int64_t ncfg,
                         const int64_t* n_live, float2* out, int kind, cudaStream_t st) {
  if (C < 1 || C > kCh || L < 3 || L + 3 > kGuard || (L + 2) * (L + 2) > 1152) return QGX_ERR_UNSUPPORTED;
  const TcShape sh = tc_shape(L, B, C, cplx, kind == 1 ? 2 : 4, tc_samples_per_cta(L));
  if (sh.smem > device_max_smem_optin() || sh.tmem_cols > 512) return QGX_ERR_UNSUPPORTED;
  const int64_t want = (ncfg + sh.S - 1) / sh.S;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(device_sm_count(), want));
  if (kind == 1) {
    auto k = rc_forward_tc_kernel<1>;
    QGX_CHECK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, sh.smem));
    k<<<grid, kThreadsTc, sh.smem, st>>>(table, sh, cfg, ncfg, n_live, out, nullptr);
  } else {
    auto k = rc_forward_tc_kernel<0>;
    QGX_CHECK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, sh.smem));
    k<<<grid, kThreadsTc, sh.smem, st>>>(table, sh, cfg, ncfg, n_live, out, nullptr);
  }
  return launch_status();
}

}  // namespace qgx
