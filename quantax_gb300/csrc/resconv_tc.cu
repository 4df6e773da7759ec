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
// columns each) and one commit signals the layer.
//
// Threads: three warpgroups; thread t owns TMEM lane t % 128 of the tiles j = t / 128,
// t / 128 + 3, ... (at most three), i.e. the same padded rows in every layer, so the FP32
// residual stream of those rows lives in its registers. The epilogue of a convolution
// reads the accumulator row, applies bias and GELU (or the residual add followed by the
// next block's pre-activation) and writes the packed 16-byte chunks of the row and of its
// periodic halo copies. Layer weights come from a pre-converted image in the parameter
// table, fetched one layer ahead with cp.async.bulk into a double buffer.
#include <cuda_bf16.h>

#include <algorithm>

#include "qgx_common.cuh"
#include "qgx_resconv.cuh"
#include "qgx_tc.cuh"

namespace qgx {
namespace {

constexpr int kMaxTiles = 9;  // 128-row tiles per CTA
constexpr int kCh = kTcCh;
// launch shapes of the library's forward (warpgroups, tile rows per thread, CTAs per SM),
// from timings on GB300 at L = 10, 16 channels
template <int KIND>
struct TcLaunch;
template <>
struct TcLaunch<1> {
  static constexpr int WG = 2, RPT = 2, CTAS = 3;
};
template <>
struct TcLaunch<0> {
  static constexpr int WG = 2, RPT = 2, CTAS = 2;
};
constexpr int kGuard = 32;

template <int KIND>  // 1: bf16, 0: tf32
struct TcCfg {
  static constexpr int esz = KIND == 1 ? 2 : 4;
  static constexpr int epc = 16 / esz;            // elements per 16-byte chunk
  static constexpr int chunks = kCh / epc;        // chunk planes of the 16 channels
  static constexpr int mma_per_tap = chunks / 2;  // an MMA covers 32 bytes of K
  static constexpr int layer_bytes = 9 * chunks * 256 + 64;
  static constexpr uint32_t fmt = KIND == 1 ? 1u : 2u;
  static constexpr uint32_t idesc = (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(kCh >> 3) << 17) |
                                    ((uint32_t)(128 >> 4) << 24);
};

struct TcShape {
  int L, N, Lp, NP, B, C, S, ntiles, rows_tot;
  bool cplx, sinhp1;
  int oP, oQ, oW, oBar;  // byte offsets in shared memory
  int wbuf;              // bytes between the two weight buffers
  int smem;
  uint32_t tmem_cols;
};

// samples per CTA: as many as fit in `tiles` 128-row tiles
inline int tc_samples_per_cta(int L, int tiles) { return std::max(1, std::min(32, tiles * 128 / ((L + 2) * (L + 2)))); }

inline TcShape tc_shape(int L, int B, int C, bool cplx, int esz, int S) {
  TcShape s;
  s.L = L;
  s.N = L * L;
  s.Lp = L + 2;
  s.NP = s.Lp * s.Lp;
  s.B = B;
  s.C = C;
  s.cplx = cplx;
  s.sinhp1 = false;
  s.S = S;
  s.ntiles = (S * s.NP + 127) / 128;
  s.rows_tot = kGuard + s.ntiles * 128 + kGuard;
  auto al = [](int x, int a) { return (x + a - 1) / a * a; };
  const int plane = s.rows_tot * 16, chunks = kCh * esz / 16;
  const int lb = (int)tc_layer_bytes(esz);
  int o = 0;
  s.oP = o;
  o = al(o + chunks * plane, 128);
  s.oQ = o;
  o = al(o + chunks * plane, 128);
  s.oW = o;
  s.wbuf = al(lb, 128);
  o += 2 * s.wbuf;
  s.oBar = o;
  o += 32;
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

__device__ inline void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
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

// GELU of a value that is next rounded to the operand type: BF16 keeps 8 bits, below the
// error of the hardware tanh (about 2^-11); TF32 uses the exponential form
__device__ inline float gelu_tanh_hw(float x) {
  const float k0 = 0.7978845608028654f;
  const float u = k0 * fmaf(0.044715f * x, x * x, x);
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(u));
  const float h = 0.5f * x;
  return fmaf(h, t, h);
}

template <int KIND>
__device__ inline float gelu_op(float x) {
  return KIND == 1 ? gelu_tanh_hw(x) : gelu_fast(x);
}

// The padded row of a thread's tile row: sample slot a, grid position (py, px); interior
// rows (1 <= py, px <= L) of live samples carry sites, the others are halo or padding.
struct RowPos {
  int a, py, px;
  bool live;
};

__device__ inline RowPos row_pos(int m, const TcShape& sh, int s_here) {
  RowPos r;
  r.a = m / sh.NP;
  const int p = m - r.a * sh.NP;
  r.py = p / sh.Lp;
  r.px = p - r.py * sh.Lp;
  r.live = r.a < s_here && r.py >= 1 && r.py <= sh.L && r.px >= 1 && r.px <= sh.L;
  return r;
}

// a live row packed in one register (a << 16 | py << 8 | px), -1 otherwise
__device__ inline int pack_pos(const RowPos& r) { return r.live ? (r.a << 16) | (r.py << 8) | r.px : -1; }
__device__ inline RowPos unpack_pos(int v) { return RowPos{v >> 16, (v >> 8) & 255, v & 255, v >= 0}; }

// Write the 16 channel values of a live row as packed chunks, into the row and into each
// halo row that repeats it (one more row at a boundary, three at a corner).
template <int KIND>
__device__ inline void put_row(uint8_t* buf, const TcShape& sh, const RowPos& rp, const float (&val)[16]) {
  using Cfg = TcCfg<KIND>;
  uint4 ch[Cfg::chunks];
  if (KIND == 1) {
#pragma unroll
    for (int c = 0; c < Cfg::chunks; ++c) {
      uint32_t w[4];
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        const __nv_bfloat162 b2 = __floats2bfloat162_rn(val[8 * c + 2 * h], val[8 * c + 2 * h + 1]);
        w[h] = *reinterpret_cast<const uint32_t*>(&b2);
      }
      ch[c] = make_uint4(w[0], w[1], w[2], w[3]);
    }
  } else {
#pragma unroll
    for (int c = 0; c < Cfg::chunks; ++c)
      ch[c] = make_uint4(__float_as_uint(to_tf32(val[4 * c])), __float_as_uint(to_tf32(val[4 * c + 1])),
                         __float_as_uint(to_tf32(val[4 * c + 2])), __float_as_uint(to_tf32(val[4 * c + 3])));
  }
  const int L = sh.L;
  const int y2 = rp.py == 1 ? L + 1 : (rp.py == L ? 0 : -1);
  const int x2 = rp.px == 1 ? L + 1 : (rp.px == L ? 0 : -1);
  const int base = kGuard + rp.a * sh.NP;
  const int plane = sh.rows_tot * 16;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int yy = (k & 2) ? y2 : rp.py, xx = (k & 1) ? x2 : rp.px;
    if (yy < 0 || xx < 0) continue;
    uint8_t* dst = buf + (size_t)(base + yy * sh.Lp + xx) * 16;
#pragma unroll
    for (int c = 0; c < Cfg::chunks; ++c) *reinterpret_cast<uint4*>(dst + c * plane) = ch[c];
  }
}

// The forward machinery of one CTA: shared-memory buffers, barriers, TMEM and the layer
// pipeline state that persists from one forward to the next (the weight prefetch runs across
// forwards). WG warpgroups, RPT tile rows per thread (tiles j = wg, wg + WG, ...).
template <int KIND, int WG, int RPT>
struct TcForward {
  using Cfg = TcCfg<KIND>;
  static constexpr int kThreads = 128 * WG;
  const TcShape& sh;
  const uint8_t* wimg;
  uint8_t *P, *Q, *W;
  uint64_t *mbar, *wbar;
  volatile int* fail;
  uint32_t tmem, tmem_lane;
  uint32_t lc = 0;                    // convolutions run by this CTA so far
  uint32_t w_issued = 0, w_done = 0;  // weight loads issued / waited for (thread 0)
  int tid, warp, lane, wg, row_in_tile, plane, nlayers;

  __device__ TcForward(const TcShape& shape, const uint8_t* weights, uint8_t* sm, volatile int* fail_flag)
      : sh(shape), wimg(weights), fail(fail_flag) {
    P = sm + sh.oP;
    Q = sm + sh.oQ;
    W = sm + sh.oW;
    mbar = reinterpret_cast<uint64_t*>(sm + sh.oBar);
    wbar = mbar + 1;  // two: one per weight buffer
    tid = threadIdx.x;
    warp = tid >> 5;
    lane = tid & 31;
    wg = tid >> 7;
    row_in_tile = tid & 127;
    plane = sh.rows_tot * 16;
    nlayers = 2 * sh.B;
  }

  // zeroed buffers, barriers, TMEM; the first layer's weights when the CTA has work
  __device__ void setup(uint8_t* sm, bool has_work) {
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + sh.oBar + 24);
    // P and Q start zeroed: guard and padding rows stay finite
    for (int e = tid; e < 2 * Cfg::chunks * plane / 16; e += blockDim.x)
      reinterpret_cast<uint4*>(P)[e] = make_uint4(0, 0, 0, 0);
    if (tid == 0) {
      mbar_init(mbar, 1);
      mbar_init(wbar, 1);
      mbar_init(wbar + 1, 1);
      *fail = 0;
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
    tmem = *tmem_slot;
    tmem_lane = (uint32_t)(32 * (warp & 3)) << 16;
    if (tid == 0 && has_work) {
      mbar_expect_tx(wbar, Cfg::layer_bytes);
      bulk_load(W, wimg, Cfg::layer_bytes, wbar);
      w_issued = 1;
    }
  }

  // one convolution of the buffer `in` into TMEM (all tiles); false once a wait timed out
  __device__ bool conv(const uint8_t* in, bool more_after) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    const int buf = lc & 1;
    if (tid == 0) {
      tc_fence_after();
      if (!mbar_wait(wbar + buf, (lc >> 1) & 1)) {
        *fail = 1;
      } else {
        w_done = lc + 1;
        // descriptors advance in 16-byte units of the start-address field (addresses stay
        // below 256 KB, so the additions never leave the 14-bit field)
        const uint64_t da0 = desc_noswizzle(smem_u32(in) + kGuard * 16, (uint32_t)plane, 128);
        const uint64_t db0 = desc_noswizzle(smem_u32(W + buf * sh.wbuf), 256, 128);
        // tile-major: a tile's nine taps back to back (measured on GB300: issuing tap-major,
        // alternating accumulators, is 12% slower; the taps of one tile read nearly the same rows)
        for (int j = 0; j < sh.ntiles; ++j) {
          const uint64_t daj = da0 + (uint64_t)(j * 128);
          const uint32_t dj = tmem + (uint32_t)(16 * j);
#pragma unroll
          for (int t = 0; t < 9; ++t) {
            const int off = (t / 3 - 1) * sh.Lp + (t % 3 - 1);
#pragma unroll
            for (int q = 0; q < Cfg::mma_per_tap; ++q)
              mma_tc<KIND>(dj, daj + (uint64_t)(int64_t)(off + 2 * q * sh.rows_tot),
                           db0 + (uint64_t)((t * Cfg::chunks + 2 * q) * 16), (t > 0 || q > 0) ? 1u : 0u);
          }
        }
        mma_commit(mbar);
        if (more_after) {  // next layer's weights into the other buffer (its last reader has finished)
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          mbar_expect_tx(wbar + (buf ^ 1), Cfg::layer_bytes);
          bulk_load(W + (buf ^ 1) * sh.wbuf, wimg + (size_t)((lc + 1) % nlayers) * Cfg::layer_bytes,
                    Cfg::layer_bytes, wbar + (buf ^ 1));
          w_issued = lc + 2;
        }
      }
    }
    // thread 0 waits for the commit; the others wait at the barrier without taking issue
    // slots from the other CTAs on the SM
    if (tid == 0 && !*fail && !mbar_wait(mbar, lc & 1)) *fail = 1;
    __syncthreads();
    ++lc;
    tc_fence_after();
    return *fail == 0;
  }

  // log psi of s_here configurations (packed words, row stride nw words; global or shared
  // memory) into out[0 .. s_here); more_after: another forward follows in this CTA. Returns
  // false (the same in every thread) once a wait has timed out.
  __device__ bool forward(const uint32_t* cfg, int s_here, bool more_after, float2* out) {
    const int L = sh.L, N = sh.N, nw = words_for(N);
    float x[RPT][16];  // residual stream of this thread's rows
    int pos[RPT];      // packed RowPos of those rows
    // x = s on the C channels; P = s / sqrt 2 on channel 0 (block 0's conv1 has one input channel)
#pragma unroll
    for (int k = 0; k < RPT; ++k) {
      const int j = wg + WG * k;
      pos[k] = j < sh.ntiles ? pack_pos(row_pos(j * 128 + row_in_tile, sh, s_here)) : -1;
      const RowPos rp = unpack_pos(pos[k]);
      if (!rp.live) continue;
      const int r = (rp.py - 1) * L + (rp.px - 1);
      const float sv = ((cfg[rp.a * nw + (r >> 5)] >> (r & 31)) & 1u) ? 1.0f : -1.0f;
      float v[16];
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        x[k][c] = c < sh.C ? sv : 0.0f;
        v[c] = c == 0 ? sv * 0.70710678118654752f : 0.0f;
      }
      put_row<KIND>(P, sh, rp, v);
    }
    for (int b = 0; b < sh.B; ++b) {
      // conv1: Q = gelu(conv(P) + b1)
      if (!conv(P, true)) return false;
      {
        const float* bias = reinterpret_cast<const float*>(W + ((lc - 1) & 1) * sh.wbuf + 9 * Cfg::chunks * 256);
#pragma unroll
        for (int k = 0; k < RPT; ++k) {
          const int j = wg + WG * k;
          if (j >= sh.ntiles) break;
          float v[16];
          tmem_ld_16cols(tmem + tmem_lane + (uint32_t)(16 * j), v);
          const RowPos rp = unpack_pos(pos[k]);
          if (!rp.live) continue;
#pragma unroll
          for (int c = 0; c < 16; ++c) v[c] = gelu_op<KIND>(v[c] + bias[c]);
          put_row<KIND>(Q, sh, rp, v);
        }
      }
      // conv2: x += conv(Q) + b2; then the next block's P = gelu(x / sqrt(b + 2))
      if (!conv(Q, b + 1 < sh.B || more_after)) return false;
      {
        const float* bias = reinterpret_cast<const float*>(W + ((lc - 1) & 1) * sh.wbuf + 9 * Cfg::chunks * 256);
        const float scale = rsqrtf((float)(b + 2));
#pragma unroll
        for (int k = 0; k < RPT; ++k) {
          const int j = wg + WG * k;
          if (j >= sh.ntiles) break;
          float v[16];
          tmem_ld_16cols(tmem + tmem_lane + (uint32_t)(16 * j), v);
          const RowPos rp = unpack_pos(pos[k]);
          if (!rp.live) continue;
#pragma unroll
          for (int c = 0; c < 16; ++c) {
            x[k][c] += v[c] + bias[c];
            v[c] = gelu_op<KIND>(x[k][c] * scale);
          }
          if (b + 1 < sh.B) put_row<KIND>(P, sh, rp, v);
        }
      }
    }
    // log sum exp over (channel, site) per sample: z = x / sqrt(B + 1) of the C channels
    // is gathered in shared memory (over P and Q, free now), one warp per sample
    float* Z = reinterpret_cast<float*>(P);
    __syncthreads();
    const float fs = rsqrtf((float)(sh.B + 1));
#pragma unroll
    for (int k = 0; k < RPT; ++k) {
      const RowPos rp = unpack_pos(pos[k]);
      if (!rp.live) continue;
      const int r = (rp.py - 1) * L + (rp.px - 1);
#pragma unroll
      for (int c = 0; c < 16; ++c)
        if (c < sh.C) Z[(rp.a * sh.C + c) * N + r] = x[k][c] * fs;
    }
    __syncthreads();
    const int cp = sh.cplx ? sh.C / 2 : sh.C;
    for (int a = warp; a < s_here; a += kThreads / 32) {
      const float2 lp = rc_warp_log_psi(Z + a * sh.C * N, cp * N, 1.0f, sh.cplx, sh.sinhp1, lane);
      if (lane == 0) out[a] = lp;
    }
    __syncthreads();  // Z is overwritten by the next forward's P; out may be read next
    return true;
  }

  // after a timeout: a weight copy may still be in flight; give it the bounded wait before
  // the CTA exits, then release TMEM
  __device__ void teardown() {
    if (*fail && tid == 0 && w_issued > w_done) mbar_wait(wbar + (w_done & 1), (w_done >> 1) & 1);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
      tc_fence_after();
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(sh.tmem_cols) : "memory");
    }
  }
};

__device__ inline uint8_t* aligned_smem(uint8_t* raw) {
  return reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(raw) + 1023) & ~uintptr_t(1023));
}

// log psi of ncfg packed configurations (n_live, on the device, may cap the count), S per CTA
template <int KIND, int WG, int RPT, int MINB>
__global__ void __launch_bounds__(128 * WG, MINB)
    rc_forward_tc_kernel(const uint8_t* __restrict__ wimg, TcShape sh, const uint32_t* __restrict__ cfg,
                         int64_t ncfg, const int64_t* __restrict__ n_live, float2* __restrict__ out) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* sm = aligned_smem(smem_raw);
  __shared__ int fail;
  const int S = sh.S, nw = words_for(sh.N);
  const int64_t total = n_live ? min(ncfg, *n_live) : ncfg;
  TcForward<KIND, WG, RPT> f(sh, wimg, sm, &fail);
  f.setup(sm, (int64_t)blockIdx.x * S < total);
  int64_t base = (int64_t)blockIdx.x * S;
  for (; base < total; base += (int64_t)gridDim.x * S) {
    const int s_here = (int)(total - base < S ? total - base : S);
    const bool next_group = base + (int64_t)gridDim.x * S < total;
    if (!f.forward(cfg + base * nw, s_here, next_group, out + base)) break;
  }
  if (base < total) {
    // a wait timed out: this CTA's remaining outputs become NaN, so the failure shows in
    // every energy and update computed from them
    for (int64_t b2 = base; b2 < total; b2 += (int64_t)gridDim.x * S)
      for (int a = threadIdx.x; a < S && b2 + a < total; a += blockDim.x) out[b2 + a] = make_float2(NAN, NAN);
  }
  f.teardown();
}

// ---- warp-specialised forward (BF16, QGX_CONV_GROUPED) --------------------------------
// Measured on GB300 to be slower than TcForward's three CTAs per SM (1.13 against 0.82 ms for
// 16384 forwards at L = 10, 8 blocks, 16 channels): a single
// issuing thread gets about 115 clocks per N = 16 MMA, where three CTAs issuing side by side get
// about 47 between them. It runs on request, and its bit-identical results check TcForward.
// One CTA per SM holds kWsGroups independent sample groups: each group has the S samples and
// ntiles tiles of a TcShape, its own P and Q buffers, its own TMEM accumulator columns and two
// barriers (`full`: the group's convolution has finished, signalled by tcgen05.commit;
// `ready`: the group's 256 epilogue threads have written the next convolution's input). One
// MMA warp serves the groups in whatever order they become ready, so the tensor core works
// on one group's layer while the other groups run their epilogues; the weights of every
// layer stay resident in shared memory, loaded once per CTA. The epilogue arithmetic, the
// halo-padded layout and the log-sum-exp are those of TcForward.
// G groups of WG warpgroups, RPT tile rows per thread (a group holds up to WG * RPT tiles)
template <int G, int WG, int RPT>
struct WsCfg {
  static constexpr int kGroupThreads = 128 * WG;
  static constexpr int kMmaWarp = G * kGroupThreads / 32;
  static constexpr int kThreads = G * kGroupThreads + 32;
};
// the launch shape (G = 3 groups of 3 samples at L = 10: the per-layer-synchronous kernel's
// three CTAs per SM, in one CTA)
constexpr int kWsG = 3, kWsWG = 2, kWsRPT = 2;

struct WsShape {
  TcShape sh;   // one group's shape (its own buffer offsets are not used)
  int lb;       // bytes of one layer's weight image
  int oG;       // byte offset of group 0's P and Q; group g at oG + g * gbytes
  int gbytes;   // P and Q of one group
  int oBar;     // barriers, TMEM slot, failure flag
  int smem;
  uint32_t tmem_cols;
};

// false when the shape does not fit (shared memory, TMEM, the log-sum-exp scratch)
template <int G, int WG, int RPT>
inline bool ws_shape(int L, int B, int C, bool cplx, WsShape* w) {
  constexpr int tiles = WG * RPT;
  if ((L + 2) * (L + 2) > tiles * 128) return false;
  w->sh = tc_shape(L, B, C, cplx, 2, tc_samples_per_cta(L, tiles));
  const TcShape& sh = w->sh;
  if (sh.ntiles > tiles) return false;
  auto al = [](int x, int a) { return (x + a - 1) / a * a; };
  w->lb = (int)tc_layer_bytes(2);
  const int plane = sh.rows_tot * 16;
  w->oG = al(2 * B * w->lb, 128);
  w->gbytes = al(2 * 2 * plane, 128);  // P and Q, two 16-byte chunk planes each
  w->oBar = w->oG + G * w->gbytes;
  w->smem = w->oBar + 64 + 1024;
  uint32_t cols = 32;
  while (cols < (uint32_t)(G * sh.ntiles * 16)) cols <<= 1;
  w->tmem_cols = cols;
  return w->smem <= 227 * 1024 && w->smem <= device_max_smem_optin() && cols <= 512 &&
         sh.S * sh.C * sh.N * 4 <= w->gbytes;
}

// non-blocking probe of an mbarrier phase
__device__ inline bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ inline void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ inline void group_sync(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }

// barrier over the group's threads that also ORs a flag across them (the same result in all)
__device__ inline bool group_sync_or(int id, int n, bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\t"
      "bar.red.or.pred q, %2, %3, p;\n\tselp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(id), "r"(n)
      : "memory");
  return r != 0;
}

template <int G, int WG, int RPT>
__global__ void __launch_bounds__(WsCfg<G, WG, RPT>::kThreads, 1)
    rc_forward_ws_kernel(const uint8_t* __restrict__ wimg, WsShape ws, const uint32_t* __restrict__ cfg,
                         int64_t ncfg, const int64_t* __restrict__ n_live, float2* __restrict__ out) {
  using Cfg = TcCfg<1>;
  constexpr int kWsGroups = G, kWsWG = WG, kWsRPT = RPT;
  constexpr int kWsGroupThreads = WsCfg<G, WG, RPT>::kGroupThreads, kWsMmaWarp = WsCfg<G, WG, RPT>::kMmaWarp;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* sm = aligned_smem(smem_raw);
  const TcShape& sh = ws.sh;
  uint8_t* W = sm;
  uint64_t* wbar = reinterpret_cast<uint64_t*>(sm + ws.oBar);
  uint64_t* full = wbar + 1;
  uint64_t* ready = full + kWsGroups;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(ready + kWsGroups);
  volatile int* fail = reinterpret_cast<volatile int*>(tmem_slot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int S = sh.S, nw = words_for(sh.N), nlayers = 2 * sh.B, plane = sh.rows_tot * 16;
  const int64_t total = n_live ? min(ncfg, *n_live) : ncfg;
  const int64_t stride = (int64_t)gridDim.x * kWsGroups * S;  // samples per round of all groups
  const bool any_work = (int64_t)blockIdx.x * kWsGroups * S < total;

  // zeroed activation buffers (guard and padding rows stay finite), barriers, TMEM, weights
  for (int e = tid; e < kWsGroups * ws.gbytes / 16; e += blockDim.x)
    reinterpret_cast<uint4*>(sm + ws.oG)[e] = make_uint4(0, 0, 0, 0);
  if (tid == 0) {
    mbar_init(wbar, 1);
    for (int g = 0; g < kWsGroups; ++g) {
      mbar_init(full + g, 1);
      mbar_init(ready + g, kWsGroupThreads / 32);  // one arrival per epilogue warp
    }
    *fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(ws.tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  if (tid == 0 && any_work) {
    mbar_expect_tx(wbar, (uint32_t)(nlayers * ws.lb));
    bulk_load(W, wimg, (uint32_t)(nlayers * ws.lb), wbar);
  }

  if (warp == kWsMmaWarp) {
    // ---- MMA warp: one elected lane issues every group's convolutions ----
    if (lane == 0 && any_work) {
      int64_t left[kWsGroups];
      uint32_t lc[kWsGroups];
      int layer[kWsGroups];
      uint64_t daP[kWsGroups], daQ[kWsGroups];  // A descriptors of each group's P and Q at row 0
#pragma unroll
      for (int g = 0; g < kWsGroups; ++g) {
        const int64_t b0 = ((int64_t)blockIdx.x * kWsGroups + g) * S;
        left[g] = b0 < total ? (total - b0 + stride - 1) / stride * nlayers : 0;
        lc[g] = 0;
        layer[g] = 0;
        const uint32_t pg = smem_u32(sm + ws.oG + g * ws.gbytes) + kGuard * 16;
        daP[g] = desc_noswizzle(pg, (uint32_t)plane, 128);
        daQ[g] = desc_noswizzle(pg + 2 * plane, (uint32_t)plane, 128);
      }
      if (!mbar_wait(wbar, 0)) *fail = 1;
      const uint64_t db_base = desc_noswizzle(smem_u32(W), 256, 128);
      uint64_t t_last = global_timer();
      while (!*fail) {
        bool pending = false, progressed = false;
#pragma unroll
        for (int g = 0; g < kWsGroups; ++g) {
          if (left[g] == 0) continue;
          pending = true;
          if (!mbar_test(ready + g, lc[g] & 1)) continue;
          tc_fence_after();
          const int l = layer[g];
          const uint64_t da0 = (l & 1) ? daQ[g] : daP[g];
          const uint64_t db0 = db_base + (uint64_t)((l * ws.lb) >> 4);
          const uint32_t d0 = tmem + (uint32_t)(g * sh.ntiles * 16);
          for (int j = 0; j < sh.ntiles; ++j) {  // tile-major, as in TcForward::conv
            const uint64_t daj = da0 + (uint64_t)(j * 128);
#pragma unroll
            for (int t = 0; t < 9; ++t) {
              const int off = (t / 3 - 1) * sh.Lp + (t % 3 - 1);
              mma_tc<1>(d0 + (uint32_t)(16 * j), daj + (uint64_t)(int64_t)off,
                        db0 + (uint64_t)(t * Cfg::chunks * 16), t > 0 ? 1u : 0u);
            }
          }
          mma_commit(full + g);
          layer[g] = l + 1 == nlayers ? 0 : l + 1;
          ++lc[g];
          --left[g];
          progressed = true;
        }
        if (!pending) break;
        if (progressed) {
          t_last = global_timer();
        } else if (global_timer() - t_last > kWaitLimitNs) {
          *fail = 1;
        }
      }
      // after a failure: no MMA may still run when TMEM is released
#pragma unroll
      for (int g = 0; g < kWsGroups; ++g)
        if (*fail && lc[g] > 0) mbar_wait(full + g, (lc[g] - 1) & 1);
    }
  } else {
    // ---- epilogue: the 256 threads of group g ----
    const int g = warp / (4 * kWsWG);
    const int tg = tid - g * kWsGroupThreads;
    const int wg = tg >> 7, row_in_tile = tg & 127;
    const uint32_t tl = tmem + (uint32_t)(g * sh.ntiles * 16) + ((uint32_t)(32 * (warp & 3)) << 16);
    uint8_t* P = sm + ws.oG + g * ws.gbytes;
    uint8_t* Q = P + 2 * plane;
    const int L = sh.L, N = sh.N;
    int64_t base = ((int64_t)blockIdx.x * kWsGroups + g) * S;
    bool bad = any_work && !mbar_wait(wbar, 0);  // the biases are read from the weight image
    uint32_t conv = 0;
    float x[kWsRPT][16];
    int pos[kWsRPT];
    // the input of a forward: x = s on the C channels; P = s / sqrt 2 on channel 0
    auto load_input = [&](int64_t b0) {
      const int s_here = (int)(total - b0 < S ? total - b0 : S);
      const uint32_t* c0 = cfg + b0 * nw;
#pragma unroll
      for (int k = 0; k < kWsRPT; ++k) {
        const int j = wg + kWsWG * k;
        pos[k] = j < sh.ntiles ? pack_pos(row_pos(j * 128 + row_in_tile, sh, s_here)) : -1;
        const RowPos rp = unpack_pos(pos[k]);
        if (!rp.live) continue;
        const int r = (rp.py - 1) * L + (rp.px - 1);
        const float sv = ((c0[rp.a * nw + (r >> 5)] >> (r & 31)) & 1u) ? 1.0f : -1.0f;
        float v[16];
#pragma unroll
        for (int c = 0; c < 16; ++c) {
          x[k][c] = c < sh.C ? sv : 0.0f;
          v[c] = c == 0 ? sv * 0.70710678118654752f : 0.0f;
        }
        put_row<1>(P, sh, rp, v);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(ready + g);
    };
    if (!bad && base < total) load_input(base);
    for (; base < total; base += stride) {
      for (int l = 0; l < nlayers && !bad; ++l) {
        if (!mbar_wait(full + g, conv & 1)) {
          bad = true;
          break;
        }
        ++conv;
        tc_fence_after();
        const int b = l >> 1;
        const float* bias = reinterpret_cast<const float*>(W + l * ws.lb + 9 * Cfg::chunks * 256);
        const float scale = rsqrtf((float)(b + 2));
#pragma unroll
        for (int k = 0; k < kWsRPT; ++k) {
          const int j = wg + kWsWG * k;
          if (j >= sh.ntiles) break;
          float v[16];
          tmem_ld_16cols(tl + (uint32_t)(16 * j), v);
          const RowPos rp = unpack_pos(pos[k]);
          if (!rp.live) continue;
          if ((l & 1) == 0) {  // conv1: Q = gelu(conv(P) + b1)
#pragma unroll
            for (int c = 0; c < 16; ++c) v[c] = gelu_op<1>(v[c] + bias[c]);
            put_row<1>(Q, sh, rp, v);
          } else {  // conv2: x += conv(Q) + b2; the next block's P = gelu(x / sqrt(b + 2))
#pragma unroll
            for (int c = 0; c < 16; ++c) {
              x[k][c] += v[c] + bias[c];
              v[c] = gelu_op<1>(x[k][c] * scale);
            }
            if (b + 1 < sh.B) put_row<1>(P, sh, rp, v);
          }
        }
        if (l + 1 < nlayers) {
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(ready + g);
        }
      }
      // the same decision in every thread of the group before its named barriers
      if (group_sync_or(1 + g, kWsGroupThreads, bad || *fail != 0)) {
        bad = true;
        break;
      }
      tc_fence_before();
      // log sum exp over (channel, site) per sample, z = x / sqrt(B + 1) gathered over P and Q
      // (all of this group's convolutions have finished, and the MMA warp reads them again
      // only after the next input has been written and signalled)
      const int s_here = (int)(total - base < S ? total - base : S);
      float* Z = reinterpret_cast<float*>(P);
      const float fs = rsqrtf((float)(sh.B + 1));
#pragma unroll
      for (int k = 0; k < kWsRPT; ++k) {
        const RowPos rp = unpack_pos(pos[k]);
        if (!rp.live) continue;
        const int r = (rp.py - 1) * L + (rp.px - 1);
#pragma unroll
        for (int c = 0; c < 16; ++c)
          if (c < sh.C) Z[(rp.a * sh.C + c) * N + r] = x[k][c] * fs;
      }
      group_sync(1 + g, kWsGroupThreads);
      const int cp = sh.cplx ? sh.C / 2 : sh.C;
      for (int a = tg >> 5; a < s_here; a += kWsGroupThreads / 32) {
        const float2 lp = rc_warp_log_psi(Z + a * sh.C * N, cp * N, 1.0f, sh.cplx, sh.sinhp1, lane);
        if (lane == 0) out[base + a] = lp;
      }
      group_sync(1 + g, kWsGroupThreads);  // Z is overwritten by the next input
      if (base + stride < total) load_input(base + stride);
    }
    if (bad) {
      // a wait timed out: this group's remaining outputs become NaN, so the failure shows in
      // every energy and update computed from them
      for (; base < total; base += stride)
        for (int a = tg; a < S && base + a < total; a += kWsGroupThreads) out[base + a] = make_float2(NAN, NAN);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ws.tmem_cols) : "memory");
  }
}

// weight images for the tensor-core kernels from the FP32 table slices
__global__ void rc_tc_image_kernel(float* __restrict__ table, int B, int C) {
  uint8_t* tb = reinterpret_cast<uint8_t*>(table);
  uint8_t* img_bf = tb + tc_image_offset(B, C, 1);
  uint8_t* img_tf = tb + tc_image_offset(B, C, 0);
  const int lb_bf = (int)tc_layer_bytes(2), lb_tf = (int)tc_layer_bytes(4);
  const int per_layer = 9 * kCh * kCh + kCh;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)2 * B * per_layer;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int l = (int)(e / per_layer), rem = (int)(e % per_layer);
    const int cin = layer_cin(l, C);
    const float* tl = table + layer_offset(l, C);
    if (rem >= 9 * kCh * kCh) {
      const int o = rem - 9 * kCh * kCh;
      const float bv = o < C ? tl[cin * 9 * C + o] : 0.0f;
      reinterpret_cast<float*>(img_bf + (size_t)l * lb_bf + 9 * 2 * 256)[o] = bv;
      reinterpret_cast<float*>(img_tf + (size_t)l * lb_tf + 9 * 4 * 256)[o] = bv;
      continue;
    }
    const int tap = rem / (kCh * kCh), i = (rem / kCh) % kCh, o = rem % kCh;
    const float w = (i < cin && o < C) ? tl[(i * 9 + tap) * C + o] : 0.0f;
    // [tap][chunk][o][e]: chunk = i / (elements per chunk), e = i % (elements per chunk)
    *reinterpret_cast<__nv_bfloat16*>(img_bf + (size_t)l * lb_bf + ((tap * 2 + i / 8) * kCh + o) * 16 + (i % 8) * 2) =
        __float2bfloat16_rn(w);
    *reinterpret_cast<float*>(img_tf + (size_t)l * lb_tf + ((tap * 4 + i / 4) * kCh + o) * 16 + (i % 4) * 4) =
        to_tf32(w);
  }
}

}  // namespace

int rc_prepare_tc_images(float* table, int B, int C, cudaStream_t st) {
  rc_tc_image_kernel<<<16, 256, 0, st>>>(table, B, C);
  return launch_status();
}

namespace {

template <int KIND, int WG, int RPT, int MINB>
int launch_tc_variant(const uint8_t* wimg, const TcShape& sh, const uint32_t* cfg, int64_t ncfg,
                      const int64_t* n_live, float2* out, cudaStream_t st) {
  auto k = rc_forward_tc_kernel<KIND, WG, RPT, MINB>;
  // MINB CTAs per SM: the launch bounds cap the registers for it, the shape's shared memory
  // and TMEM columns were checked against it; the dynamic shared memory requested is raised
  // so that no more than MINB CTAs (and their TMEM allocations) share an SM
  const int smem = std::max(sh.smem, std::min(device_max_smem_optin(), (227 * 1024) / (MINB + 1) + 1024));
  QGX_CHECK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  const int64_t want = (ncfg + sh.S - 1) / sh.S;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)device_sm_count() * MINB, want));
  k<<<grid, 128 * WG, smem, st>>>(wimg, sh, cfg, ncfg, n_live, out);
  return launch_status();
}

// shape of the tensor-core kernels for a launch configuration; false if unsupported
template <int KIND>
bool tc_launch_shape(int L, int B, int C, bool cplx, TcShape* sh) {
  using T = TcLaunch<KIND>;
  constexpr int tiles = T::WG * T::RPT;
  if ((L + 2) * (L + 2) > tiles * 128) return false;
  *sh = tc_shape(L, B, C, cplx, TcCfg<KIND>::esz, tc_samples_per_cta(L, tiles));
  return sh->ntiles <= tiles && sh->smem * T::CTAS <= 227 * 1024 && sh->smem <= device_max_smem_optin() &&
         sh->tmem_cols * T::CTAS <= 512;
}

// dynamic shared memory requested: raised so that no more than CTAS CTAs (and their TMEM
// allocations) share an SM
template <int KIND>
int tc_smem_request(const TcShape& sh) {
  return std::max(sh.smem, std::min(device_max_smem_optin(), (227 * 1024) / (TcLaunch<KIND>::CTAS + 1) + 1024));
}

// the warp-specialised BF16 forward; QGX_ERR_UNSUPPORTED when its shape does not fit
int launch_ws(const float* table, int L, int B, int C, bool cplx, bool sinhp1, const uint32_t* cfg, int64_t ncfg,
              const int64_t* n_live, float2* out, cudaStream_t st) {
  WsShape ws;
  if (!ws_shape<kWsG, kWsWG, kWsRPT>(L, B, C, cplx, &ws)) return QGX_ERR_UNSUPPORTED;
  ws.sh.sinhp1 = sinhp1;
  const uint8_t* wimg = reinterpret_cast<const uint8_t*>(table) + tc_image_offset(B, C, 1);
  auto k = rc_forward_ws_kernel<kWsG, kWsWG, kWsRPT>;
  QGX_CHECK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, ws.smem));
  const int64_t blocks = (ncfg + ws.sh.S - 1) / ws.sh.S;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(device_sm_count(), (blocks + kWsG - 1) / kWsG));
  k<<<grid, WsCfg<kWsG, kWsWG, kWsRPT>::kThreads, ws.smem, st>>>(wimg, ws, cfg, ncfg, n_live, out);
  return launch_status();
}

template <int KIND>
int launch_tc(const float* table, int L, int B, int C, bool cplx, bool sinhp1, const uint32_t* cfg, int64_t ncfg,
              const int64_t* n_live, float2* out, bool grouped, cudaStream_t st) {
  using T = TcLaunch<KIND>;
  if (KIND == 1 && grouped) {
    const int rc = launch_ws(table, L, B, C, cplx, sinhp1, cfg, ncfg, n_live, out, st);
    if (rc != QGX_ERR_UNSUPPORTED) return rc;
  }
  TcShape sh;
  if (!tc_launch_shape<KIND>(L, B, C, cplx, &sh)) return QGX_ERR_UNSUPPORTED;
  sh.sinhp1 = sinhp1;
  const uint8_t* wimg = reinterpret_cast<const uint8_t*>(table) + tc_image_offset(B, C, KIND);
  auto k = rc_forward_tc_kernel<KIND, T::WG, T::RPT, T::CTAS>;
  const int smem = tc_smem_request<KIND>(sh);
  QGX_CHECK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  const int64_t want = (ncfg + sh.S - 1) / sh.S;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)device_sm_count() * T::CTAS, want));
  k<<<grid, 128 * T::WG, smem, st>>>(wimg, sh, cfg, ncfg, n_live, out);
  return launch_status();
}

}  // namespace

int rc_launch_forward_tc(const float* table, int L, int B, int C, bool cplx, bool sinhp1, const uint32_t* cfg,
                         int64_t ncfg, const int64_t* n_live, float2* out, int kind, bool grouped, cudaStream_t st) {
  if (C < 1 || C > kCh || L < 3 || L + 3 > kGuard) return QGX_ERR_UNSUPPORTED;
  if (kind == 1) return launch_tc<1>(table, L, B, C, cplx, sinhp1, cfg, ncfg, n_live, out, grouped, st);
  return launch_tc<0>(table, L, B, C, cplx, sinhp1, cfg, ncfg, n_live, out, false, st);
}

}  // namespace qgx
