// ResConv kernels (quantax/model/conv_nets.py:26-183): batched forward over packed
// configurations, the SpinExchange Metropolis step (propose / accept) and local energies
// over compacted connected configurations.
//
// Network: x0 = s repeated over C channels (block 0's residual is repeated over the
// channels, conv_nets.py:88-91); per block b:
//   P = x / sqrt(b+1) (/ sqrt 2 in block 0, else gelu), Q = gelu(conv1(P) + b1),
//   x += conv2(Q) (+ b2 except in the last block);
// final z = x / sqrt(B+1), complex output z_c + i z_{c+C/2} (pair_cpl), and
// log psi = logsumexp(z) - log(C' N) (exp_by_scale + ConvSymmetrize over translations).
// Convolutions: 3x3, circular, cross-correlation. gelu: tanh approximation.
//
// Work layout of the FP32 forward: one CTA holds S samples' activations (three C x N buffers
// per sample) and the current layer's weights in shared memory. In the site order a thread
// computes all C output channels of two sites of one sample; in the blocked order (even L, see
// rc_blocked_site) it computes 8 (or 4) output channels of a 2 x 2 block of sites. Threads of a
// warp share their output channels, so every weight load is a warp-wide broadcast.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "qgx_common.cuh"
#include "qgx_resconv.cuh"

namespace qgx {
namespace {

constexpr int kFwdThreads = 256;
constexpr int kFwdSPT = 2;      // sites per thread in the FP32 convolutions
constexpr int kFwdSamples = 5;  // samples per CTA: 5 x 50 site pairs fill 256 threads at L = 10
constexpr int kMaxSitesConv = 256;  // L <= 16

struct ConvNet {
  int L, N, B, C;
  bool cplx;
  int prec;     // QGX_CONV_*: arithmetic of the forward convolutions
  bool sinhp1;  // final activation sinhp1_by_scale instead of exp_by_scale
  bool grouped;  // QGX_CONV_GROUPED: the warp-specialised BF16 kernel
  // rbm_m > 0: not a ResConv but RBM_Dense with rbm_m hidden units on N sites (the symmetrised
  // pipelines below evaluate its images T_g s); rbm_vbias: its table holds a visible bias
  int rbm_m = 0;
  int rbm_vbias = 0;
};

inline ConvNet make_rbm_net(int n, int m, int has_vbias) {
  ConvNet net{0, n, 0, 0, false, QGX_CONV_FP32, false, false};
  net.rbm_m = m;
  net.rbm_vbias = has_vbias != 0;
  return net;
}

// the complex_out argument of the entry points: QGX_RESCONV_COMPLEX | QGX_RESCONV_SINHP1
inline ConvNet make_net(int L, int B, int C, int out_flags, int prec) {
  return ConvNet{L, L * L, B, C, (out_flags & QGX_RESCONV_COMPLEX) != 0, prec & ~QGX_CONV_GROUPED,
                 (out_flags & QGX_RESCONV_SINHP1) != 0, (prec & QGX_CONV_GROUPED) != 0};
}

__host__ __device__ inline int64_t nparams_rc(int B, int C) {
  // reference ravel order: per block conv1.weight, conv1.bias, conv2.weight, conv2.bias (not in the last block)
  int64_t n = 0;
  for (int b = 0; b < B; ++b) {
    n += (int64_t)C * layer_cin(2 * b, C) * 9 + C;
    n += (int64_t)C * C * 9 + (b == B - 1 ? 0 : C);
  }
  return n;
}

// params (reference order) -> table
__global__ void rc_prepare_kernel(const float* __restrict__ params, int B, int C, float* __restrict__ table) {
  int64_t pofs = 0;
  for (int l = 0; l < 2 * B; ++l) {
    const int cin = layer_cin(l, C);
    const bool has_bias = !(l == 2 * B - 1);
    const int64_t toff = layer_offset(l, C);
    const int64_t nw = (int64_t)C * cin * 9;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nw; e += (int64_t)gridDim.x * blockDim.x) {
      // params weight layout (o, i, ky, kx) -> table (i, tap, o)
      const int o = (int)(e / (cin * 9));
      const int rem = (int)(e % (cin * 9));
      const int i = rem / 9, tap = rem % 9;
      table[toff + ((int64_t)i * 9 + tap) * C + o] = params[pofs + e];
    }
    for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < C; o += gridDim.x * blockDim.x)
      table[toff + (int64_t)cin * 9 * C + o] = has_bias ? params[pofs + nw + o] : 0.0f;
    pofs += nw + (has_bias ? C : 0);
  }
}

__device__ inline void stage_floats(float* dst, const float* src, int64_t n) {
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) dst[e] = __ldg(src + e);
}

// Floats between consecutive samples' activations in the forward's shared memory: C N padded to
// G modulo 32, G the work items per sample (site groups ceil(N / kFwdSPT) in site order, 2 x 2
// blocks N / 4 in blocked order), so that item a G + g (sample a, group or block g) falls in
// bank (a G + g) mod 32 and a warp whose 32 consecutive items span two samples touches 32
// different banks (with a stride of C N, a multiple of 32 at L = 10, the two samples' items
// collide on up to 16 banks).
__host__ __device__ inline int rc_sample_stride(int C, int N, bool blocked) {
  const int G = blocked ? N / 4 : (N + kFwdSPT - 1) / kFwdSPT;
  return C * N + (((G - C * N) % 32) + 32) % 32;
}

// Blocked site order of the FP32 forward at even L: the lattice is cut into N / 4 blocks of
// 2 x 2 sites, block (by, bx) = by L/2 + bx, and site (y, x) of a channel plane is stored at
// ((y & 1) 2 + (x & 1)) N/4 + block: four planes of N / 4 floats, one per position in the block.
// A thread then owns the four sites of one block; for a fixed tap, the 32 lanes of a warp read
// 32 different blocks of one plane (consecutive addresses up to the periodic wrap).
__host__ __device__ inline int rc_blocked_site(int y, int x, int L) {
  return ((y & 1) * 2 + (x & 1)) * (L * L / 4) + (y >> 1) * (L / 2) + (x >> 1);
}

// floats before the layer weights in the forward's shared memory: the three activation buffers,
// rounded up to a multiple of 4 (the sample stride need not be one)
__host__ __device__ inline int64_t rc_weights_offset(int S, int SS) { return (3LL * S * SS + 3) / 4 * 4; }

// c += a * b on a pair of floats with one packed FP32 instruction (each lane is an IEEE fma,
// the same result as two fmaf calls, in half the issue slots)
__device__ inline void fma_pair(float2& c, float2 a, float2 b) {
  unsigned long long cc, aa, bb;
  asm("mov.b64 %0, {%1, %2};" : "=l"(cc) : "f"(c.x), "f"(c.y));
  asm("mov.b64 %0, {%1, %2};" : "=l"(aa) : "f"(a.x), "f"(a.y));
  asm("mov.b64 %0, {%1, %2};" : "=l"(bb) : "f"(b.x), "f"(b.y));
  asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(cc) : "l"(aa), "l"(bb));
  asm("mov.b64 {%0, %1}, %2;" : "=f"(c.x), "=f"(c.y) : "l"(cc));
}

// out[a][o][r] = act(sum_{i,tap} W[i][tap][o] in[a][i][nbr(r,tap)] + bias[o]); mode 0: gelu and store,
// mode 1: accumulate into out (residual add). A thread computes the C outputs of SPT sites
// r = g + k G (G = ceil(N / SPT)), so consecutive threads gather consecutive sites (no bank
// conflicts) and every broadcast weight load feeds SPT x 4 FMAs, issued as packed pairs of
// output channels (fma.rn.f32x2).
template <int C, int SPT>
__device__ inline void conv_layer(const float* __restrict__ in, int cin, float* __restrict__ out,
                                  const float* __restrict__ w, const int16_t* __restrict__ nbr, int N, int S,
                                  int mode, int ss) {  // ss: floats between samples' activations
  const float* bias = w + cin * 9 * C;
  const int G = (N + SPT - 1) / SPT;
  for (int it = threadIdx.x; it < S * G; it += blockDim.x) {
    const int a = it / G, g = it - a * G;
    int r[SPT];
    int nb[SPT][9];
#pragma unroll
    for (int k = 0; k < SPT; ++k) {
      r[k] = g + k * G;
      const int rc = r[k] < N ? r[k] : N - 1;  // a site past the end reads a valid one, is not stored
#pragma unroll
      for (int t = 0; t < 9; ++t) nb[k][t] = nbr[rc * 9 + t];
    }
    float2 acc[SPT][C / 2];  // output channels (2 h, 2 h + 1)
#pragma unroll
    for (int k = 0; k < SPT; ++k)
#pragma unroll
      for (int h = 0; h < C / 2; ++h) acc[k][h] = make_float2(bias[2 * h], bias[2 * h + 1]);
    const float* ina = in + (int64_t)a * ss;
    for (int i = 0; i < cin; ++i) {
      const float* ini = ina + i * N;
#pragma unroll
      for (int t = 0; t < 9; ++t) {
        float2 v[SPT];
#pragma unroll
        for (int k = 0; k < SPT; ++k) {
          const float x = ini[nb[k][t]];
          v[k] = make_float2(x, x);
        }
        const float4* wp = reinterpret_cast<const float4*>(w + (i * 9 + t) * C);
#pragma unroll
        for (int o4 = 0; o4 < C / 4; ++o4) {
          const float4 ww = wp[o4];
#pragma unroll
          for (int k = 0; k < SPT; ++k) {
            fma_pair(acc[k][2 * o4], v[k], make_float2(ww.x, ww.y));
            fma_pair(acc[k][2 * o4 + 1], v[k], make_float2(ww.z, ww.w));
          }
        }
      }
    }
#pragma unroll
    for (int k = 0; k < SPT; ++k) {
      if (r[k] >= N) continue;
      float* oa = out + (int64_t)a * ss + r[k];
      if (mode == 0) {
#pragma unroll
        for (int h = 0; h < C / 2; ++h) {
          oa[2 * h * N] = gelu_tanh(acc[k][h].x);
          oa[(2 * h + 1) * N] = gelu_tanh(acc[k][h].y);
        }
      } else {
#pragma unroll
        for (int h = 0; h < C / 2; ++h) {
          oa[2 * h * N] += acc[k][h].x;
          oa[(2 * h + 1) * N] += acc[k][h].y;
        }
      }
    }
  }
}

// out[a][o][b] = act(sum_{i,tap} W[i][tap][o] in[a][i][b + tap] + bias[o]) in the blocked site
// order (rc_blocked_site), same modes as conv_layer. A thread computes CO output channels
// (group h of C / CO) of the four sites of one 2 x 2 block: per input channel it gathers the
// block's 4 x 4 input patch (16 loads; patch[k] = in[nbr[16 block + k]]) and per tap reads CO
// broadcast weights that feed 4 sites. Per multiply-add that is 0.6 times the shared-memory
// reads of conv_layer<C, 2> (34 against 54 per input channel for 144 packed FMAs). Each output
// sums bias, then input channels in order, taps in order: the same operations in the same
// order as conv_layer, so both give the same floats. Items of one channel group fill whole
// warps, so a warp's weight loads are broadcasts. In mode 1 with pnext, the updated residual x
// is also written as the next block's pre-activation pnext = gelu(x pscale) (the separate pass
// of the site-order kernel, the same floats). CIN > 0 fixes the input channel count at compile
// time (the C-channel layers); the input-channel loop is unrolled four times either way
// (measured: 2.77 ms per 16384 forwards at L = 10 against 2.93 without; eight and sixteen were
// slower).
template <int C, int CO, int CIN = 0>
__device__ inline void conv_layer_blocked(const float* __restrict__ in, int cin_rt, float* __restrict__ out,
                                          const float* __restrict__ w, const int16_t* __restrict__ nbr, int N,
                                          int S, int mode, int ss, float* __restrict__ pnext = nullptr,
                                          float pscale = 1.0f) {
  static_assert(C % CO == 0 && CO % 4 == 0, "output channel groups of 4k channels");
  constexpr int H = C / CO;
  const int cin = CIN > 0 ? CIN : cin_rt;
  const float* bias = w + cin * 9 * C;
  const int NB = N >> 2;
  const int items = S * NB;
  const int per = (items + 31) & ~31;  // items of one channel group, rounded to whole warps
  for (int it = threadIdx.x; it < H * per; it += blockDim.x) {
    const int h = it / per, j = it - h * per;
    if (j >= items) continue;
    const int a = j / NB, g = j - a * NB;
    const int o0 = h * CO;
    int nb[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) nb[k] = nbr[g * 16 + k];
    float2 acc[4][CO / 2];  // block position q = 2 py + px; output channels (o0 + 2 e, o0 + 2 e + 1)
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int e = 0; e < CO / 2; ++e) acc[q][e] = make_float2(bias[o0 + 2 * e], bias[o0 + 2 * e + 1]);
    const float* ina = in + (int64_t)a * ss;
#pragma unroll 4
    for (int i = 0; i < cin; ++i) {
      const float* ini = ina + i * N;
      float d[16];
#pragma unroll
      for (int k = 0; k < 16; ++k) d[k] = ini[nb[k]];
#pragma unroll
      for (int t = 0; t < 9; ++t) {
        const int dy = t / 3, dx = t % 3;
        const float4* wp = reinterpret_cast<const float4*>(w + (i * 9 + t) * C + o0);
#pragma unroll
        for (int o4 = 0; o4 < CO / 4; ++o4) {
          const float4 ww = wp[o4];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const float x = d[((q >> 1) + dy) * 4 + (q & 1) + dx];
            fma_pair(acc[q][2 * o4], make_float2(x, x), make_float2(ww.x, ww.y));
            fma_pair(acc[q][2 * o4 + 1], make_float2(x, x), make_float2(ww.z, ww.w));
          }
        }
      }
    }
    float* oa = out + (int64_t)a * ss + (int64_t)o0 * N + g;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      float* oq = oa + q * NB;
      if (mode == 0) {
#pragma unroll
        for (int e = 0; e < CO / 2; ++e) {
          oq[2 * e * N] = gelu_tanh(acc[q][e].x);
          oq[(2 * e + 1) * N] = gelu_tanh(acc[q][e].y);
        }
      } else if (pnext == nullptr) {
#pragma unroll
        for (int e = 0; e < CO / 2; ++e) {
          oq[2 * e * N] += acc[q][e].x;
          oq[(2 * e + 1) * N] += acc[q][e].y;
        }
      } else {
        float* pq = pnext + (oq - out);
#pragma unroll
        for (int e = 0; e < CO / 2; ++e) {
          const float x0 = oq[2 * e * N] + acc[q][e].x, x1 = oq[(2 * e + 1) * N] + acc[q][e].y;
          oq[2 * e * N] = x0;
          oq[(2 * e + 1) * N] = x1;
          pq[2 * e * N] = gelu_tanh(x0 * pscale);
          pq[(2 * e + 1) * N] = gelu_tanh(x1 * pscale);
        }
      }
    }
  }
}

// Asks L1 for the 128-byte lines of the n floats at src, one prefetch per line, every address
// inside [src, src + n). Issued for the next layer's weights before a convolution, so that the
// staging after it reads L1 rather than L2.
__device__ inline void prefetch_l1(const float* src, int64_t n) {
  const size_t a0 = __cvta_generic_to_global(src), a1 = __cvta_generic_to_global(src + n);
  for (size_t k = threadIdx.x;; k += blockDim.x) {
    const size_t a = k == 0 ? a0 : (a0 & ~size_t(127)) + 128 * k;
    if (a >= a1) break;
    asm volatile("prefetch.global.L1 [%0];" ::"l"(a));
  }
}

// 4 x 4 input patches of the 2 x 2 blocks (rows 2 by - 1 .. 2 by + 2, columns 2 bx - 1 .. 2 bx + 2,
// periodic) as blocked indices, and the blocked index of every site r = y L + x
__device__ inline void build_blocked_tables(int16_t* patch, int16_t* site, int L) {
  const int N = L * L, NB = N / 4, Lh = L / 2;
  for (int e = threadIdx.x; e < NB * 16; e += blockDim.x) {
    const int g = e >> 4, u = (e >> 2) & 3, v = e & 3;
    const int y = (2 * (g / Lh) - 1 + u + L) % L, x = (2 * (g % Lh) - 1 + v + L) % L;
    patch[e] = (int16_t)rc_blocked_site(y, x, L);
  }
  for (int r = threadIdx.x; r < N; r += blockDim.x) site[r] = (int16_t)rc_blocked_site(r / L, r % L, L);
}

__device__ inline void build_nbr(int16_t* nbr, int L) {
  const int N = L * L;
  for (int e = threadIdx.x; e < N * 9; e += blockDim.x) {
    const int r = e / 9, t = e % 9;
    const int y = r / L, x = r % L;
    const int dy = t / 3 - 1, dx = t % 3 - 1;
    nbr[e] = (int16_t)(((y + dy + L) % L) * L + (x + dx + L) % L);
  }
}

struct RcBlockedOrder {  // element c N + r of the site order -> its place in the blocked order
  const int16_t* site;
  int N;
  __device__ int operator()(int e) const {
    const int c = e / N;
    return c * N + site[e - c * N];
  }
};

// output channels per thread in conv_layer_blocked: 8 where C allows (two groups at C = 16)
template <int C>
constexpr int rc_blocked_co() { return C % 8 == 0 ? 8 : 4; }

// Forward of ncfg packed configurations (nw words each). n_live (device, may be NULL)
// caps the count at run time. out: (re, im) of log psi per configuration.
// BLK (even L): activations in the blocked site order and conv_layer_blocked; otherwise site
// order and conv_layer. Both give the same floats: every convolution output is the same chain
// of operations, and the final sum runs over the site order in both.
template <int C, bool BLK>
__global__ void __launch_bounds__(kFwdThreads, 2)
    rc_forward_kernel(const float* __restrict__ table, ConvNet net, const uint32_t* __restrict__ cfg, int64_t ncfg,
                      const int64_t* __restrict__ n_live, float2* __restrict__ out, int S) {
  extern __shared__ float4 smem4[];
  float* sm = reinterpret_cast<float*>(smem4);
  const int N = net.N, nw = words_for(N);
  const int SS = rc_sample_stride(C, N, BLK);
  float* X = sm;
  float* P = X + (int64_t)S * SS;
  float* Q = P + (int64_t)S * SS;
  float* Wl = sm + rc_weights_offset(S, SS);  // 16-byte aligned: the weights are read as float4
  int16_t* nbr = reinterpret_cast<int16_t*>(Wl + C * 9 * C + C);
  int16_t* site = nbr + (BLK ? N * 4 : 0);  // blocked index of each site (BLK only)
  if (BLK)
    build_blocked_tables(nbr, site, net.L);
  else
    build_nbr(nbr, net.L);
  const int64_t total = n_live ? min(ncfg, *n_live) : ncfg;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t base = (int64_t)blockIdx.x * S; base < total; base += (int64_t)gridDim.x * S) {
    const int s_here = (int)(total - base < S ? total - base : S);
    __syncthreads();
    for (int e = threadIdx.x; e < S * N; e += blockDim.x) {
      const int a = e / N, r = e % N;
      float v = 0.0f;
      if (a < s_here) v = ((cfg[(base + a) * nw + (r >> 5)] >> (r & 31)) & 1u) ? 1.0f : -1.0f;
      const int k = BLK ? site[r] : r;
      for (int c = 0; c < C; ++c) X[(int64_t)a * SS + c * N + k] = v;
    }
    for (int b = 0; b < net.B; ++b) {
      const float scale = rsqrtf((float)(b + 1)) * (b == 0 ? 0.70710678118654752f : 1.0f);
      const int cin = b == 0 ? 1 : C;
      __syncthreads();
      if (!BLK || b == 0) {  // blocked: blocks b >= 1 get P from the previous block's second convolution
        for (int e = threadIdx.x; e < S * cin * N; e += blockDim.x) {
          const int a = e / (cin * N), rem = e % (cin * N);
          const float v = X[(int64_t)a * SS + rem] * scale;
          P[(int64_t)a * SS + rem] = b == 0 ? v : gelu_tanh(v);
        }
      }
      stage_floats(Wl, table + layer_offset(2 * b, C), layer_floats(2 * b, C));
      if (BLK) prefetch_l1(table + layer_offset(2 * b + 1, C), layer_floats(2 * b + 1, C));
      __syncthreads();
      if (BLK && cin == C)
        conv_layer_blocked<C, rc_blocked_co<C>(), C>(P, C, Q, Wl, nbr, N, S, 0, SS);
      else if (BLK)
        conv_layer_blocked<C, rc_blocked_co<C>()>(P, cin, Q, Wl, nbr, N, S, 0, SS);
      else
        conv_layer<C, kFwdSPT>(P, cin, Q, Wl, nbr, N, S, 0, SS);
      __syncthreads();
      stage_floats(Wl, table + layer_offset(2 * b + 1, C), layer_floats(2 * b + 1, C));
      // the next layer in order: the next block's first convolution, or block 0's for the next samples
      const int lnext = b + 1 < net.B ? 2 * b + 2 : 0;
      if (BLK) prefetch_l1(table + layer_offset(lnext, C), layer_floats(lnext, C));
      __syncthreads();
      if (BLK)
        conv_layer_blocked<C, rc_blocked_co<C>(), C>(Q, C, X, Wl, nbr, N, S, 1, SS, b + 1 < net.B ? P : nullptr,
                                                     rsqrtf((float)(b + 2)));
      else
        conv_layer<C, kFwdSPT>(Q, C, X, Wl, nbr, N, S, 1, SS);
    }
    __syncthreads();
    // log of the mean final activation over (channel, site) per sample, one warp per sample
    const float fs = rsqrtf((float)(net.B + 1));
    const int cp = net.cplx ? C / 2 : C;
    for (int a = warp; a < s_here; a += kFwdThreads / 32) {
      const float* za = X + (int64_t)a * SS;
      const float2 lp = BLK ? rc_warp_log_psi_at(za, cp * N, fs, net.cplx, net.sinhp1, lane, RcBlockedOrder{site, N})
                            : rc_warp_log_psi(za, cp * N, fs, net.cplx, net.sinhp1, lane);
      if (lane == 0) out[base + a] = lp;
    }
  }
}

// ---- SpinExchange step ----------------------------------------------------------------
// proposal of chain c at draw t: site i uniform among the hopping spins, j uniform in the
// padded neighbour row of i (-1: no move). Only proposals that change the configuration are
// evaluated (as the reference's chunked sweep does, sampler/metropolis.py:216-242): a changed
// one is appended to the compacted batch comp at an atomic position, recorded in comp_idx[c]
// (-1: unchanged); *n_live counts them. Every configuration's forward is independent of the
// others in its batch, so the order of the batch does not change any result.
__global__ void rc_propose_kernel(const uint32_t* __restrict__ spins, uint32_t* __restrict__ comp,
                                  int32_t* __restrict__ comp_idx, unsigned long long* __restrict__ n_live, int64_t ns,
                                  int n, uint64_t seed, const uint64_t* __restrict__ step_base, int t,
                                  const int32_t* __restrict__ nbr, int z, int hop, int proposal) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= ns) return;
  const uint64_t step = *step_base + (uint64_t)t;
  const int nw = words_for(n);
  uint32_t w[8];
  for (int k = 0; k < nw; ++k) w[k] = spins[c * nw + k];
  const u32x4 r = draw(seed, (uint64_t)c, step, kTagPropose);
  if (proposal == QGX_PROPOSAL_LOCAL_FLIP) {
    // LocalFlip (common_samplers.py:28-33): one uniform site, always a change
    const int k = (int)bounded(r.x, (uint32_t)n);
    w[k >> 5] ^= 1u << (k & 31);
  } else if (!propose_exchange(w, n, nw, r, nbr, z, hop)) {
    comp_idx[c] = -1;
    return;
  }
  const unsigned long long pos = atomicAdd(n_live, 1ull);
  for (int k = 0; k < nw; ++k) comp[pos * nw + k] = w[k];
  comp_idx[c] = (int32_t)pos;
}

// Metropolis test of the changed chains against their compacted log psi; thread 0 resets the
// live count for the next step (its forward has finished reading it)
__global__ void rc_accept_kernel(uint32_t* __restrict__ spins, float2* __restrict__ lp,
                                 const uint32_t* __restrict__ comp, const float2* __restrict__ lp_comp,
                                 const int32_t* __restrict__ comp_idx, unsigned long long* __restrict__ n_live,
                                 int32_t* __restrict__ accepts, int64_t ns, int n, uint64_t seed,
                                 const uint64_t* __restrict__ step_base, int t, float reweight) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c == 0) *n_live = 0ull;
  if (c >= ns) return;
  const int32_t idx = comp_idx[c];
  if (idx < 0) return;
  const uint64_t step = *step_base + (uint64_t)t;
  const u32x4 r = draw(seed, (uint64_t)c, step, kTagPropose);
  const float rhs = log1pf(-unit_float(r.y));
  if (reweight * (lp_comp[idx].x - lp[c].x) > rhs) {
    const int nw = words_for(n);
    for (int k = 0; k < nw; ++k) spins[c * nw + k] = comp[(int64_t)idx * nw + k];
    lp[c] = lp_comp[idx];
    if (accepts) accepts[c] += 1;
  }
}

// ---- local energies ----------------------------------------------------------------------
__device__ inline int bit_at(const uint32_t* s, int k) { return (int)((s[k >> 5] >> (k & 31)) & 1u); }

// number of connected configurations with a non-zero element per sample
__global__ void rc_conn_count_kernel(qgx_operator_t op, const uint32_t* __restrict__ spins, int64_t ns, int n,
                                     int64_t* __restrict__ counts) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= ns) return;
  const uint32_t* s = spins + c * words_for(n);
  int64_t k = 0;
  for (int t = 0; t < op.n_f1; ++t) k += op.f1_J[2 * t + bit_at(s, op.f1_i[t])] != 0.0;
  for (int t = 0; t < op.n_f2; ++t)
    k += op.f2_J[4 * t + 2 * bit_at(s, op.f2_ij[2 * t]) + bit_at(s, op.f2_ij[2 * t + 1])] != 0.0;
  counts[c] = k;
}

// exclusive prefix sum of counts into offsets[0..ns], single block
__global__ void rc_scan_kernel(const int64_t* __restrict__ counts, int64_t ns, int64_t* __restrict__ offsets) {
  __shared__ int64_t part[1024];
  const int t = threadIdx.x;
  const int64_t per = (ns + blockDim.x - 1) / blockDim.x;
  const int64_t lo = min(ns, t * per), hi = min(ns, lo + per);
  int64_t s = 0;
  for (int64_t i = lo; i < hi; ++i) s += counts[i];
  part[t] = s;
  __syncthreads();
  if (t == 0) {
    int64_t acc = 0;
    for (int k = 0; k < (int)blockDim.x; ++k) {
      const int64_t v = part[k];
      part[k] = acc;
      acc += v;
    }
    offsets[ns] = acc;
  }
  __syncthreads();
  int64_t acc = part[t];
  for (int64_t i = lo; i < hi; ++i) {
    offsets[i] = acc;
    acc += counts[i];
  }
}

__global__ void rc_conn_write_kernel(qgx_operator_t op, const uint32_t* __restrict__ spins, int64_t ns, int n,
                                     const int64_t* __restrict__ offsets, uint32_t* __restrict__ conn,
                                     double* __restrict__ elem) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= ns) return;
  const int nw = words_for(n);
  const uint32_t* s = spins + c * nw;
  int64_t k = offsets[c];
  for (int t = 0; t < op.n_f1; ++t) {
    const int i = op.f1_i[t];
    const double e = op.f1_J[2 * t + bit_at(s, i)];
    if (e == 0.0) continue;
    for (int q = 0; q < nw; ++q) conn[k * nw + q] = s[q] ^ ((q == (i >> 5)) ? (1u << (i & 31)) : 0u);
    elem[k++] = e;
  }
  for (int t = 0; t < op.n_f2; ++t) {
    const int i = op.f2_ij[2 * t], j = op.f2_ij[2 * t + 1];
    const double e = op.f2_J[4 * t + 2 * bit_at(s, i) + bit_at(s, j)];
    if (e == 0.0) continue;
    for (int q = 0; q < nw; ++q) {
      uint32_t v = s[q];
      if (q == (i >> 5)) v ^= 1u << (i & 31);
      if (q == (j >> 5)) v ^= 1u << (j & 31);
      conn[k * nw + q] = v;
    }
    elem[k++] = e;
  }
}

// E_loc(s) = diag(s) + sum_k elem_k exp(log psi(s'_k) - log psi(s)), complex
// the Philox step base of a sweep, and the live count of the compacted proposals (zero)
__global__ void rc_set_step_kernel(uint64_t* __restrict__ step_base, uint64_t step0) {
  step_base[0] = step0;
  step_base[1] = 0;
}

__global__ void rc_eloc_reduce_kernel(qgx_operator_t op, const uint32_t* __restrict__ spins, int64_t ns, int n,
                                      const float2* __restrict__ lp, const int64_t* __restrict__ offsets,
                                      const double* __restrict__ elem, const float2* __restrict__ lp_conn,
                                      double* __restrict__ er, double* __restrict__ ei) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= ns) return;
  const uint32_t* s = spins + c * words_for(n);
  double d = op.c0;
  for (int t = 0; t < op.n_z; ++t) d += op.z_J[t] * (bit_at(s, op.z_i[t]) ? 1.0 : -1.0);
  for (int t = 0; t < op.n_zz; ++t)
    d += op.zz_J[t] * ((bit_at(s, op.zz_ij[2 * t]) == bit_at(s, op.zz_ij[2 * t + 1])) ? 1.0 : -1.0);
  double re = d, im = 0.0;
  const float2 l0 = lp[c];
  for (int64_t k = offsets[c]; k < offsets[c + 1]; ++k) {
    const float2 l = lp_conn[k];
    const double m = exp((double)l.x - (double)l0.x);
    const double ph = (double)l.y - (double)l0.y;
    re += elem[k] * m * cos(ph);
    im += elem[k] * m * sin(ph);
  }
  er[c] = re;
  if (ei) ei[c] = im;
}

// ---- symmetry projection (quantax/symmetry/symmetry.py:325-392) -----------------------------
struct SymmDev {
  const int16_t* perm;
  const double* weight;
  int nperm, nsymm;
};

// the symmetrised configurations of the jacobian: T_g s per (sample, g), log psi(T_g s),
// log psi_symm(s) and the weights; cfg == nullptr means no symmetry
struct SymmJac {
  const uint32_t* cfg;
  const float2* lp_g;
  const float2* lp_sym;
  const double* weight;
  int nsymm;
};

// row c * nsymm + g of out = T_g s_c (bits past n stay 0); n_live_exp = live count x nsymm
__global__ void rc_symm_expand_kernel(const uint32_t* __restrict__ cfg, int64_t ncfg, const int64_t* __restrict__ n_live,
                                      int n, const int16_t* __restrict__ perm, int nperm, int nsymm,
                                      uint32_t* __restrict__ out, int64_t* __restrict__ n_live_exp) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t total = n_live ? min(ncfg, *n_live) : ncfg;
  if (idx == 0 && n_live_exp) *n_live_exp = total * nsymm;
  const int64_t c = idx / nsymm;
  const int g = (int)(idx - c * nsymm);
  if (c >= total) return;
  const int nw = words_for(n);
  const uint32_t* src = cfg + c * nw;
  const int16_t* p = perm + (int64_t)(g % nperm) * n;
  const bool flip = g >= nperm;
  uint32_t* dst = out + idx * nw;
  for (int k = 0; k < nw; ++k) {
    const int nb = min(32, n - 32 * k);
    uint32_t w = 0;
    for (int b = 0; b < nb; ++b) {
      int j = p[32 * k + b];
      j = j < 0 ? 0 : (j >= n ? n - 1 : j);  // a malformed table stays inside the row
      w |= ((src[j >> 5] >> (j & 31)) & 1u) << b;
    }
    if (flip) w ^= nb == 32 ? 0xffffffffu : ((1u << nb) - 1u);
    dst[k] = w;
  }
}

// log psi_symm(s_c) = log sum_g w_g exp(log psi(T_g s_c)), stable in the largest |psi(T_g s)|
__global__ void rc_symm_combine_kernel(const float2* __restrict__ lp_g, int64_t ncfg, const int64_t* __restrict__ n_live,
                                       int nsymm, const double* __restrict__ weight, float2* __restrict__ out) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t total = n_live ? min(ncfg, *n_live) : ncfg;
  if (c >= total) return;
  const float2* l = lp_g + c * nsymm;
  float m = -INFINITY;
  for (int g = 0; g < nsymm; ++g) m = fmaxf(m, l[g].x);
  if (m == -INFINITY) {
    out[c] = make_float2(-INFINITY, 0.0f);
    return;
  }
  // FP32 arithmetic: the inputs are FP32 log psi, and FP64 transcendentals run at a small
  // fraction of the FP32 rate on this GPU
  float zr = 0.0f, zi = 0.0f;
  for (int g = 0; g < nsymm; ++g) {
    const float e = expf(l[g].x - m);
    float sn, cs;
    sincosf(l[g].y, &sn, &cs);
    const float ar = e * cs, ai = e * sn;
    const float wr = (float)weight[2 * g], wi = (float)weight[2 * g + 1];
    zr += wr * ar - wi * ai;
    zi += wr * ai + wi * ar;
  }
  out[c] = make_float2(m + 0.5f * logf(zr * zr + zi * zi), atan2f(zi, zr));
}

// ---- per-sample log-derivatives (Variational.jacobian, quantax/state/variational.py:424-511) ----
__device__ inline float gelu_tanh_grad(float x) {
  const float k0 = 0.7978845608028654f;
  const float u = k0 * fmaf(0.044715f * x, x * x, x);
  const float t = tanhf(u);
  return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * k0 * fmaf(3.0f * 0.044715f, x * x, 1.0f);
}

constexpr int kJacThreads = 256;

// dW[o][i][t] += sum_r g[k][o][r] in[i][nbr(r,t)] and db[o] = sum_r g[k][o][r] for both
// cotangents k, written to the O rows at the layer's parameter offset (reference layout
// (o, i, ky, kx) then bias). Thread = (cotangent, 4 output channels, input channel, half of
// the sites); the two halves are summed with a lane shuffle.
template <int C>
__device__ inline void weight_grads(const float* __restrict__ g /*[2][C][N]*/, const float* __restrict__ in /*[cin][N]*/,
                                    int cin, const int16_t* __restrict__ nbr, int N, bool has_bias,
                                    float* __restrict__ o_re, float* __restrict__ o_im, bool accumulate) {
  constexpr int G = C / 4;
  const int items = 2 * G * cin * 2;  // cotangent x o-group x input channel x half
  // every lane of a warp runs the same iterations (blockDim is a multiple of 32), so the
  // full-warp shuffles below always see all 32 lanes; lanes past `items` add zeros
  for (int base = 0; base < items; base += blockDim.x) {
    const int it = base + threadIdx.x;
    const bool active = it < items;
    const int half = it & 1;
    const int rest = active ? it >> 1 : 0;
    const int i = rest % cin;
    const int og = (rest / cin) % G;
    const int k = rest / (cin * G);
    float acc[4][9];
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int t = 0; t < 9; ++t) acc[q][t] = 0.0f;
    float bacc[4] = {0.f, 0.f, 0.f, 0.f};
    const float* gk = g + (int64_t)k * C * N + (4 * og) * N;
    const float* ini = in + (int64_t)i * N;
    const int r0 = half ? N / 2 : 0, r1 = !active ? 0 : (half ? N : N / 2);
    for (int r = r0; r < r1; ++r) {
      float gv[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) gv[q] = gk[q * N + r];
#pragma unroll
      for (int t = 0; t < 9; ++t) {
        const float v = ini[nbr[r * 9 + t]];
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[q][t] = fmaf(gv[q], v, acc[q][t]);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) bacc[q] += gv[q];
    }
    // the two halves sit in adjacent lanes (items are laid out half-fastest)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
#pragma unroll
      for (int t = 0; t < 9; ++t) acc[q][t] += __shfl_xor_sync(0xffffffffu, acc[q][t], 1);
      bacc[q] += __shfl_xor_sync(0xffffffffu, bacc[q], 1);
    }
    if (active && half == 0) {
      float* row = k == 0 ? o_re : o_im;
      if (row) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int o = 4 * og + q;
#pragma unroll
          for (int t = 0; t < 9; ++t) {
            float* dst = row + ((int64_t)o * cin + i) * 9 + t;
            *dst = accumulate ? *dst + acc[q][t] : acc[q][t];
          }
          if (has_bias && i == 0) {
            float* dst = row + (int64_t)C * cin * 9 + o;
            *dst = accumulate ? *dst + bacc[q] : bacc[q];
          }
        }
      }
    }
  }
}

// gin[k][i][r] = sum_{t,o} W[o][i][t] g[k][o][nbr(r, 8 - t)] (transposed convolution), WT = W as [t][o][i]
template <int C>
__device__ inline void input_grads(const float* __restrict__ g, const float* __restrict__ WT, int cin,
                                   const int16_t* __restrict__ nbr, int N, float* __restrict__ gin) {
  for (int it = threadIdx.x; it < 2 * N; it += blockDim.x) {
    const int k = it / N, r = it - k * N;
    float acc[C];
#pragma unroll
    for (int i = 0; i < C; ++i) acc[i] = 0.0f;
    const float* gk = g + (int64_t)k * C * N;
#pragma unroll
    for (int t = 0; t < 9; ++t) {
      const int rn = nbr[r * 9 + (8 - t)];
      auto term = [&](int o) {
        const float v = gk[o * N + rn];
        const float4* wp = reinterpret_cast<const float4*>(WT + (t * C + o) * C);
#pragma unroll
        for (int i4 = 0; i4 < C / 4; ++i4) {
          const float4 w = wp[i4];
          acc[4 * i4] = fmaf(v, w.x, acc[4 * i4]);
          acc[4 * i4 + 1] = fmaf(v, w.y, acc[4 * i4 + 1]);
          acc[4 * i4 + 2] = fmaf(v, w.z, acc[4 * i4 + 2]);
          acc[4 * i4 + 3] = fmaf(v, w.w, acc[4 * i4 + 3]);
        }
      };
      if constexpr (C <= 8) {
        // left to itself the compiler unrolls all 8 output channels here and spills 4 KB per
        // thread; four at a time keeps every value in registers
#pragma unroll 4
        for (int o = 0; o < C; ++o) term(o);
      } else {
        for (int o = 0; o < C; ++o) term(o);
      }
    }
#pragma unroll
    for (int i = 0; i < C; ++i)  // constant indices keep acc in registers
      if (i < cin) gin[((int64_t)k * C + i) * N + r] = acc[i];
  }
}

// stage layer l's table slice into W and its transpose WT[t][o][i]
template <int C>
__device__ inline void stage_layer(const float* table, int l, float* W, float* WT) {
  const int cin = layer_cin(l, C);
  const float* src = table + layer_offset(l, C);
  const int nf = cin * 9 * C + C;
  for (int e = threadIdx.x; e < nf; e += blockDim.x) W[e] = __ldg(src + e);
  for (int e = threadIdx.x; e < 9 * C * C; e += blockDim.x) {
    const int t = e / (C * C), o = (e / C) % C, i = e % C;
    WT[e] = i < cin ? __ldg(src + (i * 9 + t) * C + o) : 0.0f;
  }
}

template <int C>
__global__ void __launch_bounds__(kJacThreads)
    rc_jacobian_kernel(const float* __restrict__ table, ConvNet net, const uint32_t* __restrict__ spins, int64_t ns,
                       float* __restrict__ o_re, float* __restrict__ o_im, int64_t ldo, float* __restrict__ scratch,
                       SymmJac sj) {
  extern __shared__ float4 smem4[];
  float* sm = reinterpret_cast<float*>(smem4);
  const int N = net.N, B = net.B, nw = words_for(N);
  const int CN = C * N;
  float* X = sm;                 // [C][N] block input / running activation
  float* P = X + CN;             // [C][N] pre(X_b)
  float* Qa = P + CN;            // [C][N] conv1 pre-activation A, then gelu(A)
  float* G = Qa + CN;            // [2][C][N] cotangent of X
  float* GA = G + 2 * CN;        // [2][C][N] cotangent of A
  float* GP = GA + 2 * CN;       // [2][C][N] cotangent of P
  float* W = GP + 2 * CN;        // layer table slice (C*9*C + C)
  float* WT = W + C * 9 * C + C; // [9][C][C]
  int16_t* nbr = reinterpret_cast<int16_t*>(WT + 9 * C * C);
  __shared__ float red[2][kJacThreads / 32];
  build_nbr(nbr, net.L);
  float* mine = scratch + (int64_t)blockIdx.x * B * 2 * CN;  // X_b and A_b of every block
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const float fs = rsqrtf((float)(B + 1));
  const int cp = net.cplx ? C / 2 : C;
  const int ng = sj.cfg ? sj.nsymm : 1;
  for (int64_t smp = blockIdx.x; smp < ns; smp += gridDim.x) {
   for (int g = 0; g < ng; ++g) {
    // v = d log psi_symm / d log psi(T_g s) = w_g psi(T_g s) / psi_symm(s); 1 without symmetry
    float vr = 1.0f, vi = 0.0f;
    const uint32_t* src = spins + smp * nw;
    if (sj.cfg) {
      const int64_t k = smp * sj.nsymm + g;
      src = sj.cfg + k * nw;
      const float2 lg = sj.lp_g[k], ls = sj.lp_sym[smp];
      const double mag = exp((double)lg.x - (double)ls.x), ph = (double)lg.y - (double)ls.y;
      const double ar = mag * cos(ph), ai = mag * sin(ph), wr = sj.weight[2 * g], wi = sj.weight[2 * g + 1];
      vr = (float)(wr * ar - wi * ai);
      vi = (float)(wr * ai + wi * ar);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < N; e += blockDim.x) {
      const float v = ((src[e >> 5] >> (e & 31)) & 1u) ? 1.0f : -1.0f;
      for (int c = 0; c < C; ++c) X[c * N + e] = v;
    }
    // ---- forward, saving X_b and A_b
    for (int b = 0; b < B; ++b) {
      const float scale = rsqrtf((float)(b + 1)) * (b == 0 ? 0.70710678118654752f : 1.0f);
      const int cin = b == 0 ? 1 : C;
      __syncthreads();
      float* xs = mine + (int64_t)b * 2 * CN;
      for (int e = threadIdx.x; e < CN; e += blockDim.x) {
        xs[e] = X[e];
        const float v = X[e] * scale;
        if (e < cin * N) P[e] = b == 0 ? v : gelu_tanh(v);
      }
      stage_layer<C>(table, 2 * b, W, WT);
      __syncthreads();
      // A = conv1(P) + b1 (pre-activation kept: conv_layer mode 1 on a zeroed buffer)
      for (int e = threadIdx.x; e < CN; e += blockDim.x) Qa[e] = 0.0f;
      __syncthreads();
      conv_layer<C, 1>(P, cin, Qa, W, nbr, N, 1, 1, C * N);
      __syncthreads();
      for (int e = threadIdx.x; e < CN; e += blockDim.x) {
        xs[CN + e] = Qa[e];
        Qa[e] = gelu_tanh(Qa[e]);
      }
      stage_layer<C>(table, 2 * b + 1, W, WT);
      __syncthreads();
      conv_layer<C, 1>(Qa, C, X, W, nbr, N, 1, 1, C * N);
    }
    __syncthreads();
    // ---- output cotangents: w_e = f'(z_e) / sum f, f = exp (exp_by_scale) or sinh + 1
    float m = -INFINITY;
    for (int e = threadIdx.x; e < cp * N; e += blockDim.x) m = fmaxf(m, net.sinhp1 ? fabsf(X[e] * fs) : X[e] * fs);
    m = warp_max(m);
    if (lane == 0) red[0][warp] = m;
    __syncthreads();
    m = red[0][0];
    for (int w = 1; w < kJacThreads / 32; ++w) m = fmaxf(m, red[0][w]);
    __syncthreads();
    float sr = 0.0f, si = 0.0f;
    for (int e = threadIdx.x; e < cp * N; e += blockDim.x) {
      if (net.sinhp1) {
        float fr, fi, gr, gi;
        sinhp1_shifted(X[e] * fs, net.cplx ? X[cp * N + e] * fs : 0.0f, m, net.cplx, &fr, &fi, &gr, &gi);
        sr += fr;
        si += fi;
        continue;
      }
      const float ex = expf(X[e] * fs - m);
      float sn = 0.0f, cs = 1.0f;
      if (net.cplx) sincosf(X[cp * N + e] * fs, &sn, &cs);
      sr = fmaf(ex, cs, sr);
      si = fmaf(ex, sn, si);
    }
    sr = warp_sum(sr);
    si = warp_sum(si);
    if (lane == 0) {
      red[0][warp] = sr;
      red[1][warp] = si;
    }
    __syncthreads();
    sr = 0.0f;
    si = 0.0f;
    for (int w = 0; w < kJacThreads / 32; ++w) {
      sr += red[0][w];
      si += red[1][w];
    }
    // 1 / (sr + i si)
    const float den = sr * sr + si * si;
    const float ir = sr / den, ii = -si / den;
    for (int e = threadIdx.x; e < cp * N; e += blockDim.x) {
      float ar, ai;
      if (net.sinhp1) {
        float fr, fi;
        sinhp1_shifted(X[e] * fs, net.cplx ? X[cp * N + e] * fs : 0.0f, m, net.cplx, &fr, &fi, &ar, &ai);
      } else {
        const float ex = expf(X[e] * fs - m);
        float sn = 0.0f, cs = 1.0f;
        if (net.cplx) sincosf(X[cp * N + e] * fs, &sn, &cs);
        ar = ex * cs;
        ai = ex * sn;
      }
      const float ur = ar * ir - ai * ii, ui = ar * ii + ai * ir;  // f'(z) / sum f
      const float wr = vr * ur - vi * ui, wi = vr * ui + vi * ur;  // times v
      if (net.cplx) {
        G[e] = wr * fs;               // d Re / d y_c
        G[cp * N + e] = -wi * fs;     // d Re / d y_{c+C/2}
        G[CN + e] = wi * fs;          // d Im / d y_c
        G[CN + cp * N + e] = wr * fs; // d Im / d y_{c+C/2}
      } else {
        G[e] = wr * fs;
        G[CN + e] = 0.0f;
      }
    }
    // ---- backward
    float* row_re = o_re + smp * ldo;
    float* row_im = o_im ? o_im + smp * ldo : nullptr;
    int64_t poff = nparams_rc(B, C);
    for (int b = B - 1; b >= 0; --b) {
      const int cin = b == 0 ? 1 : C;
      const bool last = b == B - 1;
      const int64_t n2 = (int64_t)C * C * 9 + (last ? 0 : C);
      const int64_t n1 = (int64_t)C * cin * 9 + C;
      poff -= n1 + n2;
      const float scale = rsqrtf((float)(b + 1)) * (b == 0 ? 0.70710678118654752f : 1.0f);
      const float* xs = mine + (int64_t)b * 2 * CN;
      __syncthreads();
      for (int e = threadIdx.x; e < CN; e += blockDim.x) {
        const float a = xs[CN + e];
        Qa[e] = gelu_tanh(a);
        const float v = xs[e] * scale;
        if (e < cin * N) P[e] = b == 0 ? v : gelu_tanh(v);
      }
      stage_layer<C>(table, 2 * b + 1, W, WT);
      __syncthreads();
      // conv2: grads of W2, b2 and of Q (into GA)
      weight_grads<C>(G, Qa, C, nbr, N, !last, row_re + poff + n1, row_im ? row_im + poff + n1 : nullptr, g > 0);
      input_grads<C>(G, WT, C, nbr, N, GA);
      __syncthreads();
      for (int e = threadIdx.x; e < 2 * CN; e += blockDim.x) GA[e] *= gelu_tanh_grad(xs[CN + (e % CN)]);
      stage_layer<C>(table, 2 * b, W, WT);
      __syncthreads();
      weight_grads<C>(GA, P, cin, nbr, N, true, row_re + poff, row_im ? row_im + poff : nullptr, g > 0);
      if (b > 0) {
        input_grads<C>(GA, WT, cin, nbr, N, GP);
        __syncthreads();
        for (int e = threadIdx.x; e < 2 * CN; e += blockDim.x) {
          const int ee = e % CN;
          G[e] += GP[e] * gelu_tanh_grad(xs[ee] * scale) * scale;
        }
      }
    }
   }
  }
}

template <int C>
int launch_jacobian_c(const float* table, const ConvNet& net, const uint32_t* spins, int64_t ns, float* o_re,
                      float* o_im, int64_t ldo, float* scratch, int64_t scratch_floats, const SymmJac& sj,
                      cudaStream_t st) {
  const int CN = C * net.N;
  const int64_t sf = 3LL * CN + 6LL * CN + C * 9 * C + C + 9 * C * C;
  const int smem = (int)(sf * 4 + net.N * 9 * 2 + 16);
  auto k = rc_jacobian_kernel<C>;
  if (smem > 48 * 1024) QGX_CHECK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  int per_sm = 0;
  QGX_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kJacThreads, smem));
  if (per_sm < 1) return QGX_ERR_UNSUPPORTED;
  const int64_t per_cta = (int64_t)net.B * 2 * CN;
  int64_t grid = std::min<int64_t>((int64_t)device_sm_count() * per_sm, ns);
  grid = std::min<int64_t>(grid, scratch_floats / per_cta);
  if (grid < 1) return QGX_ERR_ARG;
  k<<<(unsigned)grid, kJacThreads, smem, st>>>(table, net, spins, ns, o_re, o_im, ldo, scratch, sj);
  return launch_status();
}

// shared memory of the FP32 forward with S samples per CTA, in the blocked order (blk, even L
// only) or the site order
int rc_smem_bytes(const ConvNet& net, int S, bool blk) {
  const int64_t f = rc_weights_offset(S, rc_sample_stride(net.C, net.N, blk)) + (int64_t)net.C * 9 * net.C + net.C;
  const int64_t tables = blk ? (int64_t)net.N * 4 + net.N : (int64_t)net.N * 9;  // int16 entries
  return (int)(f * 4 + tables * 2 + 16);
}

// samples per CTA in the blocked order: the count whose work items (channel groups x samples x
// blocks, each group rounded to whole warps) fill the 256 threads' passes best, among the counts
// whose shared memory leaves room for two CTAs per SM (any count that fits, if none does): 5 at
// L = 10 with 16 channels (2 x 128 items, 250 of them used), 32 at L = 4
template <int C>
int rc_blocked_samples(const ConvNet& net) {
  constexpr int H = C / rc_blocked_co<C>();
  const int NB = net.N / 4;
  const int cap = device_max_smem_optin();
  const int two = (cap + 1024) / 2 - 1024;  // 1 KB of each CTA's shared memory is reserved
  for (int limit : {two, cap}) {
    int best = 0;
    double best_fill = 0.0;
    for (int s = 1; s <= 64 && rc_smem_bytes(net, s, true) <= limit; ++s) {
      const int per = (s * NB + 31) & ~31;
      const int passes = (H * per + kFwdThreads - 1) / kFwdThreads;
      const double fill = (double)H * s * NB / ((double)passes * kFwdThreads);
      if (fill > best_fill + 1e-9) best_fill = fill, best = s;
    }
    if (best > 0) return best;
  }
  return 1;
}

template <int C>
int launch_forward_c(const float* table, const ConvNet& net, const uint32_t* cfg, int64_t ncfg, const int64_t* n_live,
                     float2* out, cudaStream_t st) {
  // site order: kFwdSamples per CTA (5 x 50 site pairs fill 256 threads at L = 10), fewer where
  // their buffers would not fit (L = 16: 4)
  int S = kFwdSamples;
  while (S > 1 && rc_smem_bytes(net, S, false) > device_max_smem_optin()) --S;
  // The blocked order (even L) where it does not lengthen a thread's serial work: a thread
  // computes 4 x CO outputs per layer there against 2 x C in the site order, more at fewer than
  // 12 channels. That only pays when the batch gives every SM two CTAs (measured at L = 4 with 8
  // channels: 30 against 15 us for 512 configurations, 84 against 182 us for 32768). Both orders
  // give the same floats, so the choice never changes a result.
  bool blk = false;
  if (net.L % 2 == 0) {
    const int sb = rc_blocked_samples<C>(net);
    blk = 4 * rc_blocked_co<C>() <= 2 * C || (ncfg + sb - 1) / sb >= 2LL * device_sm_count();
    if (blk) S = sb;
  }
  const int smem = rc_smem_bytes(net, S, blk);
  if (smem > device_max_smem_optin()) return QGX_ERR_UNSUPPORTED;
  auto k = blk ? rc_forward_kernel<C, true> : rc_forward_kernel<C, false>;
  if (smem > 48 * 1024) QGX_CHECK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  int per_sm = 0;
  QGX_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kFwdThreads, smem));
  if (per_sm < 1) return QGX_ERR_UNSUPPORTED;
  const int64_t want = (ncfg + S - 1) / S;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)device_sm_count() * per_sm, want));
  k<<<grid, kFwdThreads, smem, st>>>(table, net, cfg, ncfg, n_live, out, S);
  return launch_status();
}

int launch_forward(const float* table, const ConvNet& net, const uint32_t* cfg, int64_t ncfg, const int64_t* n_live,
                   float2* out, cudaStream_t st) {
  if (net.rbm_m > 0) return rbm_log_psi_pairs(table, net.N, net.rbm_m, cfg, ncfg, n_live, out, st);
  if (net.prec != QGX_CONV_FP32)
    return rc_launch_forward_tc(table, net.L, net.B, net.C, net.cplx, net.sinhp1, cfg, ncfg, n_live, out,
                                net.prec == QGX_CONV_BF16 ? 1 : 0, net.grouped, st);
  switch (net.C) {
    case 4: return launch_forward_c<4>(table, net, cfg, ncfg, n_live, out, st);
    case 8: return launch_forward_c<8>(table, net, cfg, ncfg, n_live, out, st);
    case 12: return launch_forward_c<12>(table, net, cfg, ncfg, n_live, out, st);
    case 16: return launch_forward_c<16>(table, net, cfg, ncfg, n_live, out, st);
    default: return QGX_ERR_UNSUPPORTED;
  }
}

inline int64_t al256(int64_t b) { return (b + 255) / 256 * 256; }

// scratch of one symmetrised forward over ncfg configurations
int64_t symm_scratch_bytes(int64_t ncfg, int nw, int nsymm) {
  return al256(ncfg * nsymm * nw * 4) + al256(ncfg * nsymm * 8) + al256(8);
}

// log psi (or log psi_symm with sym) of ncfg configurations, n_live as in launch_forward
int symm_forward(const float* table, const ConvNet& net, const SymmDev* sym, const uint32_t* cfg, int64_t ncfg,
                 const int64_t* n_live, float2* out, char* scratch, cudaStream_t st, float2** lp_g_out = nullptr,
                 const uint32_t** cfg_out = nullptr) {
  if (!sym) return launch_forward(table, net, cfg, ncfg, n_live, out, st);
  const int nw = words_for(net.N);
  const int64_t ne = ncfg * sym->nsymm;
  uint32_t* cg = reinterpret_cast<uint32_t*>(scratch);
  float2* lg = reinterpret_cast<float2*>(scratch + al256(ne * nw * 4));
  int64_t* nle = reinterpret_cast<int64_t*>(scratch + al256(ne * nw * 4) + al256(ne * 8));
  rc_symm_expand_kernel<<<(unsigned)((ne + 127) / 128), 128, 0, st>>>(cfg, ncfg, n_live, net.N, sym->perm, sym->nperm,
                                                                       sym->nsymm, cg, n_live ? nle : nullptr);
  int rc = launch_forward(table, net, cg, ne, n_live ? nle : nullptr, lg, st);
  if (rc != QGX_OK) return rc;
  rc_symm_combine_kernel<<<(unsigned)((ncfg + 127) / 128), 128, 0, st>>>(lg, ncfg, n_live, sym->nsymm, sym->weight,
                                                                         out);
  if (lp_g_out) *lp_g_out = lg;
  if (cfg_out) *cfg_out = cg;
  return launch_status();
}

// ---- sweep graphs ----------------------------------------------------------------------
// A sweep is 1 + 3 nsteps launches (forward, then propose / forward / accept per step). The
// launch sequence is captured once per set of buffers and sizes into a CUDA graph (on a
// private stream, relaxed capture mode) and replayed on the caller's stream; the Philox step
// base lives in the workspace, so one graph serves every starting step.
struct SweepKey {
  const void *table, *spins, *lp, *acc, *nbr, *ws, *perm, *weight;
  int64_t nperm_nsymm;
  int64_t ns;
  int nsteps, L, N, B, C, cplx, prec, z, hop, device, rbm_m, rbm_vbias, proposal;
  uint64_t seed;
  float reweight;
  bool operator==(const SweepKey& o) const { return std::memcmp(this, &o, sizeof(SweepKey)) == 0; }
};

struct SweepGraph {
  SweepKey key;
  cudaGraphExec_t exec;
  uint64_t last_use;
};

constexpr int kMaxSweepGraphs = 32;
std::mutex g_graph_mutex;
std::vector<SweepGraph> g_graphs;
uint64_t g_graph_clock = 0;
cudaStream_t g_capture_stream[64] = {};

bool valid_net(int L, int B, int C, int out_flags) {
  return L >= 3 && L * L <= kMaxSitesConv && B >= 1 && B <= 64 && (C == 4 || C == 8 || C == 12 || C == 16) &&
         (out_flags & ~(QGX_RESCONV_COMPLEX | QGX_RESCONV_SINHP1)) == 0 &&
         (!(out_flags & QGX_RESCONV_COMPLEX) || C % 2 == 0);
}

bool valid_prec(int p) {
  return p == QGX_CONV_FP32 || p == QGX_CONV_TF32 || p == QGX_CONV_BF16 || p == (QGX_CONV_BF16 | QGX_CONV_GROUPED);
}

constexpr int kMaxSymm = 1024;

// the public descriptor checked and made internal; false on a malformed one
bool to_symm(const qgx_symm_t* s, SymmDev* d) {
  if (!s || !s->perm || !s->weight || s->nperm < 1) return false;
  d->perm = s->perm;
  d->weight = s->weight;
  d->nperm = s->nperm;
  d->nsymm = s->nperm * (s->z2 != 0 ? 2 : 1);
  return d->nsymm <= kMaxSymm;
}

// ---- the projected RBM (Variational(RBM_Dense, symm=...)) ------------------------------------
// RBM_Dense sizes the symmetrised pipelines take: a packed configuration of at most 8 words
// (the proposal kernel's registers) and the RBM kernels' hidden-unit widths
bool valid_rbm_symm(int n, int m) { return n >= 1 && n <= kMaxSitesConv && m >= 1 && m <= 2048; }

int64_t eloc_scratch_bytes(int n, int64_t ns, int max_conn) {
  const int nw = words_for(n);
  const int64_t nc = ns * (int64_t)std::max(max_conn, 1);
  return al256(ns * 8) + al256((ns + 1) * 8) + al256(nc * nw * 4) + al256(nc * 8) + al256(nc * 8) + al256(ns * 8);
}

int64_t sweep_scratch_bytes(int n, int64_t ns) {
  const int nw = words_for(n);
  return al256(ns * nw * 4) + al256(ns * 8) + al256(ns * 4) + al256(16);
}

// samples per pass of the projected RBM's log-derivatives: their images' O rows (nsymm x np
// floats each) fill at most 2^26 floats, at least one sample
int64_t rbm_symm_chunk(int64_t ns, int nsymm, int64_t np) {
  const int64_t per = (int64_t)nsymm * np;
  return std::max<int64_t>(1, std::min<int64_t>(std::min<int64_t>(ns, 65535), (int64_t(1) << 26) / per));
}

// O_symm[c][p] = sum_g v_g O(T_g s_c)[p], v_g = w_g psi(T_g s_c) / psi_symm(s_c) (the cotangents
// of variational.py:441-477 for a holomorphic-free real model), from the images' rows
// rows[(c - c0) nsymm + g][p] of the samples c0 .. c0 + gridDim.y - 1; Re to O_re, Im to O_im
// (may be NULL). FP32 sums over the group in its order.
__global__ void __launch_bounds__(256)
    rbm_symm_rows_kernel(const float* __restrict__ rows, int64_t np, int64_t c0, int nsymm,
                         const float2* __restrict__ lp_g, const float2* __restrict__ lp_sym,
                         const double* __restrict__ weight, float* __restrict__ O_re, float* __restrict__ O_im,
                         int64_t ldo) {
  extern __shared__ float2 v[];
  const int64_t cl = blockIdx.y, c = c0 + cl;
  const float2 ls = lp_sym[c];
  for (int g = threadIdx.x; g < nsymm; g += blockDim.x) {
    const float2 lg = lp_g[c * nsymm + g];
    const float e = expf(lg.x - ls.x);
    float sn, cs;
    sincosf(lg.y - ls.y, &sn, &cs);
    const float ar = e * cs, ai = e * sn;
    const float wr = (float)weight[2 * g], wi = (float)weight[2 * g + 1];
    v[g] = make_float2(wr * ar - wi * ai, wr * ai + wi * ar);
  }
  __syncthreads();
  const float* base = rows + cl * nsymm * np;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
    float re = 0.0f, im = 0.0f;
    for (int g = 0; g < nsymm; ++g) {
      const float o = base[(int64_t)g * np + p];
      re = fmaf(v[g].x, o, re);
      im = fmaf(v[g].y, o, im);
    }
    O_re[c * ldo + p] = re;
    if (O_im) O_im[c * ldo + p] = im;
  }
}

}  // namespace
}  // namespace qgx

using namespace qgx;

extern "C" {

int64_t qgx_resconv_nparams(int32_t nblocks, int32_t channels) {
  if (nblocks < 1 || channels < 1) return 0;
  return nparams_rc(nblocks, channels);
}

int64_t qgx_resconv_table_floats(int32_t nblocks, int32_t channels) {
  if (nblocks < 1 || channels < 1) return 0;
  return table_floats_rc(nblocks, channels);
}

int qgx_resconv_prepare(const float* params, int32_t nblocks, int32_t channels, float* table, qgx_stream_t stream) {
  QGX_CHECK_ARG(params && table && nblocks >= 1 && (channels == 4 || channels == 8 || channels == 12 || channels == 16));
  QGX_CHECK_ARG((reinterpret_cast<uintptr_t>(table) & 15) == 0);
  rc_prepare_kernel<<<16, 256, 0, as_cuda(stream)>>>(params, nblocks, channels, table);
  const int rc = launch_status();
  if (rc != QGX_OK) return rc;
  return rc_prepare_tc_images(table, nblocks, channels, as_cuda(stream));
}

int qgx_resconv_log_psi(const float* table, int32_t L, int32_t nblocks, int32_t channels, int32_t complex_out,
                        int32_t conv_precision, const uint32_t* spins, int64_t ns, float* log_psi,
                        qgx_stream_t stream) {
  QGX_CHECK_ARG(valid_net(L, nblocks, channels, complex_out) && valid_prec(conv_precision) && ns >= 0);
  if (ns == 0) return QGX_OK;
  QGX_CHECK_ARG(table && spins && log_psi);
  const ConvNet net = make_net(L, nblocks, channels, complex_out, conv_precision);
  return launch_forward(table, net, spins, ns, nullptr, reinterpret_cast<float2*>(log_psi), as_cuda(stream));
}

int64_t qgx_resconv_sweep_workspace_bytes(int32_t L, int64_t ns) {
  if (L < 1 || ns < 1) return 0;
  const int nw = words_for(L * L);
  // compacted proposals, their log psi, their positions, then the step base and live count
  return al256(ns * nw * 4) + al256(ns * 8) + al256(ns * 4) + al256(16);
}

}  // extern "C"

namespace qgx {
namespace {

// out_flags: the ResConv output flags (0 for an RBM); proposal: QGX_PROPOSAL_*
int sweep_impl(const float* table, const ConvNet& net, int32_t out_flags, const SymmDev* sym, uint32_t* spins,
               float* log_psi, int32_t* accepts, int64_t ns, int32_t nsteps, uint64_t seed, uint64_t step0,
               float reweight, int32_t proposal, const int32_t* nbr, int32_t z, int32_t hop, void* workspace,
               cudaStream_t st) {
  const int nw = words_for(net.N);
  char* ws = static_cast<char*>(workspace);
  uint32_t* comp = reinterpret_cast<uint32_t*>(ws);
  float2* lp_comp = reinterpret_cast<float2*>(ws + al256(ns * nw * 4));
  int32_t* comp_idx = reinterpret_cast<int32_t*>(ws + al256(ns * nw * 4) + al256(ns * 8));
  uint64_t* step_base = reinterpret_cast<uint64_t*>(ws + al256(ns * nw * 4) + al256(ns * 8) + al256(ns * 4));
  unsigned long long* n_live = reinterpret_cast<unsigned long long*>(step_base + 1);
  char* sscratch = ws + al256(ns * nw * 4) + al256(ns * 8) + al256(ns * 4) + al256(16);
  float2* lp = reinterpret_cast<float2*>(log_psi);
  const unsigned g = (unsigned)((ns + 127) / 128);
  // the launch sequence of the sweep (recorded into the graph)
  auto record = [&](cudaStream_t s) -> int {
    int rc = symm_forward(table, net, sym, spins, ns, nullptr, lp, sscratch, s);
    if (rc != QGX_OK) return rc;
    if (accepts) QGX_CHECK_CUDA(cudaMemsetAsync(accepts, 0, ns * sizeof(int32_t), s));
    for (int t = 0; t < nsteps; ++t) {
      rc_propose_kernel<<<g, 128, 0, s>>>(spins, comp, comp_idx, n_live, ns, net.N, seed, step_base, t, nbr, z,
                                          hop, proposal);
      rc = symm_forward(table, net, sym, comp, ns, reinterpret_cast<const int64_t*>(n_live), lp_comp, sscratch, s);
      if (rc != QGX_OK) return rc;
      rc_accept_kernel<<<g, 128, 0, s>>>(spins, lp, comp, lp_comp, comp_idx, n_live, accepts, ns, net.N, seed,
                                         step_base, t, reweight);
    }
    return launch_status();
  };
  int dev = 0;
  QGX_CHECK_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return QGX_ERR_UNSUPPORTED;
  rc_set_step_kernel<<<1, 1, 0, st>>>(step_base, step0);
  QGX_CHECK_CUDA(cudaGetLastError());
  SweepKey key;
  std::memset(&key, 0, sizeof(key));
  key.table = table;
  key.spins = spins;
  key.lp = log_psi;
  key.acc = accepts;
  key.nbr = nbr;
  key.ws = workspace;
  if (sym) {
    key.perm = sym->perm;
    key.weight = sym->weight;
    key.nperm_nsymm = ((int64_t)sym->nperm << 32) | sym->nsymm;
  }
  key.ns = ns;
  key.nsteps = nsteps;
  key.L = net.L;
  key.N = net.N;
  key.B = net.B;
  key.C = net.C;
  key.cplx = out_flags;
  key.prec = net.prec | (net.grouped ? QGX_CONV_GROUPED : 0);
  key.rbm_m = net.rbm_m;
  key.rbm_vbias = net.rbm_vbias;
  key.proposal = proposal;
  key.z = z;
  key.hop = hop;
  key.device = dev;
  key.seed = seed;
  key.reweight = reweight;
  std::lock_guard<std::mutex> lock(g_graph_mutex);
  SweepGraph* hit = nullptr;
  for (auto& e : g_graphs)
    if (e.key == key) hit = &e;
  if (!hit) {
    if (!g_capture_stream[dev]) QGX_CHECK_CUDA(cudaStreamCreateWithFlags(&g_capture_stream[dev], cudaStreamNonBlocking));
    cudaStream_t cs = g_capture_stream[dev];
    QGX_CHECK_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed));
    const int rc = record(cs);
    cudaGraph_t graph = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(cs, &graph);
    if (rc != QGX_OK) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    QGX_CHECK_CUDA(ce);
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    QGX_CHECK_CUDA(ie);
    if ((int)g_graphs.size() >= kMaxSweepGraphs) {  // evict the least recently used
      auto lru = std::min_element(g_graphs.begin(), g_graphs.end(),
                                  [](const SweepGraph& a, const SweepGraph& b) { return a.last_use < b.last_use; });
      cudaGraphExecDestroy(lru->exec);
      g_graphs.erase(lru);
    }
    g_graphs.push_back(SweepGraph{key, exec, 0});
    hit = &g_graphs.back();
  }
  hit->last_use = ++g_graph_clock;
  QGX_CHECK_CUDA(cudaGraphLaunch(hit->exec, st));
  return QGX_OK;
}

}  // namespace
}  // namespace qgx

extern "C" {

int qgx_resconv_sweep(const float* table, int32_t L, int32_t nblocks, int32_t channels, int32_t complex_out,
                      int32_t conv_precision, uint32_t* spins, float* log_psi, int32_t* accepts, int64_t ns, int32_t nsteps, uint64_t seed,
                      uint64_t step0, float reweight, const int32_t* nbr, int32_t z, int32_t hop, void* workspace,
                      int64_t workspace_bytes, qgx_stream_t stream) {
  QGX_CHECK_ARG(valid_net(L, nblocks, channels, complex_out) && valid_prec(conv_precision) && ns >= 0 &&
                nsteps >= 0);
  QGX_CHECK_ARG(nbr && z > 0 && (hop == 1 || hop == -1));
  if (ns == 0) return QGX_OK;
  QGX_CHECK_ARG(table && spins && log_psi && workspace);
  QGX_CHECK_ARG(workspace_bytes >= qgx_resconv_sweep_workspace_bytes(L, ns));
  QGX_CHECK_ARG((reinterpret_cast<uintptr_t>(workspace) & 255) == 0);
  return sweep_impl(table, make_net(L, nblocks, channels, complex_out, conv_precision), complex_out, nullptr, spins,
                    log_psi, accepts, ns, nsteps, seed, step0, reweight, QGX_PROPOSAL_SPIN_EXCHANGE, nbr, z, hop,
                    workspace, as_cuda(stream));
}

int64_t qgx_resconv_sweep_symm_workspace_bytes(int32_t L, int64_t ns, int32_t nsymm) {
  if (L < 1 || ns < 1 || nsymm < 1) return 0;
  return qgx_resconv_sweep_workspace_bytes(L, ns) + symm_scratch_bytes(ns, words_for(L * L), nsymm);
}

int qgx_resconv_sweep_symm(const float* table, int32_t L, int32_t nblocks, int32_t channels, int32_t complex_out,
                           int32_t conv_precision, const qgx_symm_t* symm, uint32_t* spins, float* log_psi,
                           int32_t* accepts, int64_t ns, int32_t nsteps, uint64_t seed, uint64_t step0, float reweight,
                           const int32_t* nbr, int32_t z, int32_t hop, void* workspace, int64_t workspace_bytes,
                           qgx_stream_t stream) {
  SymmDev sym;
  QGX_CHECK_ARG(to_symm(symm, &sym));
  QGX_CHECK_ARG(valid_net(L, nblocks, channels, complex_out) && valid_prec(conv_precision) && ns >= 0 &&
                nsteps >= 0);
  QGX_CHECK_ARG(nbr && z > 0 && (hop == 1 || hop == -1));
  if (ns == 0) return QGX_OK;
  QGX_CHECK_ARG(table && spins && log_psi && workspace);
  QGX_CHECK_ARG(workspace_bytes >= qgx_resconv_sweep_symm_workspace_bytes(L, ns, sym.nsymm));
  QGX_CHECK_ARG((reinterpret_cast<uintptr_t>(workspace) & 255) == 0);
  return sweep_impl(table, make_net(L, nblocks, channels, complex_out, conv_precision), complex_out, &sym, spins,
                    log_psi, accepts, ns, nsteps, seed, step0, reweight, QGX_PROPOSAL_SPIN_EXCHANGE, nbr, z, hop,
                    workspace, as_cuda(stream));
}

int64_t qgx_resconv_eloc_workspace_bytes(int32_t L, int64_t ns, int32_t max_conn) {
  if (L < 1 || ns < 1 || max_conn < 0) return 0;
  const int nw = words_for(L * L);
  const int64_t nc = ns * (int64_t)std::max(max_conn, 1);
  return al256(ns * 8) + al256((ns + 1) * 8) + al256(nc * nw * 4) + al256(nc * 8) + al256(nc * 8) + al256(ns * 8);
}

}  // extern "C"

namespace qgx {
namespace {

int eloc_impl(const float* table, const ConvNet& net, const SymmDev* sym, const qgx_operator_t* op,
              const uint32_t* spins, int64_t ns, double* eloc_re, double* eloc_im, void* workspace, cudaStream_t st) {
  const int max_conn = op->n_f1 + op->n_f2;
  const int nw = words_for(net.N);
  const int64_t nc = ns * (int64_t)std::max(max_conn, 1);
  char* ws = static_cast<char*>(workspace);
  int64_t off = 0;
  auto take = [&](int64_t b) {
    char* p = ws + off;
    off += al256(b);
    return p;
  };
  int64_t* counts = reinterpret_cast<int64_t*>(take(ns * 8));
  int64_t* offsets = reinterpret_cast<int64_t*>(take((ns + 1) * 8));
  uint32_t* conn = reinterpret_cast<uint32_t*>(take(nc * nw * 4));
  double* elem = reinterpret_cast<double*>(take(nc * 8));
  float2* lp_conn = reinterpret_cast<float2*>(take(nc * 8));
  float2* lp = reinterpret_cast<float2*>(take(ns * 8));
  char* sscratch = sym ? take(symm_scratch_bytes(nc, nw, sym->nsymm)) : nullptr;
  const unsigned g = (unsigned)((ns + 127) / 128);
  rc_conn_count_kernel<<<g, 128, 0, st>>>(*op, spins, ns, net.N, counts);
  rc_scan_kernel<<<1, 1024, 0, st>>>(counts, ns, offsets);
  rc_conn_write_kernel<<<g, 128, 0, st>>>(*op, spins, ns, net.N, offsets, conn, elem);
  int rc = symm_forward(table, net, sym, spins, ns, nullptr, lp, sscratch, st);
  if (rc != QGX_OK) return rc;
  if ((rc = symm_forward(table, net, sym, conn, nc, offsets + ns, lp_conn, sscratch, st)) != QGX_OK) return rc;
  rc_eloc_reduce_kernel<<<g, 128, 0, st>>>(*op, spins, ns, net.N, lp, offsets, elem, lp_conn, eloc_re, eloc_im);
  return launch_status();
}

int jacobian_impl(const float* table, int32_t L, int32_t nblocks, int32_t channels, int32_t complex_out,
                  const SymmDev* sym, const uint32_t* spins, int64_t ns, float* O_re, float* O_im, int64_t ldo,
                  void* workspace, int64_t workspace_bytes, cudaStream_t st) {
  const ConvNet net = make_net(L, nblocks, channels, complex_out, QGX_CONV_FP32);
  char* ws = static_cast<char*>(workspace);
  int64_t scratch_bytes = workspace_bytes;
  SymmJac sj{nullptr, nullptr, nullptr, nullptr, 1};
  if (sym) {
    // log psi(T_g s) and log psi_symm(s) by the FP32 forward, then one backward per element
    const int nw = words_for(net.N);
    const int64_t sb = symm_scratch_bytes(ns, nw, sym->nsymm);
    float2* lp_sym = reinterpret_cast<float2*>(ws + sb);
    float2* lp_g = nullptr;
    const uint32_t* cfg = nullptr;
    int rc = symm_forward(table, net, sym, spins, ns, nullptr, lp_sym, ws, st, &lp_g, &cfg);
    if (rc != QGX_OK) return rc;
    sj = SymmJac{cfg, lp_g, lp_sym, sym->weight, sym->nsymm};
    ws += sb + al256(ns * 8);
    scratch_bytes -= sb + al256(ns * 8);
  }
  float* scratch = reinterpret_cast<float*>(ws);
  const int64_t sf = scratch_bytes / 4;
  switch (channels) {
    case 4: return launch_jacobian_c<4>(table, net, spins, ns, O_re, O_im, ldo, scratch, sf, sj, st);
    case 8: return launch_jacobian_c<8>(table, net, spins, ns, O_re, O_im, ldo, scratch, sf, sj, st);
    case 12: return launch_jacobian_c<12>(table, net, spins, ns, O_re, O_im, ldo, scratch, sf, sj, st);
    case 16: return launch_jacobian_c<16>(table, net, spins, ns, O_re, O_im, ldo, scratch, sf, sj, st);
    default: return QGX_ERR_UNSUPPORTED;
  }
}

}  // namespace
}  // namespace qgx

extern "C" {

int qgx_resconv_eloc(const float* table, int32_t L, int32_t nblocks, int32_t channels, int32_t complex_out,
                     int32_t conv_precision, const qgx_operator_t* op, const uint32_t* spins, int64_t ns, double* eloc_re, double* eloc_im,
                     void* workspace, int64_t workspace_bytes, qgx_stream_t stream) {
  QGX_CHECK_ARG(op && valid_net(L, nblocks, channels, complex_out) && valid_prec(conv_precision) && ns >= 0);
  if (ns == 0) return QGX_OK;
  QGX_CHECK_ARG(table && spins && eloc_re && workspace);
  QGX_CHECK_ARG(workspace_bytes >= qgx_resconv_eloc_workspace_bytes(L, ns, op->n_f1 + op->n_f2));
  QGX_CHECK_ARG((reinterpret_cast<uintptr_t>(workspace) & 255) == 0);
  return eloc_impl(table, make_net(L, nblocks, channels, complex_out, conv_precision), nullptr, op, spins, ns,
                   eloc_re, eloc_im, workspace, as_cuda(stream));
}

int64_t qgx_resconv_eloc_symm_workspace_bytes(int32_t L, int64_t ns, int32_t max_conn, int32_t nsymm) {
  if (L < 1 || ns < 1 || max_conn < 0 || nsymm < 1) return 0;
  const int64_t nc = ns * (int64_t)std::max(max_conn, 1);
  return qgx_resconv_eloc_workspace_bytes(L, ns, max_conn) + symm_scratch_bytes(nc, words_for(L * L), nsymm);
}

int qgx_resconv_eloc_symm(const float* table, int32_t L, int32_t nblocks, int32_t channels, int32_t complex_out,
                          int32_t conv_precision, const qgx_symm_t* symm, const qgx_operator_t* op,
                          const uint32_t* spins, int64_t ns, double* eloc_re, double* eloc_im, void* workspace,
                          int64_t workspace_bytes, qgx_stream_t stream) {
  SymmDev sym;
  QGX_CHECK_ARG(to_symm(symm, &sym));
  QGX_CHECK_ARG(op && valid_net(L, nblocks, channels, complex_out) && valid_prec(conv_precision) && ns >= 0);
  if (ns == 0) return QGX_OK;
  QGX_CHECK_ARG(table && spins && eloc_re && workspace);
  QGX_CHECK_ARG(workspace_bytes >= qgx_resconv_eloc_symm_workspace_bytes(L, ns, op->n_f1 + op->n_f2, sym.nsymm));
  QGX_CHECK_ARG((reinterpret_cast<uintptr_t>(workspace) & 255) == 0);
  return eloc_impl(table, make_net(L, nblocks, channels, complex_out, conv_precision), &sym, op, spins, ns,
                   eloc_re, eloc_im, workspace, as_cuda(stream));
}

int64_t qgx_resconv_log_psi_symm_workspace_bytes(int32_t L, int64_t ns, int32_t nsymm) {
  if (L < 1 || ns < 1 || nsymm < 1) return 0;
  return symm_scratch_bytes(ns, words_for(L * L), nsymm);
}

int qgx_resconv_log_psi_symm(const float* table, int32_t L, int32_t nblocks, int32_t channels, int32_t complex_out,
                             int32_t conv_precision, const qgx_symm_t* symm, const uint32_t* spins, int64_t ns,
                             float* log_psi, void* workspace, int64_t workspace_bytes, qgx_stream_t stream) {
  SymmDev sym;
  QGX_CHECK_ARG(to_symm(symm, &sym));
  QGX_CHECK_ARG(valid_net(L, nblocks, channels, complex_out) && valid_prec(conv_precision) && ns >= 0);
  if (ns == 0) return QGX_OK;
  QGX_CHECK_ARG(table && spins && log_psi && workspace);
  QGX_CHECK_ARG(workspace_bytes >= qgx_resconv_log_psi_symm_workspace_bytes(L, ns, sym.nsymm));
  QGX_CHECK_ARG((reinterpret_cast<uintptr_t>(workspace) & 255) == 0);
  const ConvNet net = make_net(L, nblocks, channels, complex_out, conv_precision);
  return symm_forward(table, net, &sym, spins, ns, nullptr, reinterpret_cast<float2*>(log_psi),
                      static_cast<char*>(workspace), as_cuda(stream));
}

int64_t qgx_resconv_jacobian_workspace_bytes(int32_t L, int32_t nblocks, int32_t channels) {
  if (L < 1 || nblocks < 1 || channels < 1) return 0;
  // per resident CTA: X_b and A_b of every block; sized for 4 CTAs on each of up to 160 SMs
  return 4LL * 160 * nblocks * 2 * channels * L * L * 4;
}

int qgx_resconv_jacobian(const float* table, int32_t L, int32_t nblocks, int32_t channels, int32_t complex_out,
                         const uint32_t* spins, int64_t ns, float* O_re, float* O_im, int64_t ldo, void* workspace,
                         int64_t workspace_bytes, qgx_stream_t stream) {
  QGX_CHECK_ARG(valid_net(L, nblocks, channels, complex_out) && ns >= 0);
  QGX_CHECK_ARG(ldo >= qgx_resconv_nparams(nblocks, channels));
  if (ns == 0) return QGX_OK;
  QGX_CHECK_ARG(table && spins && O_re && workspace && workspace_bytes > 0);
  QGX_CHECK_ARG(!(complex_out & QGX_RESCONV_COMPLEX) || O_im);
  return jacobian_impl(table, L, nblocks, channels, complex_out, nullptr, spins, ns, O_re, O_im, ldo, workspace,
                       workspace_bytes, as_cuda(stream));
}

int64_t qgx_resconv_jacobian_symm_workspace_bytes(int32_t L, int32_t nblocks, int32_t channels, int64_t ns,
                                                  int32_t nsymm) {
  if (L < 1 || nblocks < 1 || channels < 1 || ns < 1 || nsymm < 1) return 0;
  return symm_scratch_bytes(ns, words_for(L * L), nsymm) + al256(ns * 8) +
         qgx_resconv_jacobian_workspace_bytes(L, nblocks, channels);
}

int qgx_resconv_jacobian_symm(const float* table, int32_t L, int32_t nblocks, int32_t channels, int32_t complex_out,
                              const qgx_symm_t* symm, const uint32_t* spins, int64_t ns, float* O_re, float* O_im,
                              int64_t ldo, void* workspace, int64_t workspace_bytes, qgx_stream_t stream) {
  SymmDev sym;
  QGX_CHECK_ARG(to_symm(symm, &sym));
  QGX_CHECK_ARG(valid_net(L, nblocks, channels, complex_out) && ns >= 0);
  QGX_CHECK_ARG(ldo >= qgx_resconv_nparams(nblocks, channels));
  if (ns == 0) return QGX_OK;
  QGX_CHECK_ARG(table && spins && O_re && workspace);
  QGX_CHECK_ARG(!(complex_out & QGX_RESCONV_COMPLEX) || O_im);
  QGX_CHECK_ARG(workspace_bytes >= qgx_resconv_jacobian_symm_workspace_bytes(L, nblocks, channels, ns, sym.nsymm));
  QGX_CHECK_ARG((reinterpret_cast<uintptr_t>(workspace) & 255) == 0);
  return jacobian_impl(table, L, nblocks, channels, complex_out, &sym, spins, ns, O_re, O_im, ldo, workspace,
                       workspace_bytes, as_cuda(stream));
}

// ---- the projected RBM: psi_symm(s) = sum_g w_g psi(T_g s) for RBM_Dense (symmetry.py:325-392 on
// any model, variational.py:261-266); the images run through the RBM forward and closed-form
// log-derivatives, everything else is the ResConv projection's pipeline
int64_t qgx_rbm_log_psi_symm_workspace_bytes(int32_t n, int64_t ns, int32_t nsymm) {
  if (n < 1 || ns < 1 || nsymm < 1) return 0;
  return symm_scratch_bytes(ns, words_for(n), nsymm);
}

int qgx_rbm_log_psi_symm(const float* table, int32_t n, int32_t m, const qgx_symm_t* symm, const uint32_t* spins,
                         int64_t ns, float* log_psi, void* workspace, int64_t workspace_bytes, qgx_stream_t stream) {
  SymmDev sym;
  QGX_CHECK_ARG(to_symm(symm, &sym));
  QGX_CHECK_ARG(valid_rbm_symm(n, m) && ns >= 0);
  if (ns == 0) return QGX_OK;
  QGX_CHECK_ARG(table && spins && log_psi && workspace);
  QGX_CHECK_ARG(workspace_bytes >= qgx_rbm_log_psi_symm_workspace_bytes(n, ns, sym.nsymm));
  QGX_CHECK_ARG((reinterpret_cast<uintptr_t>(workspace) & 255) == 0);
  return symm_forward(table, make_rbm_net(n, m, 0), &sym, spins, ns, nullptr, reinterpret_cast<float2*>(log_psi),
                      static_cast<char*>(workspace), as_cuda(stream));
}

int64_t qgx_rbm_sweep_symm_workspace_bytes(int32_t n, int64_t ns, int32_t nsymm) {
  if (n < 1 || ns < 1 || nsymm < 1) return 0;
  return sweep_scratch_bytes(n, ns) + symm_scratch_bytes(ns, words_for(n), nsymm);
}

int qgx_rbm_sweep_symm(const float* table, int32_t n, int32_t m, const qgx_symm_t* symm, uint32_t* spins,
                       float* log_psi, int32_t* accepts, int64_t ns, int32_t nsteps, uint64_t seed, uint64_t step0,
                       float reweight, int32_t proposal, const int32_t* nbr, int32_t z, int32_t hop, void* workspace,
                       int64_t workspace_bytes, qgx_stream_t stream) {
  SymmDev sym;
  QGX_CHECK_ARG(to_symm(symm, &sym));
  QGX_CHECK_ARG(valid_rbm_symm(n, m) && ns >= 0 && nsteps >= 0);
  QGX_CHECK_ARG(proposal == QGX_PROPOSAL_LOCAL_FLIP || proposal == QGX_PROPOSAL_SPIN_EXCHANGE);
  if (proposal == QGX_PROPOSAL_SPIN_EXCHANGE) QGX_CHECK_ARG(nbr && z > 0 && (hop == 1 || hop == -1));
  if (ns == 0) return QGX_OK;
  QGX_CHECK_ARG(table && spins && log_psi && workspace);
  QGX_CHECK_ARG(workspace_bytes >= qgx_rbm_sweep_symm_workspace_bytes(n, ns, sym.nsymm));
  QGX_CHECK_ARG((reinterpret_cast<uintptr_t>(workspace) & 255) == 0);
  return sweep_impl(table, make_rbm_net(n, m, 0), 0, &sym, spins, log_psi, accepts, ns, nsteps, seed, step0,
                    reweight, proposal, nbr, z, hop, workspace, as_cuda(stream));
}

int64_t qgx_rbm_eloc_symm_workspace_bytes(int32_t n, int64_t ns, int32_t max_conn, int32_t nsymm) {
  if (n < 1 || ns < 1 || max_conn < 0 || nsymm < 1) return 0;
  const int64_t nc = ns * (int64_t)std::max(max_conn, 1);
  return eloc_scratch_bytes(n, ns, max_conn) + symm_scratch_bytes(nc, words_for(n), nsymm);
}

int qgx_rbm_eloc_symm(const float* table, int32_t n, int32_t m, const qgx_symm_t* symm, const qgx_operator_t* op,
                      const uint32_t* spins, int64_t ns, double* eloc_re, double* eloc_im, void* workspace,
                      int64_t workspace_bytes, qgx_stream_t stream) {
  SymmDev sym;
  QGX_CHECK_ARG(to_symm(symm, &sym));
  QGX_CHECK_ARG(op && valid_rbm_symm(n, m) && ns >= 0);
  if (ns == 0) return QGX_OK;
  QGX_CHECK_ARG(table && spins && eloc_re && workspace);
  QGX_CHECK_ARG(workspace_bytes >= qgx_rbm_eloc_symm_workspace_bytes(n, ns, op->n_f1 + op->n_f2, sym.nsymm));
  QGX_CHECK_ARG((reinterpret_cast<uintptr_t>(workspace) & 255) == 0);
  return eloc_impl(table, make_rbm_net(n, m, 0), &sym, op, spins, ns, eloc_re, eloc_im, workspace, as_cuda(stream));
}

int64_t qgx_rbm_jacobian_symm_workspace_bytes(int32_t n, int32_t m, int32_t has_vbias, int64_t ns, int32_t nsymm) {
  if (n < 1 || m < 1 || ns < 1 || nsymm < 1) return 0;
  const int64_t np = (int64_t)m * n + m + (has_vbias ? n : 0);
  return symm_scratch_bytes(ns, words_for(n), nsymm) + al256(ns * 8) +
         al256(rbm_symm_chunk(ns, nsymm, np) * nsymm * np * 4);
}

int qgx_rbm_jacobian_symm(const float* table, int32_t n, int32_t m, int32_t has_vbias, const qgx_symm_t* symm,
                          const uint32_t* spins, int64_t ns, float* O_re, float* O_im, int64_t ldo, void* workspace,
                          int64_t workspace_bytes, qgx_stream_t stream) {
  SymmDev sym;
  QGX_CHECK_ARG(to_symm(symm, &sym));
  QGX_CHECK_ARG(valid_rbm_symm(n, m) && ns >= 0);
  const int64_t np = (int64_t)m * n + m + (has_vbias ? n : 0);
  QGX_CHECK_ARG(ldo >= np);
  if (ns == 0) return QGX_OK;
  QGX_CHECK_ARG(table && spins && O_re && workspace);
  QGX_CHECK_ARG(workspace_bytes >= qgx_rbm_jacobian_symm_workspace_bytes(n, m, has_vbias, ns, sym.nsymm));
  QGX_CHECK_ARG((reinterpret_cast<uintptr_t>(workspace) & 255) == 0);
  cudaStream_t st = as_cuda(stream);
  const int nw = words_for(n);
  char* ws = static_cast<char*>(workspace);
  const int64_t sb = symm_scratch_bytes(ns, nw, sym.nsymm);
  float2* lp_sym = reinterpret_cast<float2*>(ws + sb);
  float* rows = reinterpret_cast<float*>(ws + sb + al256(ns * 8));
  float2* lp_g = nullptr;
  const uint32_t* cfg = nullptr;
  int rc = symm_forward(table, make_rbm_net(n, m, has_vbias), &sym, spins, ns, nullptr, lp_sym, ws, st, &lp_g, &cfg);
  if (rc != QGX_OK) return rc;
  const int64_t cs = rbm_symm_chunk(ns, sym.nsymm, np);
  const unsigned gx = (unsigned)std::min<int64_t>((np + 255) / 256, 1024);
  for (int64_t c0 = 0; c0 < ns; c0 += cs) {
    const int64_t cn = std::min(cs, ns - c0);
    rc = rbm_jacobian_rows(table, n, m, has_vbias, cfg + c0 * sym.nsymm * nw, cn * sym.nsymm, rows, np, st);
    if (rc != QGX_OK) return rc;
    rbm_symm_rows_kernel<<<dim3(gx, (unsigned)cn), 256, sym.nsymm * sizeof(float2), st>>>(
        rows, np, c0, sym.nsymm, lp_g, lp_sym, sym.weight, O_re, O_im, ldo);
    if ((rc = launch_status()) != QGX_OK) return rc;
  }
  return QGX_OK;
}

}  // extern "C"
