// Library plumbing, Philox known-answer entry, configuration init / packing, diagonal
// operator terms, energy statistics, reweighting, column centring and the guarded
// parameter update.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "qgx_colstats.cuh"
#include "qgx_common.cuh"

namespace qgx {

static thread_local char g_last_error[256] = {0};

void set_last_error(cudaError_t e) {
  std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s", cudaGetErrorName(e), cudaGetErrorString(e));
}

void set_last_message(const char* msg) { std::snprintf(g_last_error, sizeof(g_last_error), "%s", msg); }

int launch_status() {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_error(e);
    return QGX_ERR_CUDA;
  }
  return QGX_OK;
}

int device_sm_count() {
  int dev = 0, v = kNumSMs;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
  return v;
}

int device_max_smem_optin() {
  int dev = 0, v = 48 * 1024;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return v;
}

// ---- Philox KAT ------------------------------------------------------------------------
__global__ void philox_kernel(const uint32_t* __restrict__ ctr, const uint32_t* __restrict__ key,
                              uint32_t* __restrict__ out, int64_t n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  u32x4 c{ctr[4 * i], ctr[4 * i + 1], ctr[4 * i + 2], ctr[4 * i + 3]};
  u32x4 r = philox4x32_10(c, key[0], key[1]);
  out[4 * i] = r.x;
  out[4 * i + 1] = r.y;
  out[4 * i + 2] = r.z;
  out[4 * i + 3] = r.w;
}

// ---- configurations ---------------------------------------------------------------------
// word w of chain c = word (w % 4) of draw(seed, c, w / 4, kTagInit); bits >= n cleared
__global__ void init_uniform_kernel(uint32_t* __restrict__ spins, int64_t ns, int n, uint64_t seed) {
  const int nw = words_for(n);
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= ns * nw) return;
  const int64_t c = i / nw;
  const int w = (int)(i % nw);
  u32x4 r = draw(seed, (uint64_t)c, (uint64_t)(w >> 2), kTagInit);
  uint32_t v = (w & 3) == 0 ? r.x : (w & 3) == 1 ? r.y : (w & 3) == 2 ? r.z : r.w;
  const int rem = n - 32 * w;
  if (rem < 32) v &= (1u << rem) - 1u;
  spins[i] = v;
}

constexpr int kMaxInitWords = 32;  // n <= 1024 for the fixed-magnetisation init

// sites 0..nup-1 up, then Fisher-Yates: for i = n-1..1, j = bounded(draw(c, i).x, i+1), swap
__global__ void init_fixed_up_kernel(uint32_t* __restrict__ spins, int64_t ns, int n, int nup, uint64_t seed) {
  int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= ns) return;
  const int nw = words_for(n);
  uint32_t w[kMaxInitWords];
  for (int k = 0; k < nw; ++k) {
    const int lo = 32 * k;
    int cnt = nup - lo;
    cnt = cnt < 0 ? 0 : (cnt > 32 ? 32 : cnt);
    w[k] = cnt == 32 ? 0xFFFFFFFFu : ((1u << cnt) - 1u);
  }
  for (int i = n - 1; i > 0; --i) {
    u32x4 r = draw(seed, (uint64_t)c, (uint64_t)i, kTagInitPerm);
    const int j = (int)bounded(r.x, (uint32_t)(i + 1));
    const uint32_t bi = (w[i >> 5] >> (i & 31)) & 1u;
    const uint32_t bj = (w[j >> 5] >> (j & 31)) & 1u;
    if (bi != bj) {
      w[i >> 5] ^= 1u << (i & 31);
      w[j >> 5] ^= 1u << (j & 31);
    }
  }
  for (int k = 0; k < nw; ++k) spins[c * nw + k] = w[k];
}

__global__ void unpack_kernel(const uint32_t* __restrict__ spins, int8_t* __restrict__ out, int64_t ns, int n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= ns * n) return;
  const int nw = words_for(n);
  const int64_t c = i / n;
  const int j = (int)(i % n);
  out[i] = ((spins[c * nw + (j >> 5)] >> (j & 31)) & 1u) ? (int8_t)1 : (int8_t)-1;
}

__global__ void pack_kernel(const int8_t* __restrict__ in, uint32_t* __restrict__ spins, int64_t ns, int n) {
  const int nw = words_for(n);
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= ns * nw) return;
  const int64_t c = i / nw;
  const int w = (int)(i % nw);
  uint32_t v = 0;
  for (int b = 0; b < 32 && 32 * w + b < n; ++b) v |= (in[c * n + 32 * w + b] > 0 ? 1u : 0u) << b;
  spins[i] = v;
}

// ---- diagonal operator part -----------------------------------------------------------
__device__ inline int spin_pm(const uint32_t* s, int i) { return ((s[i >> 5] >> (i & 31)) & 1u) ? 1 : -1; }

__global__ void operator_diag_kernel(qgx_operator_t op, const uint32_t* __restrict__ spins, int64_t ns, int n,
                                     double* __restrict__ out) {
  int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= ns) return;
  const uint32_t* s = spins + c * words_for(n);
  double e = op.c0;
  for (int k = 0; k < op.n_z; ++k) e += op.z_J[k] * spin_pm(s, op.z_i[k]);
  for (int k = 0; k < op.n_zz; ++k) e += op.zz_J[k] * (spin_pm(s, op.zz_ij[2 * k]) * spin_pm(s, op.zz_ij[2 * k + 1]));
  out[c] = e;
}

// ---- block reductions -------------------------------------------------------------------
template <int NT>
__device__ inline double block_sum(double v, double* sh) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double r = 0.0;
  if (wid == 0) {
    r = lane < NT / 32 ? sh[lane] : 0.0;
    r = warp_sum(r);
    if (lane == 0) sh[0] = r;
  }
  __syncthreads();
  r = sh[0];
  __syncthreads();
  return r;
}

// Compensated sum over a block: each thread holds a Neumaier (s, c) pair.
template <int NT>
__device__ inline double block_ksum(const KahanD& k, double* sh) {
  // sum the high parts with error compensation tracked through the low parts
  double hi = block_sum<NT>(k.s, sh);
  double lo = block_sum<NT>(k.c, sh);
  return hi + lo;
}

constexpr int kStatThreads = 1024;

// Single-block energy statistics (quantax/optimizer/sr.py:180-195).
__global__ void __launch_bounds__(kStatThreads) energy_stats_kernel(const double* __restrict__ er, const double* __restrict__ ei,
                                                                   const double* __restrict__ r, int64_t ns,
                                                                   double* __restrict__ stats, double* __restrict__ ebr,
                                                                   double* __restrict__ ebi) {
  __shared__ double sh[32];
  KahanD swr, swi, sur, sui;
  for (int64_t i = threadIdx.x; i < ns; i += kStatThreads) {
    const double w = r ? r[i] : 1.0;
    const double a = er[i];
    const double b = ei ? ei[i] : 0.0;
    swr.add(a * w);
    swi.add(b * w);
    sur.add(a);
    sui.add(b);
  }
  const double inv = 1.0 / (double)ns;
  const double emr = block_ksum<kStatThreads>(swr, sh) * inv;
  const double emi = block_ksum<kStatThreads>(swi, sh) * inv;
  const double mur = block_ksum<kStatThreads>(sur, sh) * inv;
  const double mui = block_ksum<kStatThreads>(sui, sh) * inv;
  KahanD sv;
  for (int64_t i = threadIdx.x; i < ns; i += kStatThreads) {
    const double w = r ? r[i] : 1.0;
    const double a = er[i], b = ei ? ei[i] : 0.0;
    const double da = a - emr, db = b - emi;
    sv.add((da * da + db * db) * w);
    const double f = sqrt(w * inv);
    ebr[i] = (a - mur) * f;
    if (ebi) ebi[i] = (b - mui) * f;
  }
  const double var = block_ksum<kStatThreads>(sv, sh) * inv;
  if (threadIdx.x == 0) {
    stats[0] = emr;
    stats[1] = emi;
    stats[2] = var;
  }
}

// r_s = |psi_s|^(2-n) / mean = exp(x_s - xmax) / mean(exp(x - xmax)), x = (2-n) log|psi|
__global__ void __launch_bounds__(kStatThreads) reweight_kernel(const float* __restrict__ lp, int64_t ns, float n,
                                                               double* __restrict__ r) {
  __shared__ double sh[32];
  const double p = 2.0 - (double)n;
  double mx = -INFINITY;
  for (int64_t i = threadIdx.x; i < ns; i += kStatThreads) mx = fmax(mx, p * (double)lp[i]);
  // block max
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = sh[threadIdx.x];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (threadIdx.x == 0) sh[0] = v;
  }
  __syncthreads();
  mx = sh[0];
  __syncthreads();
  KahanD s;
  for (int64_t i = threadIdx.x; i < ns; i += kStatThreads) s.add(exp(p * (double)lp[i] - mx));
  const double mean = block_ksum<kStatThreads>(s, sh) / (double)ns;
  for (int64_t i = threadIdx.x; i < ns; i += kStatThreads) r[i] = exp(p * (double)lp[i] - mx) / mean;
}

// ---- column centring ------------------------------------------------------------------
constexpr int kColThreads = 256;
constexpr int kColRows = 128;  // rows per partial-sum chunk

// per column and chunk of kColRows rows: sum of O and of r O, as float-pair sums (DSum)
__global__ void col_partial_kernel(const float* __restrict__ O, int64_t ns, int64_t np, int64_t ldo,
                                   const double* __restrict__ r, double* __restrict__ part_u,
                                   double* __restrict__ part_w) {
  __shared__ float2 rs[kColRows];
  const int64_t chunk = blockIdx.y;
  const int64_t r0 = chunk * kColRows;
  const int64_t r1 = min(ns, r0 + kColRows);
  for (int64_t s = r0 + threadIdx.x; s < r1; s += blockDim.x) rs[s - r0] = split_double(r ? r[s] : 1.0);
  __syncthreads();
  const int64_t col = blockIdx.x * (int64_t)kColThreads + threadIdx.x;
  if (col >= np) return;
  DSum su, sw;
  for (int64_t s = r0; s < r1; ++s) {
    const float v = O[s * ldo + col];
    su.add(v);
    const float2 rv = rs[s - r0];
    sw.add_prod(v, rv.x, rv.y);
  }
  part_u[chunk * np + col] = su.value();
  part_w[chunk * np + col] = sw.value();
}

// O[s][col] <- (O[s][col] - mean[col]) sqrt(r_s / ns) in FP32: the mean enters as two floats
// (hi + lo), so the difference is within about two ulps of the FP64-computed one. A CTA takes
// whole rows (grid-stride over rows); VEC: rows start 16-byte aligned and are read and written
// four columns at a time
__device__ inline float center_one(float v, float2 m, float f) { return __fmul_rn(__fsub_rn(__fsub_rn(v, m.x), m.y), f); }

template <bool VEC>
__global__ void __launch_bounds__(256) col_center_kernel(float* __restrict__ O, int64_t ns, int64_t np, int64_t ldo,
                                                         const double* __restrict__ r,
                                                         const float2* __restrict__ mean2) {
  for (int64_t s = blockIdx.x; s < ns; s += gridDim.x) {
    const float f = (float)sqrt((r ? r[s] : 1.0) / (double)ns);
    float* row = O + s * ldo;
    int64_t done = 0;
    if (VEC) {
      float4* row4 = reinterpret_cast<float4*>(row);
      const int64_t n4 = np / 4;
      for (int64_t c = threadIdx.x; c < n4; c += blockDim.x) {
        float4 v = row4[c];
        const float2* m = mean2 + 4 * c;
        v.x = center_one(v.x, m[0], f);
        v.y = center_one(v.y, m[1], f);
        v.z = center_one(v.z, m[2], f);
        v.w = center_one(v.w, m[3], f);
        row4[c] = v;
      }
      done = n4 * 4;
    }
    for (int64_t col = done + threadIdx.x; col < np; col += blockDim.x) row[col] = center_one(row[col], mean2[col], f);
  }
}

__global__ void split_mean_kernel(const double* __restrict__ mean_u, int64_t np, float2* __restrict__ mean2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np; i += (int64_t)gridDim.x * blockDim.x)
    mean2[i] = split_double(mean_u[i]);
}

// out[col] = sum_s A[s][col]^2 as float-pair sums (diag(A^T A), the relative shift of
// lstsq_shift_cg, solver.py:32-36); one thread per column, rows in chunks of kColRows
__global__ void col_sumsq_kernel(const float* __restrict__ A, int64_t rows, int64_t cols, int64_t lda,
                                 double* __restrict__ part) {
  const int64_t col = blockIdx.x * (int64_t)kColThreads + threadIdx.x;
  if (col >= cols) return;
  const int64_t r0 = (int64_t)blockIdx.y * kColRows, r1 = min(rows, r0 + kColRows);
  DSum acc;
  for (int64_t s = r0; s < r1; ++s) {
    const float v = A[s * lda + col];
    acc.add_prod(v, v, 0.0f);
  }
  part[blockIdx.y * cols + col] = acc.value();
}

__global__ void col_sum_parts_kernel(const double* __restrict__ part, int64_t nchunk, int64_t cols,
                                     double* __restrict__ out) {
  const int64_t col = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (col >= cols) return;
  double s = 0.0;
  for (int64_t c = 0; c < nchunk; ++c) s += part[c * cols + col];
  out[col] = s;
}

// ---- guarded update ---------------------------------------------------------------------
__global__ void finite_check_kernel(const double* __restrict__ step, int64_t np, int32_t* __restrict__ flag) {
  bool bad = false;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np; i += (int64_t)gridDim.x * blockDim.x)
    bad |= !isfinite(step[i]);
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

__global__ void update_kernel(float* __restrict__ params, const double* __restrict__ step, int64_t np,
                              const int32_t* __restrict__ flag) {
  if (*flag) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np; i += (int64_t)gridDim.x * blockDim.x)
    params[i] = params[i] - (float)step[i];  // f32(params) - f32(step), as variational.py:574-579
}

inline unsigned blocks_for(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

// y = A x: A FP32 (rows x cols, lda), x and y FP64; one warp per row, FP64 accumulation in a
// fixed order (the momentum term Obar @ step of SPRING / MARCH / AdamSR, sr.py:244, 315, 415)
__global__ void obar_matvec_kernel(const float* __restrict__ A, int64_t rows, int64_t cols, int64_t lda,
                                   const double* __restrict__ x, double* __restrict__ y) {
  const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= rows) return;
  const float* a = A + row * lda;
  double s = 0.0;
  for (int64_t j = lane; j < cols; j += 32) s = fma((double)a[j], x[j], s);
  s = warp_sum(s);
  if (lane == 0) y[row] = s;
}

// A[:, j] <- A[:, j] * s_j in place (MARCH / AdamSR divide Obar by V, sr.py:323, 418)
__global__ void scale_columns_kernel(float* __restrict__ A, int64_t rows, int64_t cols, int64_t lda,
                                     const double* __restrict__ s) {
  const int64_t row = blockIdx.y;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < cols; j += (int64_t)gridDim.x * blockDim.x)
    A[row * lda + j] = (float)((double)A[row * lda + j] * s[j]);
}

// ---- exact sampling over a whole basis (sampler.py:72-119) --------------------------------
// idx[i] = the first j with cdf[j] > u_i cdf[dim - 1], u_i the 53-bit uniform of draw
// (seed, i, step, kTagExact): sample i of a sweep taken with probability p_j = cdf[j] - cdf[j-1]
// (a j with p_j = 0 is never taken). cdf holds inclusive prefix sums.
__global__ void exact_draw_kernel(const double* __restrict__ cdf, int64_t dim, int64_t ns, uint64_t seed,
                                  uint64_t step, int64_t* __restrict__ idx) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= ns) return;
  const u32x4 w = draw(seed, (uint64_t)i, step, kTagExact);
  const double target = unit_double(w.x, w.y) * cdf[dim - 1];
  int64_t lo = 0, hi = dim - 1;  // the answer lies in [lo, hi]: cdf[dim - 1] > target
  while (lo < hi) {
    const int64_t mid = lo + (hi - lo) / 2;
    if (cdf[mid] > target)
      hi = mid;
    else
      lo = mid + 1;
  }
  idx[i] = lo;
}

// ---- exact reconfiguration over a whole basis (sr.py:432-513) ---------------------------
// y[r][c] = sum over row r's entries e of val[e] x[col[e]][c], c < nvec (1: real vectors,
// 2: complex ones as (re, im) pairs). One warp per row, FP64; a column index outside
// [0, nrows) is skipped.
__global__ void csr_matvec_kernel(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                  const double* __restrict__ val, int64_t nrows, const double* __restrict__ x,
                                  int nvec, double* __restrict__ y) {
  const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= nrows) return;  // whole warps: 256-thread blocks hold 8 rows
  double s0 = 0.0, s1 = 0.0;
  const int64_t e1 = rowptr[row + 1];
  for (int64_t e = rowptr[row] + lane; e < e1; e += 32) {
    const int64_t c = col[e];
    if (c < 0 || c >= nrows) continue;
    s0 = fma(val[e], x[c * nvec], s0);
    if (nvec == 2) s1 = fma(val[e], x[c * 2 + 1], s1);
  }
  s0 = warp_sum(s0);
  s1 = warp_sum(s1);
  if (lane == 0) {
    y[row * nvec] = s0;
    if (nvec == 2) y[row * 2 + 1] = s1;
  }
}

// Omat = psi_s O_s in place (variational.py jacobian times psi, sr.py:500-501). Real psi:
// O (ns x cols). Complex psi ((re, im) pairs): O holds [Re O; Im O] (2 ns rows). A NaN
// product becomes 0, both parts of a complex one, as jnp.where(isnan(Omat), 0, Omat) does.
__global__ void er_weight_rows_kernel(float* __restrict__ O, int64_t ns, int64_t cols, int64_t ldo,
                                      const double* __restrict__ psi, int cplx) {
  for (int64_t row = blockIdx.y; row < ns; row += gridDim.y) {
    float* a = O + row * ldo;
    if (!cplx) {
      const double p = psi[row];
      for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < cols; j += (int64_t)gridDim.x * blockDim.x) {
        const double v = (double)a[j] * p;
        a[j] = isnan(v) ? 0.f : (float)v;
      }
    } else {
      float* b = O + (row + ns) * ldo;
      const double pr = psi[2 * row], pi = psi[2 * row + 1];
      for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < cols; j += (int64_t)gridDim.x * blockDim.x) {
        const double re = (double)a[j] * pr - (double)b[j] * pi;
        const double im = (double)a[j] * pi + (double)b[j] * pr;
        const bool bad = isnan(re) || isnan(im);
        a[j] = bad ? 0.f : (float)re;
        b[j] = bad ? 0.f : (float)im;
      }
    }
  }
}

// Obar = Omat - psi Omean^T in place (sr.py:503-504); complex: Omean as cols real parts then
// cols imaginary parts, the product psi_s Omean_k complex.
__global__ void er_center_kernel(float* __restrict__ O, int64_t ns, int64_t cols, int64_t ldo,
                                 const double* __restrict__ psi, int cplx, const double* __restrict__ omean) {
  for (int64_t row = blockIdx.y; row < ns; row += gridDim.y) {
    float* a = O + row * ldo;
    if (!cplx) {
      const double p = psi[row];
      for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < cols; j += (int64_t)gridDim.x * blockDim.x)
        a[j] = (float)((double)a[j] - p * omean[j]);
    } else {
      float* b = O + (row + ns) * ldo;
      const double pr = psi[2 * row], pi = psi[2 * row + 1];
      for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < cols; j += (int64_t)gridDim.x * blockDim.x) {
        const double mr = omean[j], mi = omean[cols + j];
        a[j] = (float)((double)a[j] - (pr * mr - pi * mi));
        b[j] = (float)((double)b[j] - (pr * mi + pi * mr));
      }
    }
  }
}

// psi from local updates against a direct forward (Metropolis.sweep, metropolis.py:201-213):
// close when |psi_l - psi_d| < 1e-8 or |psi_l / psi_d - 1| < 1e-3. On log|psi| the ratio test
// is log1p(-1e-3) < lp_l - lp_d < log1p(1e-3); the absolute test matters only for amplitudes
// near 1e-8 and is evaluated in FP32. Counts the configurations that are neither (into a
// zeroed *count) and, when out is given, writes the direct values there (out may be local).
__global__ void log_psi_mismatch_kernel(const float* local, const float* __restrict__ direct, int64_t ns,
                                        int32_t* __restrict__ count, float* out) {
  __shared__ int sh[32];
  int c = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ns; i += (int64_t)gridDim.x * blockDim.x) {
    const float l = local[i], d = direct[i];
    const float x = l - d;
    const bool close_rel = x > -1.00050033358e-3f && x < 9.99500333084e-4f;
    const bool close_abs = fabsf(__expf(l) - __expf(d)) < 1e-8f;
    c += (close_rel || close_abs) ? 0 : 1;
    if (out) out[i] = d;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
    if (t) atomicAdd(count, t);  // integer sums: the total does not depend on the order
  }
}

}  // namespace qgx

using namespace qgx;

extern "C" {

int qgx_obar_matvec(const float* A, int64_t rows, int64_t cols, int64_t lda, const double* x, double* y,
                    qgx_stream_t stream) {
  QGX_CHECK_ARG(rows >= 0 && cols >= 0 && lda >= cols);
  if (rows == 0) return QGX_OK;
  QGX_CHECK_ARG(A && x && y);
  obar_matvec_kernel<<<blocks_for(rows * 32, 256), 256, 0, as_cuda(stream)>>>(A, rows, cols, lda, x, y);
  return launch_status();
}

int qgx_scale_columns(float* A, int64_t rows, int64_t cols, int64_t lda, const double* s, qgx_stream_t stream) {
  QGX_CHECK_ARG(rows >= 0 && cols >= 0 && lda >= cols);
  if (rows == 0 || cols == 0) return QGX_OK;
  QGX_CHECK_ARG(A && s);
  cudaStream_t st = as_cuda(stream);
  const unsigned gx = (unsigned)std::min<int64_t>((cols + 255) / 256, 64);
  for (int64_t r0 = 0; r0 < rows; r0 += 65535) {
    const int64_t rr = std::min<int64_t>(65535, rows - r0);
    scale_columns_kernel<<<dim3(gx, (unsigned)rr), 256, 0, st>>>(A + r0 * lda, rr, cols, lda, s);
  }
  return launch_status();
}

int qgx_exact_draw(const double* cdf, int64_t dim, int64_t ns, uint64_t seed, uint64_t step, int64_t* idx,
                   qgx_stream_t stream) {
  QGX_CHECK_ARG(dim > 0 && ns >= 0);
  if (ns == 0) return QGX_OK;
  QGX_CHECK_ARG(cdf && idx);
  exact_draw_kernel<<<blocks_for(ns, 256), 256, 0, as_cuda(stream)>>>(cdf, dim, ns, seed, step, idx);
  return launch_status();
}

int qgx_csr_matvec(const int64_t* rowptr, const int32_t* col, const double* val, int64_t nrows, const double* x,
                   int nvec, double* y, qgx_stream_t stream) {
  QGX_CHECK_ARG(nrows >= 0 && (nvec == 1 || nvec == 2));
  if (nrows == 0) return QGX_OK;
  QGX_CHECK_ARG(rowptr && col && val && x && y);
  csr_matvec_kernel<<<blocks_for(nrows * 32, 256), 256, 0, as_cuda(stream)>>>(rowptr, col, val, nrows, x, nvec, y);
  return launch_status();
}

static dim3 er_grid(int64_t ns, int64_t cols) {
  return dim3((unsigned)std::min<int64_t>((cols + 255) / 256, 64), (unsigned)std::min<int64_t>(ns, 65535));
}

int qgx_er_weight_rows(float* O, int64_t ns, int64_t cols, int64_t ldo, const double* psi, int cplx,
                       qgx_stream_t stream) {
  QGX_CHECK_ARG(ns >= 0 && cols >= 0 && ldo >= cols);
  if (ns == 0 || cols == 0) return QGX_OK;
  QGX_CHECK_ARG(O && psi);
  er_weight_rows_kernel<<<er_grid(ns, cols), 256, 0, as_cuda(stream)>>>(O, ns, cols, ldo, psi, cplx != 0);
  return launch_status();
}

int qgx_er_center(float* O, int64_t ns, int64_t cols, int64_t ldo, const double* psi, int cplx,
                  const double* omean, qgx_stream_t stream) {
  QGX_CHECK_ARG(ns >= 0 && cols >= 0 && ldo >= cols);
  if (ns == 0 || cols == 0) return QGX_OK;
  QGX_CHECK_ARG(O && psi && omean);
  er_center_kernel<<<er_grid(ns, cols), 256, 0, as_cuda(stream)>>>(O, ns, cols, ldo, psi, cplx != 0, omean);
  return launch_status();
}

int qgx_abi_version(void) { return 1; }

const char* qgx_status_string(int status) {
  switch (status) {
    case QGX_OK: return "ok";
    case QGX_ERR_ARG: return "invalid argument";
    case QGX_ERR_CUDA: return "CUDA error";
    case QGX_ERR_TIMEOUT: return "device wait timed out";
    case QGX_ERR_NONFINITE: return "non-finite value";
    case QGX_ERR_UNSUPPORTED: return "unsupported configuration";
    case QGX_ERR_SOLVER: return "cuSOLVER error";
    default: return "unknown status";
  }
}

const char* qgx_last_error(void) { return g_last_error; }

void qgx_clear_last_error(void) { g_last_error[0] = 0; }

int qgx_philox4x32_10(const uint32_t* ctr, const uint32_t* key, uint32_t* out, int64_t n, qgx_stream_t stream) {
  QGX_CHECK_ARG(n >= 0);
  if (n == 0) return QGX_OK;
  QGX_CHECK_ARG(ctr && key && out);
  philox_kernel<<<blocks_for(n, 256), 256, 0, as_cuda(stream)>>>(ctr, key, out, n);
  return launch_status();
}

int qgx_spins_init_uniform(uint32_t* spins, int64_t ns, int32_t n, uint64_t seed, qgx_stream_t stream) {
  QGX_CHECK_ARG(ns >= 0 && n > 0);
  if (ns == 0) return QGX_OK;
  QGX_CHECK_ARG(spins);
  const int64_t tot = ns * words_for(n);
  init_uniform_kernel<<<blocks_for(tot, 256), 256, 0, as_cuda(stream)>>>(spins, ns, n, seed);
  return launch_status();
}

int qgx_spins_init_fixed_up(uint32_t* spins, int64_t ns, int32_t n, int32_t nup, uint64_t seed, qgx_stream_t stream) {
  QGX_CHECK_ARG(ns >= 0 && n > 0 && n <= 32 * kMaxInitWords && nup >= 0 && nup <= n);
  if (ns == 0) return QGX_OK;
  QGX_CHECK_ARG(spins);
  init_fixed_up_kernel<<<blocks_for(ns, 128), 128, 0, as_cuda(stream)>>>(spins, ns, n, nup, seed);
  return launch_status();
}

int qgx_spins_unpack(const uint32_t* spins, int8_t* out, int64_t ns, int32_t n, qgx_stream_t stream) {
  QGX_CHECK_ARG(ns >= 0 && n > 0);
  if (ns == 0) return QGX_OK;
  QGX_CHECK_ARG(spins && out);
  unpack_kernel<<<blocks_for(ns * n, 256), 256, 0, as_cuda(stream)>>>(spins, out, ns, n);
  return launch_status();
}

int qgx_spins_pack(const int8_t* in, uint32_t* spins, int64_t ns, int32_t n, qgx_stream_t stream) {
  QGX_CHECK_ARG(ns >= 0 && n > 0);
  if (ns == 0) return QGX_OK;
  QGX_CHECK_ARG(spins && in);
  pack_kernel<<<blocks_for(ns * words_for(n), 256), 256, 0, as_cuda(stream)>>>(in, spins, ns, n);
  return launch_status();
}

int qgx_operator_diag(const qgx_operator_t* op, const uint32_t* spins, int64_t ns, int32_t n, double* out,
                      qgx_stream_t stream) {
  QGX_CHECK_ARG(op && ns >= 0 && n > 0);
  if (ns == 0) return QGX_OK;
  QGX_CHECK_ARG(spins && out);
  operator_diag_kernel<<<blocks_for(ns, 128), 128, 0, as_cuda(stream)>>>(*op, spins, ns, n, out);
  return launch_status();
}

int qgx_energy_stats(const double* E_re, const double* E_im, const double* r, int64_t ns, double* stats,
                     double* ebar_re, double* ebar_im, qgx_stream_t stream) {
  QGX_CHECK_ARG(ns > 0 && E_re && stats && ebar_re);
  QGX_CHECK_ARG(!E_im || ebar_im);
  energy_stats_kernel<<<1, kStatThreads, 0, as_cuda(stream)>>>(E_re, E_im, r, ns, stats, ebar_re, ebar_im);
  return launch_status();
}

int qgx_reweight_factor(const float* log_psi, int64_t ns, float reweight, double* r, qgx_stream_t stream) {
  QGX_CHECK_ARG(ns > 0 && log_psi && r);
  reweight_kernel<<<1, kStatThreads, 0, as_cuda(stream)>>>(log_psi, ns, reweight, r);
  return launch_status();
}

int qgx_log_psi_mismatch(const float* local, const float* direct, int64_t ns, int32_t* count, float* out,
                         qgx_stream_t stream) {
  QGX_CHECK_ARG(ns > 0 && local && direct && count);
  QGX_CHECK_CUDA(cudaMemsetAsync(count, 0, sizeof(int32_t), as_cuda(stream)));
  log_psi_mismatch_kernel<<<blocks_for(ns, 256), 256, 0, as_cuda(stream)>>>(local, direct, ns, count, out);
  return launch_status();
}

int64_t qgx_center_columns_workspace_bytes(int64_t ns, int64_t np) {
  if (ns <= 0 || np <= 0) return 0;
  const int64_t nchunk = (ns + kColRows - 1) / kColRows;
  return (2 * nchunk * np + 2 * np) * (int64_t)sizeof(double);  // partials, the mean, its float pair
}

int qgx_center_columns(float* O, int64_t ns, int64_t np, int64_t ldo, const double* r, double* omean,
                       void* workspace, int64_t workspace_bytes, qgx_stream_t stream) {
  QGX_CHECK_ARG(ns > 0 && np > 0 && ldo >= np && O);
  QGX_CHECK_ARG(workspace && workspace_bytes >= qgx_center_columns_workspace_bytes(ns, np));
  const int64_t nchunk = (ns + kColRows - 1) / kColRows;
  QGX_CHECK_ARG(nchunk <= 65535);
  double* part_u = static_cast<double*>(workspace);
  double* part_w = part_u + nchunk * np;
  double* mean_u = part_w + nchunk * np;
  float2* mean2 = reinterpret_cast<float2*>(mean_u + np);
  cudaStream_t st = as_cuda(stream);
  dim3 g1(blocks_for(np, kColThreads), (unsigned)nchunk);
  col_partial_kernel<<<g1, kColThreads, 0, st>>>(O, ns, np, ldo, r, part_u, part_w);
  col_reduce_kernel<<<blocks_for(np, 256), 256, 0, st>>>(part_u, part_w, nchunk, np, ns, mean_u, omean, nullptr);
  split_mean_kernel<<<blocks_for(np, 256), 256, 0, st>>>(mean_u, np, mean2);
  const bool vec = (reinterpret_cast<uintptr_t>(O) & 15) == 0 && ldo % 4 == 0;
  const unsigned grid = (unsigned)std::min<int64_t>(ns, (int64_t)device_sm_count() * 8);
  if (vec)
    col_center_kernel<true><<<grid, 256, 0, st>>>(O, ns, np, ldo, r, mean2);
  else
    col_center_kernel<false><<<grid, 256, 0, st>>>(O, ns, np, ldo, r, mean2);
  return launch_status();
}

int64_t qgx_column_sumsq_workspace_bytes(int64_t rows, int64_t cols) {
  if (rows <= 0 || cols <= 0) return 0;
  return ((rows + kColRows - 1) / kColRows) * cols * (int64_t)sizeof(double);
}

int qgx_column_sumsq(const float* A, int64_t rows, int64_t cols, int64_t lda, double* out, void* workspace,
                     int64_t workspace_bytes, qgx_stream_t stream) {
  QGX_CHECK_ARG(rows > 0 && cols > 0 && lda >= cols && A && out && workspace);
  QGX_CHECK_ARG(workspace_bytes >= qgx_column_sumsq_workspace_bytes(rows, cols));
  const int64_t nchunk = (rows + kColRows - 1) / kColRows;
  QGX_CHECK_ARG(nchunk <= 65535);
  cudaStream_t st = as_cuda(stream);
  double* part = static_cast<double*>(workspace);
  col_sumsq_kernel<<<dim3(blocks_for(cols, kColThreads), (unsigned)nchunk), kColThreads, 0, st>>>(A, rows, cols, lda,
                                                                                                   part);
  col_sum_parts_kernel<<<blocks_for(cols, 256), 256, 0, st>>>(part, nchunk, cols, out);
  return launch_status();
}

int qgx_apply_update(float* params, const double* step, int64_t np, int32_t* flag, qgx_stream_t stream) {
  QGX_CHECK_ARG(np >= 0 && params && step && flag);
  cudaStream_t st = as_cuda(stream);
  QGX_CHECK_CUDA(cudaMemsetAsync(flag, 0, sizeof(int32_t), st));
  if (np == 0) return QGX_OK;
  const unsigned nb = (unsigned)std::min<int64_t>(blocks_for(np, 256), 4 * device_sm_count());
  finite_check_kernel<<<nb, 256, 0, st>>>(step, np, flag);
  update_kernel<<<nb, 256, 0, st>>>(params, step, np, flag);
  return launch_status();
}

}  // extern "C"
