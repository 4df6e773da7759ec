// RBM_Dense kernels: direct log psi, the Metropolis sweep (LocalFlip / SpinExchange),
// local energies with in-kernel connected configurations, per-sample log-derivatives and
// the centred Obar matrix.
//
// Model (quantax/model/shallow_nets.py:35-126): theta = W s + b, log psi = sum_i log cosh
// theta_i (+ a.s). Flipping site k multiplies psi by
//     prod_i cosh(theta_i - 2 W_ik s_k) / cosh(theta_i) = prod_i (C_ik - s_k t_i S_ik)
// with t = tanh(theta), C = cosh(2W), S = sinh(2W). The kernels evaluate this product per
// lane (one fma per hidden unit) and take one logf per lane, where the reference's
// ref_forward (shallow_nets.py:87-108) takes one log-cosh per hidden unit.
//
// Work layout: one warp per Markov chain / sample. Hidden units are padded to
// Mp = 128 * JT and lane l owns units {128 j + 4 l + q : j < JT, q < 4}, so every table
// row is read with one 16-byte shared-memory load per lane and j. theta and t stay in
// registers for the whole sweep; only the packed spins and log|psi| touch HBM.
#include <cuda.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "qgx_colstats.cuh"
#include "qgx_common.cuh"

namespace qgx {
namespace {

constexpr unsigned kFull = 0xffffffffu;

struct RbmTable {
  const float* Wt;  // N x Mp  (Wt[k*Mp + i] = W[i, k])
  const float* C;   // N x Mp  cosh(2 W[i, k])
  const float* S;   // N x Mp  sinh(2 W[i, k])
  const float* b;   // Mp
  const float* a;   // N (zeros without a visible bias)
};

// hidden units padded to a compiled width: 128, 256, 384, 512, 1024 or 2048 (padded units have
// zero weights and bias, so cosh = 1, sinh = 0 and they leave every ratio unchanged)
__host__ __device__ inline int padded_m(int m) {
  const int p = (m + 127) / 128 * 128;
  return p > 1024 ? 2048 : ((p > 512) ? 1024 : p);
}

// floats of the table, rounded to a multiple of 4 so staging can use 16-byte copies
__host__ __device__ inline int64_t table_floats(int n, int m) {
  const int64_t mp = padded_m(m);
  return (3 * (int64_t)n * mp + mp + n + 3) / 4 * 4;
}
// floats of the Wt | b | a part only (Wt first, then b, then a: not contiguous in the
// table, so the forward-only kernels stage Wt and b|a separately)
inline int64_t fwd_floats(int n, int m) {
  const int64_t mp = padded_m(m);
  return (int64_t)n * mp + (mp + n + 3) / 4 * 4;
}

__host__ __device__ inline RbmTable table_view(const float* base, int n, int mp) {
  RbmTable t;
  t.Wt = base;
  t.C = base + (int64_t)n * mp;
  t.S = base + 2 * (int64_t)n * mp;
  t.b = base + 3 * (int64_t)n * mp;
  t.a = t.b + mp;
  return t;
}

__global__ void prepare_kernel(const float* __restrict__ W, const float* __restrict__ b, const float* __restrict__ a,
                               int n, int m, int mp, float* __restrict__ out) {
  const int64_t nm = (int64_t)n * mp;
  const int64_t tot = table_floats(n, m);
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    if (e < nm) {
      const int k = (int)(e / mp), i = (int)(e % mp);
      const float w = i < m ? W[(int64_t)i * n + k] : 0.0f;
      out[e] = w;
      out[nm + e] = coshf(2.0f * w);
      out[2 * nm + e] = sinhf(2.0f * w);
    } else if (e >= 3 * nm) {
      const int64_t r = e - 3 * nm;
      float v = 0.0f;
      if (r < mp) {
        v = (r < m && b) ? b[r] : 0.0f;
      } else if (r < mp + n) {
        v = a ? a[r - mp] : 0.0f;
      }
      out[e] = v;
    }
  }
}

// Copy `nfloat` floats (multiple of 4, 16-byte aligned) from global to shared.
__device__ inline void stage(float* dst, const float* src, int64_t nfloat) {
  const float4* s4 = reinterpret_cast<const float4*>(src);
  float4* d4 = reinterpret_cast<float4*>(dst);
  for (int64_t e = threadIdx.x; e < nfloat / 4; e += blockDim.x) d4[e] = __ldg(s4 + e);
}

__device__ inline float spin_at(const uint32_t* sp, int k) { return ((sp[k >> 5] >> (k & 31)) & 1u) ? 1.0f : -1.0f; }

template <int JT>
__device__ inline void compute_theta(const RbmTable& T, int n, int mp, const uint32_t* sp, int lane,
                                     float (&th)[JT][4]) {
#pragma unroll
  for (int j = 0; j < JT; ++j) {
    const float4 bv = *reinterpret_cast<const float4*>(T.b + 128 * j + 4 * lane);
    th[j][0] = bv.x;
    th[j][1] = bv.y;
    th[j][2] = bv.z;
    th[j][3] = bv.w;
  }
  for (int k = 0; k < n; ++k) {
    const float sk = spin_at(sp, k);
#pragma unroll
    for (int j = 0; j < JT; ++j) {
      const float4 w = *reinterpret_cast<const float4*>(T.Wt + (int64_t)k * mp + 128 * j + 4 * lane);
      th[j][0] = fmaf(sk, w.x, th[j][0]);
      th[j][1] = fmaf(sk, w.y, th[j][1]);
      th[j][2] = fmaf(sk, w.z, th[j][2]);
      th[j][3] = fmaf(sk, w.w, th[j][3]);
    }
  }
}

// a.s summed over the warp (result valid in every lane)
__device__ inline float visible_dot(const float* a, int n, const uint32_t* sp, int lane) {
  float acc = 0.0f;
  for (int k = lane; k < n; k += 32) acc = fmaf(a[k], spin_at(sp, k), acc);
  return warp_sum(acc);
}

template <int JT>
__device__ inline float sum_logcosh(const float (&th)[JT][4]) {
  float acc = 0.0f;
#pragma unroll
  for (int j = 0; j < JT; ++j)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc += logcoshf(th[j][q]);
  return warp_sum(acc);
}

// log of prod_u (C_uk - s t_u S_uk) over the lane's units, for flipping site k
template <int JT>
__device__ inline float lane_log_flip1(const RbmTable& T, int mp, int k, float sk, const float (&t)[JT][4], int lane) {
  float prod = 1.0f;
#pragma unroll
  for (int j = 0; j < JT; ++j) {
    const float4 cv = *reinterpret_cast<const float4*>(T.C + (int64_t)k * mp + 128 * j + 4 * lane);
    const float4 sv = *reinterpret_cast<const float4*>(T.S + (int64_t)k * mp + 128 * j + 4 * lane);
    prod *= fmaf(-sk * t[j][0], sv.x, cv.x);
    prod *= fmaf(-sk * t[j][1], sv.y, cv.y);
    prod *= fmaf(-sk * t[j][2], sv.z, cv.z);
    prod *= fmaf(-sk * t[j][3], sv.w, cv.w);
  }
  return logf(prod);
}

// log of prod_u cosh(theta_u + d_u) / cosh(theta_u), d_u = -2 (W_ui si + W_uj sj), for
// flipping both sites i and j; also returns d in `d`.
template <int JT>
__device__ inline float lane_log_flip2(const RbmTable& T, int mp, int i, float si, int j, float sj,
                                       const float (&t)[JT][4], int lane, float (&d)[JT][4]) {
  float prod = 1.0f;
#pragma unroll
  for (int jj = 0; jj < JT; ++jj) {
    const float4 wi = *reinterpret_cast<const float4*>(T.Wt + (int64_t)i * mp + 128 * jj + 4 * lane);
    const float4 wj = *reinterpret_cast<const float4*>(T.Wt + (int64_t)j * mp + 128 * jj + 4 * lane);
    const float w_i[4] = {wi.x, wi.y, wi.z, wi.w};
    const float w_j[4] = {wj.x, wj.y, wj.z, wj.w};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float dd = -2.0f * fmaf(w_i[q], si, w_j[q] * sj);
      d[jj][q] = dd;
      const float e = expf(dd);
      // cosh(d) + t sinh(d) = ((1 + t) e^d + (1 - t) e^-d) / 2
      prod *= 0.5f * fmaf(1.0f + t[jj][q], e, (1.0f - t[jj][q]) / e);
    }
  }
  return logf(prod);
}

// ---------------------------------------------------------------------------------------
// Metropolis sweep: one warp per chain. CTA `cta` of `nctas` takes chains cta, cta + nctas, ...
// (a chain's result depends only on its own configuration and Philox stream, not on the CTA).
template <int JT, bool SMEM, int NT, int PROP>
__device__ inline void sweep_body(float* sm, const float* __restrict__ table, int n, int mp,
                                  uint32_t* __restrict__ spins, float* __restrict__ log_psi,
                                  int32_t* __restrict__ accepts, int64_t ns, int nsteps, uint64_t seed, uint64_t step0,
                                  float reweight, const int32_t* __restrict__ nbr, int z, int hop, int64_t table_nf,
                                  int cta, int nctas) {
  constexpr int kWarps = NT / 32;
  uint32_t* sp_all = reinterpret_cast<uint32_t*>(sm + (SMEM ? table_nf : 0));
  RbmTable T;
  if (SMEM) {
    stage(sm, table, table_nf);
    __syncthreads();
    T = table_view(sm, n, mp);
  } else {
    T = table_view(table, n, mp);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t* sp = sp_all + 32 * warp;  // this warp's packed configuration
  const int nw = words_for(n);

  for (int64_t slot = warp;; slot += kWarps) {
    const int64_t c = slot * nctas + cta;
    if (c >= ns) break;
    if (lane < nw) sp[lane] = spins[c * nw + lane];
    __syncwarp();
    float th[JT][4], t[JT][4];
    compute_theta<JT>(T, n, mp, sp, lane, th);
#pragma unroll
    for (int j = 0; j < JT; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) t[j][q] = tanhf(th[j][q]);

    int nacc = 0;
    uint32_t r0 = 0, r1 = 0, r2 = 0;
    for (int step = 0; step < nsteps; ++step) {
      const int sl = step & 31;
      if (sl == 0) {  // lane l draws the numbers of step (step + l)
        const u32x4 r = draw(seed, (uint64_t)c, step0 + (uint64_t)(step + lane), kTagPropose);
        r0 = r.x;
        r1 = r.y;
        r2 = r.z;
      }
      const uint32_t w0 = __shfl_sync(kFull, r0, sl);
      const uint32_t w1 = __shfl_sync(kFull, r1, sl);
      const uint32_t w2 = PROP == QGX_PROPOSAL_LOCAL_FLIP ? 0u : __shfl_sync(kFull, r2, sl);
      const float rhs = log1pf(-unit_float(w1));  // log(1 - u)
      if (PROP == QGX_PROPOSAL_LOCAL_FLIP) {
        const int k = (int)bounded(w0, (uint32_t)n);
        const float sk = spin_at(sp, k);
        float dl = lane_log_flip1<JT>(T, mp, k, sk, t, lane);
        dl = __shfl_sync(kFull, warp_sum(dl), 0) - 2.0f * sk * T.a[k];
        if (reweight * dl > rhs) {
#pragma unroll
          for (int j = 0; j < JT; ++j) {
            const float4 w = *reinterpret_cast<const float4*>(T.Wt + (int64_t)k * mp + 128 * j + 4 * lane);
            th[j][0] = fmaf(-2.0f * sk, w.x, th[j][0]);
            th[j][1] = fmaf(-2.0f * sk, w.y, th[j][1]);
            th[j][2] = fmaf(-2.0f * sk, w.z, th[j][2]);
            th[j][3] = fmaf(-2.0f * sk, w.w, th[j][3]);
#pragma unroll
            for (int q = 0; q < 4; ++q) t[j][q] = tanhf(th[j][q]);
          }
          __syncwarp();
          if (lane == 0) sp[k >> 5] ^= 1u << (k & 31);
          __syncwarp();
          ++nacc;
        }
      } else {
        // SpinExchange: site i uniform among sites holding the hopping particle
        uint32_t mword = 0;
        if (lane < nw) {
          const uint32_t valid = (32 * lane + 32 <= n) ? kFull : ((1u << (n - 32 * lane)) - 1u);
          mword = (hop > 0 ? sp[lane] : ~sp[lane]) & valid;
        }
        const int cnt = __popc(mword);
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int v = __shfl_up_sync(kFull, incl, o);
          if (lane >= o) incl += v;
        }
        const int total = __shfl_sync(kFull, incl, 31);
        if (total == 0) continue;
        const int r = (int)bounded(w0, (uint32_t)total);
        const int excl = incl - cnt;
        const bool own = r >= excl && r < incl;
        int pos = 0;
        if (own) {
          uint32_t mm = mword;
          for (int q = 0; q < r - excl; ++q) mm &= mm - 1u;
          pos = 32 * lane + __ffs(mm) - 1;
        }
        const int owner = __ffs(__ballot_sync(kFull, own)) - 1;
        const int i = __shfl_sync(kFull, pos, owner);
        int j = nbr[(int64_t)i * z + (int)bounded(w2, (uint32_t)z)];
        if (j < 0) j = i;
        const float si = spin_at(sp, i), sj = spin_at(sp, j);
        if (si == sj) continue;  // unchanged configuration: never accepted
        float d[JT][4];
        float dl = lane_log_flip2<JT>(T, mp, i, si, j, sj, t, lane, d);
        dl = __shfl_sync(kFull, warp_sum(dl), 0) - 2.0f * (si * T.a[i] + sj * T.a[j]);
        if (reweight * dl > rhs) {
#pragma unroll
          for (int jj = 0; jj < JT; ++jj)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              th[jj][q] += d[jj][q];
              t[jj][q] = tanhf(th[jj][q]);
            }
          __syncwarp();
          if (lane == 0) {
            sp[i >> 5] ^= 1u << (i & 31);
            sp[j >> 5] ^= 1u << (j & 31);
          }
          __syncwarp();
          ++nacc;
        }
      }
    }
    const float lp = sum_logcosh<JT>(th) + visible_dot(T.a, n, sp, lane);
    if (lane == 0) {
      log_psi[c] = lp;
      if (accepts) accepts[c] = nacc;
    }
    if (lane < nw) spins[c * nw + lane] = sp[lane];
    __syncwarp();
  }
}

template <int JT, bool SMEM, int NT, int PROP>
__global__ void __launch_bounds__(NT, 1)
    sweep_kernel(const float* __restrict__ table, int n, int mp, uint32_t* __restrict__ spins,
                 float* __restrict__ log_psi, int32_t* __restrict__ accepts, int64_t ns, int nsteps, uint64_t seed,
                 uint64_t step0, float reweight, const int32_t* __restrict__ nbr, int z, int hop,
                 int64_t table_nf) {
  extern __shared__ float4 smem4[];
  sweep_body<JT, SMEM, NT, PROP>(reinterpret_cast<float*>(smem4), table, n, mp, spins, log_psi, accepts, ns, nsteps,
                                 seed, step0, reweight, nbr, z, hop, table_nf, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------------------------------
// Local energies: one warp per sample, connected configurations generated in-kernel.
__device__ inline int bit_of(const uint32_t* sp, int k) { return (int)((sp[k >> 5] >> (k & 31)) & 1u); }

template <int JT, bool SMEM, int NT>
__device__ inline void eloc_body(float* sm, const float* __restrict__ table, int n, int mp, const qgx_operator_t& op,
                                 const uint32_t* __restrict__ spins, int64_t ns, double* __restrict__ eloc,
                                 int64_t table_nf, int cta, int nctas) {
  constexpr int kWarps = NT / 32;
  uint32_t* sp_all = reinterpret_cast<uint32_t*>(sm + (SMEM ? table_nf : 0));
  RbmTable T;
  if (SMEM) {
    stage(sm, table, table_nf);
    __syncthreads();
    T = table_view(sm, n, mp);
  } else {
    T = table_view(table, n, mp);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t* sp = sp_all + 32 * warp;
  const int nw = words_for(n);
  for (int64_t slot = warp;; slot += kWarps) {
    const int64_t c = slot * nctas + cta;
    if (c >= ns) break;
    if (lane < nw) sp[lane] = spins[c * nw + lane];
    __syncwarp();
    float th[JT][4], t[JT][4];
    compute_theta<JT>(T, n, mp, sp, lane, th);
#pragma unroll
    for (int j = 0; j < JT; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) t[j][q] = tanhf(th[j][q]);

    double ed = 0.0;
    for (int k = lane; k < op.n_z; k += 32) ed += op.z_J[k] * (double)spin_at(sp, op.z_i[k]);
    for (int k = lane; k < op.n_zz; k += 32)
      ed += op.zz_J[k] * (double)(spin_at(sp, op.zz_ij[2 * k]) * spin_at(sp, op.zz_ij[2 * k + 1]));
    ed = warp_sum(ed);

    double eo = 0.0;  // accumulated in lane 0
    for (int k = 0; k < op.n_f1; ++k) {
      const int site = op.f1_i[k];
      const int bs = bit_of(sp, site);
      const double elem = op.f1_J[2 * k + bs];
      if (elem == 0.0) continue;
      const float sk = bs ? 1.0f : -1.0f;
      const float l = warp_sum(lane_log_flip1<JT>(T, mp, site, sk, t, lane)) - 2.0f * sk * T.a[site];
      if (lane == 0) eo += elem * exp((double)l);
    }
    for (int k = 0; k < op.n_f2; ++k) {
      const int i = op.f2_ij[2 * k], j = op.f2_ij[2 * k + 1];
      const int bi = bit_of(sp, i), bj = bit_of(sp, j);
      const double elem = op.f2_J[4 * k + 2 * bi + bj];
      if (elem == 0.0) continue;
      const float si = bi ? 1.0f : -1.0f, sj = bj ? 1.0f : -1.0f;
      float d[JT][4];
      const float l = warp_sum(lane_log_flip2<JT>(T, mp, i, si, j, sj, t, lane, d)) -
                      2.0f * (si * T.a[i] + sj * T.a[j]);
      if (lane == 0) eo += elem * exp((double)l);
    }
    if (lane == 0) eloc[c] = op.c0 + ed + eo;
    __syncwarp();
  }
}

template <int JT, bool SMEM, int NT>
__global__ void __launch_bounds__(NT, 1)
    eloc_kernel(const float* __restrict__ table, int n, int mp, qgx_operator_t op, const uint32_t* __restrict__ spins,
                int64_t ns, double* __restrict__ eloc, int64_t table_nf) {
  extern __shared__ float4 smem4[];
  eloc_body<JT, SMEM, NT>(reinterpret_cast<float*>(smem4), table, n, mp, op, spins, ns, eloc, table_nf, blockIdx.x,
                          gridDim.x);
}

// ---------------------------------------------------------------------------------------
// Batched sweeps and local energies: one launch serves the jobs of several independent states
// (a serving loop's RBM jobs of one hidden-unit width class). The job table travels as a kernel
// parameter; CTAs [cta0[j], cta0[j + 1]) run job j exactly as its own launch would (same
// device function, its own chains, Philox streams and table), so every job's results are
// bit-identical to a separate call.
constexpr int kBatchJobs = QGX_RBM_BATCH_MAX_JOBS;

struct SweepJob {
  const float* table;
  uint32_t* spins;
  float* log_psi;
  int32_t* accepts;
  const int32_t* nbr;
  int64_t ns, table_nf;
  uint64_t seed, step0;
  float reweight;
  int n, mp, nsteps, z, hop;
};

struct SweepBatch {
  int njobs;
  int cta0[kBatchJobs + 1];
  SweepJob job[kBatchJobs];
};

struct ElocJob {
  qgx_operator_t op;
  const float* table;
  const uint32_t* spins;
  double* eloc;
  int64_t ns, table_nf;
  int n, mp;
};

struct ElocBatch {
  int njobs;
  int cta0[kBatchJobs + 1];
  ElocJob job[kBatchJobs];
};

__device__ inline int batch_job_of(const int* cta0, int njobs) {
  int j = 0;
  while (j + 1 < njobs && cta0[j + 1] <= (int)blockIdx.x) ++j;
  return j;
}

template <int JT, bool SMEM, int NT, int PROP>
__global__ void __launch_bounds__(NT, 1) sweep_batch_kernel(const __grid_constant__ SweepBatch b) {
  extern __shared__ float4 smem4[];
  const int j = batch_job_of(b.cta0, b.njobs);
  const SweepJob& J = b.job[j];
  sweep_body<JT, SMEM, NT, PROP>(reinterpret_cast<float*>(smem4), J.table, J.n, J.mp, J.spins, J.log_psi, J.accepts,
                                 J.ns, J.nsteps, J.seed, J.step0, J.reweight, J.nbr, J.z, J.hop, J.table_nf,
                                 (int)blockIdx.x - b.cta0[j], b.cta0[j + 1] - b.cta0[j]);
}

template <int JT, bool SMEM, int NT>
__global__ void __launch_bounds__(NT, 1) eloc_batch_kernel(const __grid_constant__ ElocBatch b) {
  extern __shared__ float4 smem4[];
  const int j = batch_job_of(b.cta0, b.njobs);
  const ElocJob& J = b.job[j];
  eloc_body<JT, SMEM, NT>(reinterpret_cast<float*>(smem4), J.table, J.n, J.mp, J.op, J.spins, J.ns, J.eloc, J.table_nf,
                          (int)blockIdx.x - b.cta0[j], b.cta0[j + 1] - b.cta0[j]);
}

// ---------------------------------------------------------------------------------------
// Forward-only kernels: stage Wt then b|a (the tail of the table) in shared memory.
template <bool SMEM>
__device__ inline RbmTable stage_forward(float* sm, const float* table, int n, int mp) {
  RbmTable T = table_view(table, n, mp);
  if (!SMEM) return T;
  const int64_t nm = (int64_t)n * mp;
  const int64_t tail = (mp + n + 3) / 4 * 4;
  stage(sm, T.Wt, nm);
  stage(sm + nm, T.b, tail);
  __syncthreads();
  RbmTable S;
  S.Wt = sm;
  S.C = nullptr;
  S.S = nullptr;
  S.b = sm + nm;
  S.a = S.b + mp;
  return S;
}

// log psi of ns configurations (n_live, device, may be NULL: a run-time cap on the count);
// written to log_psi[c], or as the pair (log psi, 0) to pairs[c] when pairs is set
template <int JT, bool SMEM, int NT>
__global__ void __launch_bounds__(NT)
    log_psi_kernel(const float* __restrict__ table, int n, int mp, const uint32_t* __restrict__ spins, int64_t ns,
                   float* __restrict__ log_psi, int64_t fwd_nf, const int64_t* __restrict__ n_live = nullptr,
                   float2* __restrict__ pairs = nullptr) {
  extern __shared__ float4 smem4[];
  float* sm = reinterpret_cast<float*>(smem4);
  constexpr int kWarps = NT / 32;
  const RbmTable T = stage_forward<SMEM>(sm, table, n, mp);
  uint32_t* sp = reinterpret_cast<uint32_t*>(sm + (SMEM ? fwd_nf : 0)) + 32 * (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = words_for(n);
  const int64_t total = n_live ? min(ns, *n_live) : ns;
  for (int64_t slot = warp;; slot += kWarps) {
    const int64_t c = slot * gridDim.x + blockIdx.x;
    if (c >= total) break;
    if (lane < nw) sp[lane] = spins[c * nw + lane];
    __syncwarp();
    float th[JT][4];
    compute_theta<JT>(T, n, mp, sp, lane, th);
    const float lp = sum_logcosh<JT>(th) + visible_dot(T.a, n, sp, lane);
    if (lane == 0) {
      if (pairs)
        pairs[c] = make_float2(lp, 0.0f);
      else
        log_psi[c] = lp;
    }
    __syncwarp();
  }
}

// t = tanh(theta) for every sample (ns x mp), input of the column statistics
template <int JT, bool SMEM, int NT>
__global__ void __launch_bounds__(NT)
    tanh_kernel(const float* __restrict__ table, int n, int mp, const uint32_t* __restrict__ spins, int64_t ns,
                float* __restrict__ tout, int64_t fwd_nf) {
  extern __shared__ float4 smem4[];
  float* sm = reinterpret_cast<float*>(smem4);
  constexpr int kWarps = NT / 32;
  const RbmTable T = stage_forward<SMEM>(sm, table, n, mp);
  uint32_t* sp = reinterpret_cast<uint32_t*>(sm + (SMEM ? fwd_nf : 0)) + 32 * (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = words_for(n);
  for (int64_t slot = warp;; slot += kWarps) {
    const int64_t c = slot * gridDim.x + blockIdx.x;
    if (c >= ns) break;
    if (lane < nw) sp[lane] = spins[c * nw + lane];
    __syncwarp();
    float th[JT][4];
    compute_theta<JT>(T, n, mp, sp, lane, th);
#pragma unroll
    for (int j = 0; j < JT; ++j) {
      float4 v = make_float4(tanhf(th[j][0]), tanhf(th[j][1]), tanhf(th[j][2]), tanhf(th[j][3]));
      *reinterpret_cast<float4*>(tout + c * mp + 128 * j + 4 * lane) = v;
    }
    __syncwarp();
  }
}

// Column sums of O (optionally weighted by r) over chunks of kChunkRows samples, with O
// generated from t and the spins: column (i, j) -> t_i s_j, column M + i -> t_i,
// column M N + M + j -> s_j.
constexpr int kChunkRows = 128;

__global__ void colsum_kernel(const float* __restrict__ tb, const uint32_t* __restrict__ spins, int n, int m, int mp,
                              int64_t np, int64_t ns, const double* __restrict__ r, double* __restrict__ part_u,
                              double* __restrict__ part_w) {
  const int64_t col = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (col >= np) return;
  const int nw = words_for(n);
  const int64_t mn = (int64_t)m * n;
  int kind, i = 0, j = 0;
  if (col < mn) {
    kind = 0;
    i = (int)(col / n);
    j = (int)(col % n);
  } else if (col < mn + m) {
    kind = 1;
    i = (int)(col - mn);
  } else {
    kind = 2;
    j = (int)(col - mn - m);
  }
  const int64_t s0 = (int64_t)blockIdx.y * kChunkRows;
  const int64_t s1 = min(ns, s0 + kChunkRows);
  float su = 0.0f;
  double sw = 0.0;
  for (int64_t s = s0; s < s1; ++s) {
    const float sj = ((spins[s * nw + (j >> 5)] >> (j & 31)) & 1u) ? 1.0f : -1.0f;
    const float ti = tb[s * mp + i];
    const float v = kind == 0 ? ti * sj : (kind == 1 ? ti : sj);
    su += v;
    if (r) sw += (double)v * r[s];
  }
  part_u[blockIdx.y * np + col] = (double)su;
  part_w[blockIdx.y * np + col] = r ? sw : (double)su;
}

// Row writer for O (centred = false) or Obar (centred = true): warp per sample.
template <int JT, bool SMEM, int NT>
__global__ void __launch_bounds__(NT)
    jacobian_kernel(const float* __restrict__ table, int n, int m, int mp, int has_vbias,
                    const uint32_t* __restrict__ spins, int64_t ns, float* __restrict__ O, int64_t ldo, bool centred,
                    const float* __restrict__ mean_f, const double* __restrict__ r, int64_t fwd_nf, bool vec4) {
  extern __shared__ float4 smem4[];
  float* sm = reinterpret_cast<float*>(smem4);
  constexpr int kWarps = NT / 32;
  const RbmTable T = stage_forward<SMEM>(sm, table, n, mp);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float* tb = sm + (SMEM ? fwd_nf : 0) + (int64_t)warp * (mp + 32);
  uint32_t* sp = reinterpret_cast<uint32_t*>(tb + mp);
  const int nw = words_for(n);
  const int64_t mn = (int64_t)m * n;
  const int64_t np = mn + m + (has_vbias ? n : 0);
  for (int64_t slot = warp;; slot += kWarps) {
    const int64_t c = slot * gridDim.x + blockIdx.x;
    if (c >= ns) break;
    if (lane < nw) sp[lane] = spins[c * nw + lane];
    __syncwarp();
    float th[JT][4];
    compute_theta<JT>(T, n, mp, sp, lane, th);
#pragma unroll
    for (int j = 0; j < JT; ++j)
      *reinterpret_cast<float4*>(tb + 128 * j + 4 * lane) =
          make_float4(tanhf(th[j][0]), tanhf(th[j][1]), tanhf(th[j][2]), tanhf(th[j][3]));
    __syncwarp();
    const float f = centred ? (float)sqrt((r ? r[c] : 1.0) / (double)ns) : 1.0f;
    float* row = O + c * ldo;
    if (vec4) {
      // 32-bit indices (a row has m n < 2^31 entries); unrolled so that several loads of
      // the column means are in flight per lane
      const int mn32 = (int)mn;
#pragma unroll 4
      for (int e4 = lane; e4 < mn32 / 4; e4 += 32) {
        const int e = 4 * e4;
        const int i = e / n, j = e - i * n;
        const float ti = tb[i];
        const uint32_t bits = sp[j >> 5] >> (j & 31);  // j % 4 == 0 so j..j+3 share a word
        float4 v = make_float4((bits & 1u) ? ti : -ti, (bits & 2u) ? ti : -ti, (bits & 4u) ? ti : -ti,
                               (bits & 8u) ? ti : -ti);
        if (centred) {
          const float4 mu = *reinterpret_cast<const float4*>(mean_f + e);
          v = make_float4((v.x - mu.x) * f, (v.y - mu.y) * f, (v.z - mu.z) * f, (v.w - mu.w) * f);
        }
        __stcs(reinterpret_cast<float4*>(row + e), v);
      }
    } else {
      for (int64_t e = lane; e < mn; e += 32) {
        const int i = (int)(e / n), j = (int)(e % n);
        float v = tb[i] * spin_at(sp, j);
        if (centred) v = (v - mean_f[e]) * f;
        __stcs(row + e, v);
      }
    }
    for (int64_t e = mn + lane; e < np; e += 32) {
      float v = e < mn + m ? tb[e - mn] : spin_at(sp, (int)(e - mn - m));
      if (centred) v = (v - mean_f[e]) * f;
      __stcs(row + e, v);
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------------------
// RBM_Conv (quantax/model/shallow_nets.py:129-190): one circular convolution over the whole
// lattice, theta_{c,x} = b_c + sum_k W_c[(k - x + lo) mod L] s_k per lattice axis (lo =
// (L - 1) / 2, SAME padding), psi = prod_{c,x} cosh theta_{c,x}. It is the dense RBM with
// m = C N hidden units (c, x) whose weights are translated copies of W_c: the conv table is
// that dense table, followed by the conv parameters (W_c row-major over the lattice, then b).
struct ConvGeom {
  int L0, L1, lo0, lo1, N, C;
};

// index into W_c of the weight joining site k to output x
__host__ __device__ inline int conv_tap(const ConvGeom& g, int k, int x) {
  const int k0 = k / g.L1, k1 = k % g.L1, x0 = x / g.L1, x1 = x % g.L1;
  const int d0 = ((k0 - x0 + g.lo0) % g.L0 + g.L0) % g.L0;
  const int d1 = ((k1 - x1 + g.lo1) % g.L1 + g.L1) % g.L1;
  return d0 * g.L1 + d1;
}

// the site whose weight to output x is W_c[d]: inverse of conv_tap in k
__device__ inline int conv_site(const ConvGeom& g, int x, int d) {
  const int x0 = x / g.L1, x1 = x % g.L1, d0 = d / g.L1, d1 = d % g.L1;
  const int k0 = ((x0 + d0 - g.lo0) % g.L0 + g.L0) % g.L0;
  const int k1 = ((x1 + d1 - g.lo1) % g.L1 + g.L1) % g.L1;
  return k0 * g.L1 + k1;
}

__host__ __device__ inline int64_t conv_param_floats(int N, int C) { return (int64_t)C * N + C; }

__global__ void conv_prepare_kernel(const float* __restrict__ params, ConvGeom g, int mp, float* __restrict__ out) {
  const int n = g.N, m = g.C * g.N;
  const int64_t nm = (int64_t)n * mp;
  const int64_t tot = table_floats(n, m), np = conv_param_floats(g.N, g.C);
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot + np; e += (int64_t)gridDim.x * blockDim.x) {
    if (e >= tot) {
      out[e] = params[e - tot];
    } else if (e < nm) {
      const int k = (int)(e / mp), i = (int)(e % mp);
      const float w = i < m ? params[(int64_t)(i / n) * n + conv_tap(g, k, i % n)] : 0.0f;
      out[e] = w;
      out[nm + e] = coshf(2.0f * w);
      out[2 * nm + e] = sinhf(2.0f * w);
    } else if (e >= 3 * nm) {
      const int64_t r = e - 3 * nm;  // b (mp), then the visible bias (zero)
      out[e] = (r < m) ? params[(int64_t)g.C * n + r / n] : 0.0f;
    }
  }
}

// O[s][c N + d] = sum_x t_{c,x} s_{site(x, d)}, O[s][C N + c] = sum_x t_{c,x}, t = tanh theta:
// the log-derivatives of the shared weights and biases (variational.py:424-511). One CTA per
// sample; theta is summed over k in the dense forward's order.
__global__ void __launch_bounds__(256) conv_jacobian_kernel(const float* __restrict__ cparams, ConvGeom g,
                                                            const uint32_t* __restrict__ spins, int64_t ns,
                                                            float* __restrict__ O, int64_t ldo) {
  extern __shared__ float4 smem4[];
  float* sm = reinterpret_cast<float*>(smem4);
  const int N = g.N, CN = g.C * g.N, nw = (N + 31) / 32;
  float* s = sm;          // N
  float* W = s + N;       // C N
  float* t = W + CN;      // C N
  for (int e = threadIdx.x; e < CN; e += blockDim.x) W[e] = cparams[e];
  const float* b = cparams + CN;
  for (int64_t smp = blockIdx.x; smp < ns; smp += gridDim.x) {
    __syncthreads();
    const uint32_t* sp = spins + smp * nw;
    for (int k = threadIdx.x; k < N; k += blockDim.x) s[k] = spin_at(sp, k);
    __syncthreads();
    for (int i = threadIdx.x; i < CN; i += blockDim.x) {
      const int c = i / N, x = i % N;
      float th = b[c];
      for (int k = 0; k < N; ++k) th = fmaf(s[k], W[c * N + conv_tap(g, k, x)], th);
      t[i] = tanhf(th);
    }
    __syncthreads();
    float* row = O + smp * ldo;
    for (int i = threadIdx.x; i < CN + g.C; i += blockDim.x) {
      float acc = 0.0f;
      if (i < CN) {
        const int c = i / N, d = i % N;
        for (int x = 0; x < N; ++x) acc = fmaf(t[c * N + x], s[conv_site(g, x, d)], acc);
      } else {
        const int c = i - CN;
        for (int x = 0; x < N; ++x) acc += t[c * N + x];
      }
      row[i] = acc;
    }
  }
}

// ---------------------------------------------------------------------------------------
// launch helpers
template <int JT>
constexpr int threads_for() {
  return JT <= 2 ? 1024 : (JT == 4 ? 512 : 256);
}

// Shared-memory plan: stage `stage_floats` when it fits next to the per-warp scratch.
inline bool fits_smem(int nthreads, int64_t stage_floats, int64_t per_warp_floats, size_t* bytes) {
  const int64_t extra = per_warp_floats * (nthreads / 32) * 4;
  const int64_t want = stage_floats * 4 + extra;
  const bool ok = want <= device_max_smem_optin();
  *bytes = (size_t)(ok ? want : extra);
  return ok;
}

// Raise the dynamic shared-memory limit and size the grid from the occupancy: at most
// (resident blocks per SM x SMs) blocks, and no more blocks than work items.
template <typename K>
int configure(K kernel, int nthreads, size_t smem, int64_t items, int* grid) {
  if (smem > 48 * 1024)
    QGX_CHECK_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  QGX_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, nthreads, smem));
  if (per_sm < 1) return QGX_ERR_UNSUPPORTED;
  const int64_t cap = (int64_t)device_sm_count() * per_sm;
  *grid = (int)std::max<int64_t>(1, std::min<int64_t>(cap, items));
  return QGX_OK;
}

template <int JT, bool SMEM, int PROP>
int launch_sweep_v(const float* table, int n, int mp, uint32_t* spins, float* log_psi, int32_t* accepts, int64_t ns,
                   int nsteps, uint64_t seed, uint64_t step0, float reweight, const int32_t* nbr, int z, int hop,
                   size_t smem, cudaStream_t st) {
  constexpr int NT = threads_for<JT>();
  auto k = sweep_kernel<JT, SMEM, NT, PROP>;
  int grid, rc;
  if ((rc = configure(k, NT, smem, ns, &grid)) != QGX_OK) return rc;
  k<<<grid, NT, smem, st>>>(table, n, mp, spins, log_psi, accepts, ns, nsteps, seed, step0, reweight, nbr, z, hop,
                            table_floats(n, mp));
  return launch_status();
}

template <int JT>
int launch_sweep(const float* table, int n, int mp, uint32_t* spins, float* log_psi, int32_t* accepts, int64_t ns,
                 int nsteps, uint64_t seed, uint64_t step0, float reweight, int proposal, const int32_t* nbr, int z,
                 int hop, cudaStream_t st) {
  size_t smem;
  const bool sm = fits_smem(threads_for<JT>(), table_floats(n, mp), 32, &smem);
  if (proposal == QGX_PROPOSAL_LOCAL_FLIP) {
    return sm ? launch_sweep_v<JT, true, QGX_PROPOSAL_LOCAL_FLIP>(table, n, mp, spins, log_psi, accepts, ns, nsteps,
                                                                  seed, step0, reweight, nbr, z, hop, smem, st)
              : launch_sweep_v<JT, false, QGX_PROPOSAL_LOCAL_FLIP>(table, n, mp, spins, log_psi, accepts, ns, nsteps,
                                                                   seed, step0, reweight, nbr, z, hop, smem, st);
  }
  return sm ? launch_sweep_v<JT, true, QGX_PROPOSAL_SPIN_EXCHANGE>(table, n, mp, spins, log_psi, accepts, ns, nsteps,
                                                                   seed, step0, reweight, nbr, z, hop, smem, st)
            : launch_sweep_v<JT, false, QGX_PROPOSAL_SPIN_EXCHANGE>(table, n, mp, spins, log_psi, accepts, ns, nsteps,
                                                                    seed, step0, reweight, nbr, z, hop, smem, st);
}

template <int JT>
int launch_eloc(const float* table, int n, int mp, const qgx_operator_t& op, const uint32_t* spins, int64_t ns,
                double* eloc, cudaStream_t st) {
  constexpr int NT = threads_for<JT>();
  size_t smem;
  int grid, rc;
  if (fits_smem(NT, table_floats(n, mp), 32, &smem)) {
    auto k = eloc_kernel<JT, true, NT>;
    if ((rc = configure(k, NT, smem, ns, &grid)) != QGX_OK) return rc;
    k<<<grid, NT, smem, st>>>(table, n, mp, op, spins, ns, eloc, table_floats(n, mp));
  } else {
    auto k = eloc_kernel<JT, false, NT>;
    if ((rc = configure(k, NT, smem, ns, &grid)) != QGX_OK) return rc;
    k<<<grid, NT, smem, st>>>(table, n, mp, op, spins, ns, eloc, table_floats(n, mp));
  }
  return launch_status();
}

constexpr int kFwdThreads = 256;

template <int JT>
int launch_log_psi(const float* table, int n, int mp, const uint32_t* spins, int64_t ns, float* log_psi,
                   cudaStream_t st, const int64_t* n_live = nullptr, float2* pairs = nullptr) {
  const int64_t ff = fwd_floats(n, mp);
  size_t smem;
  int grid, rc;
  if (fits_smem(kFwdThreads, ff, 32, &smem)) {
    auto k = log_psi_kernel<JT, true, kFwdThreads>;
    if ((rc = configure(k, kFwdThreads, smem, (ns + 7) / 8, &grid)) != QGX_OK) return rc;
    k<<<grid, kFwdThreads, smem, st>>>(table, n, mp, spins, ns, log_psi, ff, n_live, pairs);
  } else {
    auto k = log_psi_kernel<JT, false, kFwdThreads>;
    if ((rc = configure(k, kFwdThreads, smem, (ns + 7) / 8, &grid)) != QGX_OK) return rc;
    k<<<grid, kFwdThreads, smem, st>>>(table, n, mp, spins, ns, log_psi, ff, n_live, pairs);
  }
  return launch_status();
}

template <int JT>
int launch_tanh(const float* table, int n, int mp, const uint32_t* spins, int64_t ns, float* tout, cudaStream_t st) {
  const int64_t ff = fwd_floats(n, mp);
  size_t smem;
  int grid, rc;
  if (fits_smem(kFwdThreads, ff, 32, &smem)) {
    auto k = tanh_kernel<JT, true, kFwdThreads>;
    if ((rc = configure(k, kFwdThreads, smem, (ns + 7) / 8, &grid)) != QGX_OK) return rc;
    k<<<grid, kFwdThreads, smem, st>>>(table, n, mp, spins, ns, tout, ff);
  } else {
    auto k = tanh_kernel<JT, false, kFwdThreads>;
    if ((rc = configure(k, kFwdThreads, smem, (ns + 7) / 8, &grid)) != QGX_OK) return rc;
    k<<<grid, kFwdThreads, smem, st>>>(table, n, mp, spins, ns, tout, ff);
  }
  return launch_status();
}

template <int JT>
int launch_jacobian(const float* table, int n, int m, int mp, int has_vbias, const uint32_t* spins, int64_t ns,
                    float* O, int64_t ldo, bool centred, const float* mean_f, const double* r, cudaStream_t st) {
  const int64_t ff = fwd_floats(n, mp);
  const bool vec4 = (n % 4 == 0) && (ldo % 4 == 0) && ((reinterpret_cast<uintptr_t>(O) & 15) == 0);
  size_t smem;
  int grid, rc;
  if (fits_smem(kFwdThreads, ff, mp + 32, &smem)) {
    auto k = jacobian_kernel<JT, true, kFwdThreads>;
    if ((rc = configure(k, kFwdThreads, smem, (ns + 7) / 8, &grid)) != QGX_OK) return rc;
    k<<<grid, kFwdThreads, smem, st>>>(table, n, m, mp, has_vbias, spins, ns, O, ldo, centred, mean_f, r, ff, vec4);
  } else {
    auto k = jacobian_kernel<JT, false, kFwdThreads>;
    if ((rc = configure(k, kFwdThreads, smem, (ns + 7) / 8, &grid)) != QGX_OK) return rc;
    k<<<grid, kFwdThreads, smem, st>>>(table, n, m, mp, has_vbias, spins, ns, O, ldo, centred, mean_f, r, ff, vec4);
  }
  return launch_status();
}

#define QGX_DISPATCH_JT(mp, CALL)          \
  switch ((mp) / 128) {                    \
    case 1: return CALL(1);                \
    case 2: return CALL(2);                \
    case 3: return CALL(3);                \
    case 4: return CALL(4);                \
    case 8: return CALL(8);                \
    case 16: return CALL(16);              \
    default: return QGX_ERR_UNSUPPORTED;   \
  }

constexpr int kMaxSites = 1024;  // 32 packed words per configuration

inline bool mp_supported(int mp) {
  const int jt = mp / 128;
  return jt == 1 || jt == 2 || jt == 3 || jt == 4 || jt == 8 || jt == 16;
}

// CTA ranges of a batch: job j gets min(resident capacity, ceil(ns_j / warps per CTA)) CTAs
// (one chain per warp where the GPU holds them all); false when the grid would overflow int
template <typename K>
int batch_grid(K kernel, int nthreads, size_t smem, const int64_t* ns, int njobs, int* cta0) {
  if (smem > 48 * 1024)
    QGX_CHECK_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  QGX_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, nthreads, smem));
  if (per_sm < 1) return QGX_ERR_UNSUPPORTED;
  const int64_t cap = (int64_t)device_sm_count() * per_sm, warps = nthreads / 32;
  int64_t acc = 0;
  for (int j = 0; j < njobs; ++j) {
    cta0[j] = (int)acc;
    acc += std::max<int64_t>(1, std::min<int64_t>(cap, (ns[j] + warps - 1) / warps));
    if (acc > 0x7fffffffLL) return QGX_ERR_UNSUPPORTED;
  }
  cta0[njobs] = (int)acc;
  return QGX_OK;
}

// one launch for the jobs idx[0..cnt) (all of width class JT, shared-memory staging SMEM and
// proposal PROP)
template <int JT, bool SMEM, int PROP>
int launch_sweep_batch(const qgx_rbm_sweep_job_t* jobs, const int* idx, int cnt, cudaStream_t st) {
  constexpr int NT = threads_for<JT>();
  auto k = sweep_batch_kernel<JT, SMEM, NT, PROP>;
  SweepBatch b;
  std::memset(&b, 0, sizeof(b));
  b.njobs = cnt;
  size_t smem = 0;
  int64_t ns[kBatchJobs];
  for (int q = 0; q < cnt; ++q) {
    const qgx_rbm_sweep_job_t& J = jobs[idx[q]];
    const int mp = padded_m(J.m);
    size_t bytes;
    fits_smem(NT, table_floats(J.n, mp), 32, &bytes);
    smem = std::max(smem, bytes);
    b.job[q] = SweepJob{J.table, J.spins, J.log_psi, J.accepts, J.nbr, J.ns, table_floats(J.n, mp), J.seed, J.step0,
                        J.reweight, J.n, mp, J.nsteps, J.z, J.hop};
    ns[q] = J.ns;
  }
  int rc = batch_grid(k, NT, smem, ns, cnt, b.cta0);
  if (rc != QGX_OK) return rc;
  k<<<b.cta0[cnt], NT, smem, st>>>(b);
  return launch_status();
}

template <int JT, bool SMEM>
int launch_eloc_batch(const qgx_rbm_eloc_job_t* jobs, const int* idx, int cnt, cudaStream_t st) {
  constexpr int NT = threads_for<JT>();
  auto k = eloc_batch_kernel<JT, SMEM, NT>;
  ElocBatch b;
  std::memset(&b, 0, sizeof(b));
  b.njobs = cnt;
  size_t smem = 0;
  int64_t ns[kBatchJobs];
  for (int q = 0; q < cnt; ++q) {
    const qgx_rbm_eloc_job_t& J = jobs[idx[q]];
    const int mp = padded_m(J.m);
    size_t bytes;
    fits_smem(NT, table_floats(J.n, mp), 32, &bytes);
    smem = std::max(smem, bytes);
    b.job[q] = ElocJob{*J.op, J.table, J.spins, J.eloc, J.ns, table_floats(J.n, mp), J.n, mp};
    ns[q] = J.ns;
  }
  int rc = batch_grid(k, NT, smem, ns, cnt, b.cta0);
  if (rc != QGX_OK) return rc;
  k<<<b.cta0[cnt], NT, smem, st>>>(b);
  return launch_status();
}

// the class of a job: width JT, shared-memory staging of its table, proposal
struct BatchClass {
  int jt, smem, prop;
  bool operator==(const BatchClass& o) const { return jt == o.jt && smem == o.smem && prop == o.prop; }
};

template <int JT>
int sweep_batch_jt(const qgx_rbm_sweep_job_t* jobs, const int* idx, int cnt, bool sm, int prop, cudaStream_t st) {
  if (prop == QGX_PROPOSAL_LOCAL_FLIP)
    return sm ? launch_sweep_batch<JT, true, QGX_PROPOSAL_LOCAL_FLIP>(jobs, idx, cnt, st)
              : launch_sweep_batch<JT, false, QGX_PROPOSAL_LOCAL_FLIP>(jobs, idx, cnt, st);
  return sm ? launch_sweep_batch<JT, true, QGX_PROPOSAL_SPIN_EXCHANGE>(jobs, idx, cnt, st)
            : launch_sweep_batch<JT, false, QGX_PROPOSAL_SPIN_EXCHANGE>(jobs, idx, cnt, st);
}

template <int JT>
int eloc_batch_jt(const qgx_rbm_eloc_job_t* jobs, const int* idx, int cnt, bool sm, cudaStream_t st) {
  return sm ? launch_eloc_batch<JT, true>(jobs, idx, cnt, st) : launch_eloc_batch<JT, false>(jobs, idx, cnt, st);
}

// whether job (n, mp)'s table is staged in shared memory by the kernels of width JT
inline bool stages_in_smem(int jt, int n, int mp) {
  size_t bytes;
  const int nt = jt <= 2 ? 1024 : (jt == 4 ? 512 : 256);  // threads_for<JT>()
  return fits_smem(nt, table_floats(n, mp), 32, &bytes);
}

}  // namespace

// The RBM forward and log-derivatives that the symmetrised pipelines of resconv.cu run on the
// images T_g s of a projected RBM: log psi as (log psi, 0) pairs with a run-time live count,
// and the O rows of every image (closed form, uncentred).
int rbm_log_psi_pairs(const float* table, int n, int m, const uint32_t* cfg, int64_t ncfg, const int64_t* n_live,
                      float2* out, cudaStream_t st) {
  const int mp = padded_m(m);
#define CALL(JT) launch_log_psi<JT>(table, n, mp, cfg, ncfg, nullptr, st, n_live, out)
  QGX_DISPATCH_JT(mp, CALL)
#undef CALL
}

int rbm_jacobian_rows(const float* table, int n, int m, int has_vbias, const uint32_t* cfg, int64_t rows, float* O,
                      int64_t ldo, cudaStream_t st) {
  const int mp = padded_m(m);
#define CALL(JT) launch_jacobian<JT>(table, n, m, mp, has_vbias, cfg, rows, O, ldo, false, nullptr, nullptr, st)
  QGX_DISPATCH_JT(mp, CALL)
#undef CALL
}

}  // namespace qgx

using namespace qgx;

extern "C" {

int64_t qgx_rbm_table_floats(int32_t n, int32_t m) {
  if (n <= 0 || m <= 0) return 0;
  return table_floats(n, m);
}

int qgx_rbm_prepare(const float* W, const float* b, const float* a, int32_t n, int32_t m, float* table,
                    qgx_stream_t stream) {
  QGX_CHECK_ARG(W && table && n > 0 && m > 0 && n <= kMaxSites);
  QGX_CHECK_ARG((reinterpret_cast<uintptr_t>(table) & 15) == 0);
  const int mp = padded_m(m);
  QGX_CHECK_ARG(mp_supported(mp));
  const int64_t tot = table_floats(n, m);
  const unsigned g = (unsigned)std::min<int64_t>((tot + 255) / 256, 4096);
  prepare_kernel<<<g, 256, 0, as_cuda(stream)>>>(W, b, a, n, m, mp, table);
  return launch_status();
}

static bool conv_geom(int32_t L0, int32_t L1, int32_t channels, ConvGeom* g) {
  if (L0 < 1 || L1 < 1 || channels < 1) return false;
  const int64_t N = (int64_t)L0 * L1;
  if (N > kMaxSites || channels * N > 2048) return false;
  *g = ConvGeom{L0, L1, (L0 - 1) / 2, (L1 - 1) / 2, (int)N, channels};
  return true;
}

int64_t qgx_rbm_conv_table_floats(int32_t L0, int32_t L1, int32_t channels) {
  ConvGeom g;
  if (!conv_geom(L0, L1, channels, &g)) return 0;
  return table_floats(g.N, g.C * g.N) + (conv_param_floats(g.N, g.C) + 3) / 4 * 4;
}

int qgx_rbm_conv_prepare(const float* params, int32_t L0, int32_t L1, int32_t channels, float* table,
                         qgx_stream_t stream) {
  ConvGeom g;
  QGX_CHECK_ARG(conv_geom(L0, L1, channels, &g) && params && table);
  QGX_CHECK_ARG((reinterpret_cast<uintptr_t>(table) & 15) == 0);
  const int mp = padded_m(g.C * g.N);
  const int64_t tot = table_floats(g.N, g.C * g.N) + conv_param_floats(g.N, g.C);
  const unsigned blocks = (unsigned)std::min<int64_t>((tot + 255) / 256, 4096);
  conv_prepare_kernel<<<blocks, 256, 0, as_cuda(stream)>>>(params, g, mp, table);
  return launch_status();
}

int qgx_rbm_conv_jacobian(const float* table, int32_t L0, int32_t L1, int32_t channels, const uint32_t* spins,
                          int64_t ns, float* O, int64_t ldo, qgx_stream_t stream) {
  ConvGeom g;
  QGX_CHECK_ARG(conv_geom(L0, L1, channels, &g) && ns >= 0 && ldo >= conv_param_floats(g.N, g.C));
  if (ns == 0) return QGX_OK;
  QGX_CHECK_ARG(table && spins && O);
  const float* cparams = table + table_floats(g.N, g.C * g.N);
  const size_t smem = (size_t)(g.N + 2 * g.C * g.N) * sizeof(float);
  if (smem > 48 * 1024)
    QGX_CHECK_CUDA(cudaFuncSetAttribute(conv_jacobian_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const unsigned grid = (unsigned)std::min<int64_t>(ns, (int64_t)device_sm_count() * 8);
  conv_jacobian_kernel<<<grid, 256, smem, as_cuda(stream)>>>(cparams, g, spins, ns, O, ldo);
  return launch_status();
}

int qgx_rbm_log_psi(const float* table, int32_t n, int32_t m, const uint32_t* spins, int64_t ns, float* log_psi,
                    qgx_stream_t stream) {
  QGX_CHECK_ARG(n > 0 && m > 0 && n <= kMaxSites && ns >= 0);
  if (ns == 0) return QGX_OK;
  QGX_CHECK_ARG(table && spins && log_psi);
  const int mp = padded_m(m);
#define CALL(JT) launch_log_psi<JT>(table, n, mp, spins, ns, log_psi, as_cuda(stream))
  QGX_DISPATCH_JT(mp, CALL)
#undef CALL
}

int qgx_rbm_sweep(const float* table, int32_t n, int32_t m, uint32_t* spins, float* log_psi, int32_t* accepts,
                  int64_t ns, int32_t nsteps, uint64_t seed, uint64_t step0, float reweight, int32_t proposal,
                  const int32_t* nbr, int32_t z, int32_t hop, qgx_stream_t stream) {
  QGX_CHECK_ARG(n > 0 && m > 0 && n <= kMaxSites && ns >= 0 && nsteps >= 0);
  QGX_CHECK_ARG(proposal == QGX_PROPOSAL_LOCAL_FLIP || proposal == QGX_PROPOSAL_SPIN_EXCHANGE);
  if (proposal == QGX_PROPOSAL_SPIN_EXCHANGE) QGX_CHECK_ARG(nbr && z > 0 && (hop == 1 || hop == -1));
  if (ns == 0) return QGX_OK;
  QGX_CHECK_ARG(table && spins && log_psi);
  const int mp = padded_m(m);
#define CALL(JT) \
  launch_sweep<JT>(table, n, mp, spins, log_psi, accepts, ns, nsteps, seed, step0, reweight, proposal, nbr, z, hop, as_cuda(stream))
  QGX_DISPATCH_JT(mp, CALL)
#undef CALL
}

int qgx_rbm_sweep_batched(const qgx_rbm_sweep_job_t* jobs, int32_t njobs, int32_t* launches,
                         qgx_stream_t stream) {
  QGX_CHECK_ARG(njobs >= 0 && njobs <= QGX_RBM_BATCH_MAX_JOBS && (njobs == 0 || jobs));
  if (launches) *launches = 0;
  BatchClass cls[kBatchJobs];
  bool live[kBatchJobs] = {};
  for (int j = 0; j < njobs; ++j) {
    const qgx_rbm_sweep_job_t& J = jobs[j];
    QGX_CHECK_ARG(J.n > 0 && J.m > 0 && J.n <= kMaxSites && J.ns >= 0 && J.nsteps >= 0);
    QGX_CHECK_ARG(J.proposal == QGX_PROPOSAL_LOCAL_FLIP || J.proposal == QGX_PROPOSAL_SPIN_EXCHANGE);
    if (J.proposal == QGX_PROPOSAL_SPIN_EXCHANGE) QGX_CHECK_ARG(J.nbr && J.z > 0 && (J.hop == 1 || J.hop == -1));
    if (J.ns == 0) continue;
    QGX_CHECK_ARG(J.table && J.spins && J.log_psi);
    const int mp = padded_m(J.m);
    if (!mp_supported(mp)) return QGX_ERR_UNSUPPORTED;
    cls[j] = BatchClass{mp / 128, stages_in_smem(mp / 128, J.n, mp) ? 1 : 0, J.proposal};
    live[j] = true;
  }
  const cudaStream_t st = as_cuda(stream);
  for (int j = 0; j < njobs; ++j) {
    if (!live[j]) continue;
    int idx[kBatchJobs], cnt = 0;
    for (int q = j; q < njobs; ++q)
      if (live[q] && cls[q] == cls[j]) {
        idx[cnt++] = q;
        live[q] = false;
      }
    const bool sm = cls[j].smem != 0;
    int rc = QGX_ERR_UNSUPPORTED;
    switch (cls[j].jt) {
      case 1: rc = sweep_batch_jt<1>(jobs, idx, cnt, sm, cls[j].prop, st); break;
      case 2: rc = sweep_batch_jt<2>(jobs, idx, cnt, sm, cls[j].prop, st); break;
      case 3: rc = sweep_batch_jt<3>(jobs, idx, cnt, sm, cls[j].prop, st); break;
      case 4: rc = sweep_batch_jt<4>(jobs, idx, cnt, sm, cls[j].prop, st); break;
      case 8: rc = sweep_batch_jt<8>(jobs, idx, cnt, sm, cls[j].prop, st); break;
      case 16: rc = sweep_batch_jt<16>(jobs, idx, cnt, sm, cls[j].prop, st); break;
      default: break;
    }
    if (rc != QGX_OK) return rc;
    if (launches) ++*launches;
  }
  return QGX_OK;
}

int qgx_rbm_eloc_batched(const qgx_rbm_eloc_job_t* jobs, int32_t njobs, int32_t* launches,
                         qgx_stream_t stream) {
  QGX_CHECK_ARG(njobs >= 0 && njobs <= QGX_RBM_BATCH_MAX_JOBS && (njobs == 0 || jobs));
  if (launches) *launches = 0;
  BatchClass cls[kBatchJobs];
  bool live[kBatchJobs] = {};
  for (int j = 0; j < njobs; ++j) {
    const qgx_rbm_eloc_job_t& J = jobs[j];
    QGX_CHECK_ARG(J.op && J.n > 0 && J.m > 0 && J.n <= kMaxSites && J.ns >= 0);
    if (J.ns == 0) continue;
    QGX_CHECK_ARG(J.table && J.spins && J.eloc);
    const int mp = padded_m(J.m);
    if (!mp_supported(mp)) return QGX_ERR_UNSUPPORTED;
    cls[j] = BatchClass{mp / 128, stages_in_smem(mp / 128, J.n, mp) ? 1 : 0, 0};
    live[j] = true;
  }
  const cudaStream_t st = as_cuda(stream);
  for (int j = 0; j < njobs; ++j) {
    if (!live[j]) continue;
    int idx[kBatchJobs], cnt = 0;
    for (int q = j; q < njobs; ++q)
      if (live[q] && cls[q] == cls[j]) {
        idx[cnt++] = q;
        live[q] = false;
      }
    const bool sm = cls[j].smem != 0;
    int rc = QGX_ERR_UNSUPPORTED;
    switch (cls[j].jt) {
      case 1: rc = eloc_batch_jt<1>(jobs, idx, cnt, sm, st); break;
      case 2: rc = eloc_batch_jt<2>(jobs, idx, cnt, sm, st); break;
      case 3: rc = eloc_batch_jt<3>(jobs, idx, cnt, sm, st); break;
      case 4: rc = eloc_batch_jt<4>(jobs, idx, cnt, sm, st); break;
      case 8: rc = eloc_batch_jt<8>(jobs, idx, cnt, sm, st); break;
      case 16: rc = eloc_batch_jt<16>(jobs, idx, cnt, sm, st); break;
      default: break;
    }
    if (rc != QGX_OK) return rc;
    if (launches) ++*launches;
  }
  return QGX_OK;
}

int qgx_rbm_eloc(const float* table, int32_t n, int32_t m, const qgx_operator_t* op, const uint32_t* spins,
                 int64_t ns, double* eloc, qgx_stream_t stream) {
  QGX_CHECK_ARG(op && n > 0 && m > 0 && n <= kMaxSites && ns >= 0);
  if (ns == 0) return QGX_OK;
  QGX_CHECK_ARG(table && spins && eloc);
  const int mp = padded_m(m);
#define CALL(JT) launch_eloc<JT>(table, n, mp, *op, spins, ns, eloc, as_cuda(stream))
  QGX_DISPATCH_JT(mp, CALL)
#undef CALL
}

int qgx_rbm_jacobian(const float* table, int32_t n, int32_t m, int32_t has_vbias, const uint32_t* spins, int64_t ns,
                     float* O, int64_t ldo, qgx_stream_t stream) {
  QGX_CHECK_ARG(n > 0 && m > 0 && n <= kMaxSites && ns >= 0);
  const int64_t np = (int64_t)m * n + m + (has_vbias ? n : 0);
  QGX_CHECK_ARG(ldo >= np);
  if (ns == 0) return QGX_OK;
  QGX_CHECK_ARG(table && spins && O);
  const int mp = padded_m(m);
#define CALL(JT) launch_jacobian<JT>(table, n, m, mp, has_vbias, spins, ns, O, ldo, false, nullptr, nullptr, as_cuda(stream))
  QGX_DISPATCH_JT(mp, CALL)
#undef CALL
}

int64_t qgx_rbm_obar_workspace_bytes(int32_t n, int32_t m, int64_t ns) {
  if (n <= 0 || m <= 0 || ns <= 0) return 0;
  const int64_t mp = padded_m(m);
  const int64_t np = (int64_t)m * n + m + n;
  const int64_t nchunk = (ns + kChunkRows - 1) / kChunkRows;
  // tanh buffer | part_u | part_w | mean_f  (each region 256-byte aligned)
  auto al = [](int64_t b) { return (b + 255) / 256 * 256; };
  return al(ns * mp * 4) + 2 * al(nchunk * np * 8) + al(np * 4);
}

int qgx_rbm_obar(const float* table, int32_t n, int32_t m, int32_t has_vbias, const uint32_t* spins, const double* r,
                 int64_t ns, float* Obar, int64_t ldo, double* omean, void* workspace, int64_t workspace_bytes,
                 qgx_stream_t stream) {
  QGX_CHECK_ARG(n > 0 && m > 0 && n <= kMaxSites && ns > 0);
  const int64_t np = (int64_t)m * n + m + (has_vbias ? n : 0);
  QGX_CHECK_ARG(ldo >= np && table && spins && Obar);
  QGX_CHECK_ARG(workspace && workspace_bytes >= qgx_rbm_obar_workspace_bytes(n, m, ns));
  QGX_CHECK_ARG((reinterpret_cast<uintptr_t>(workspace) & 255) == 0);
  const int mp = padded_m(m);
  if (!mp_supported(mp)) return QGX_ERR_UNSUPPORTED;
  const int64_t nchunk = (ns + kChunkRows - 1) / kChunkRows;
  QGX_CHECK_ARG(nchunk <= 65535);
  auto al = [](int64_t b) { return (b + 255) / 256 * 256; };
  char* ws = static_cast<char*>(workspace);
  float* tb = reinterpret_cast<float*>(ws);
  double* part_u = reinterpret_cast<double*>(ws + al(ns * mp * 4));
  double* part_w = reinterpret_cast<double*>(ws + al(ns * mp * 4) + al(nchunk * np * 8));
  float* mean_f = reinterpret_cast<float*>(ws + al(ns * mp * 4) + 2 * al(nchunk * np * 8));
  cudaStream_t st = as_cuda(stream);
  int rc;
#define CALL(JT) launch_tanh<JT>(table, n, mp, spins, ns, tb, st)
  switch (mp / 128) {
    case 1: rc = CALL(1); break;
    case 2: rc = CALL(2); break;
    case 3: rc = CALL(3); break;
    case 4: rc = CALL(4); break;
    case 8: rc = CALL(8); break;
    case 16: rc = CALL(16); break;
    default: return QGX_ERR_UNSUPPORTED;
  }
#undef CALL
  if (rc != QGX_OK) return rc;
  colsum_kernel<<<dim3((unsigned)((np + 255) / 256), (unsigned)nchunk), 256, 0, st>>>(tb, spins, n, m, mp, np, ns, r,
                                                                                     part_u, part_w);
  col_reduce_kernel<<<(unsigned)((np + 255) / 256), 256, 0, st>>>(part_u, part_w, nchunk, np, ns, nullptr, omean,
                                                                  mean_f);
  if ((rc = launch_status()) != QGX_OK) return rc;
#define CALL(JT) launch_jacobian<JT>(table, n, m, mp, has_vbias, spins, ns, Obar, ldo, true, mean_f, r, st)
  QGX_DISPATCH_JT(mp, CALL)
#undef CALL
}

// ---- no-allocation variant of qgx_rbm_obar -----------------------------------------------
// Scratch for callers that cannot allocate: one static device array per GPU that loads the
// library. Host code must not use the symbol's name as an address: the device address is
// looked up with cudaGetSymbolAddress (with that device current) and cached per device,
// together with the CUDA context it belongs to. A different current context on that device
// (the primary context released and created again, e.g. after cudaDeviceReset, which also
// reloads the module) makes the next call look the address up again, so a stale address is
// never used.
static __device__ __align__(256) unsigned char g_obar_scratch[QGX_RBM_OBAR_STATIC_SCRATCH_BYTES];

namespace {
constexpr int kMaxScratchDevices = 64;
std::mutex g_scratch_mutex;
void* g_scratch_ptr[kMaxScratchDevices] = {};
CUcontext g_scratch_ctx[kMaxScratchDevices] = {};

using CtxGetCurrent = CUresult (*)(CUcontext*);

CtxGetCurrent ctx_get_current_fn() {
  static std::once_flag once;
  static CtxGetCurrent fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<CtxGetCurrent>(p);
  });
  return fn;
}

int scratch_for_current_device(void** out) {
  int dev = 0;
  QGX_CHECK_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxScratchDevices) return QGX_ERR_UNSUPPORTED;
  CtxGetCurrent get_ctx = ctx_get_current_fn();
  if (!get_ctx) return QGX_ERR_UNSUPPORTED;
  CUcontext ctx = nullptr;
  if (get_ctx(&ctx) != CUDA_SUCCESS) return QGX_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!ctx || !g_scratch_ptr[dev] || g_scratch_ctx[dev] != ctx) {
    // no context bound yet, or a different one: the lookup binds the device's primary
    // context (creating it if needed) and loads the module into it
    void* p = nullptr;
    QGX_CHECK_CUDA(cudaGetSymbolAddress(&p, g_obar_scratch));
    if (get_ctx(&ctx) != CUDA_SUCCESS || !ctx) return QGX_ERR_UNSUPPORTED;
    g_scratch_ptr[dev] = p;
    g_scratch_ctx[dev] = ctx;
  }
  *out = g_scratch_ptr[dev];
  return QGX_OK;
}
}  // namespace

int qgx_rbm_obar_noalloc(const float* table, int32_t n, int32_t m, int32_t has_vbias, const uint32_t* spins,
                         const double* r, int64_t ns, float* Obar, int64_t ldo, double* omean, qgx_stream_t stream) {
  QGX_CHECK_ARG(n > 0 && m > 0 && ns > 0);
  const int64_t need = qgx_rbm_obar_workspace_bytes(n, m, ns);
  if (need > QGX_RBM_OBAR_STATIC_SCRATCH_BYTES) {
    char msg[200];
    std::snprintf(msg, sizeof(msg),
                  "qgx_rbm_obar_noalloc: n=%d m=%d ns=%lld needs %lld bytes of scratch, the static array holds %lld",
                  n, m, (long long)ns, (long long)need, (long long)QGX_RBM_OBAR_STATIC_SCRATCH_BYTES);
    set_last_message(msg);
    return QGX_ERR_ARG;
  }
  void* scratch = nullptr;
  const int rc = scratch_for_current_device(&scratch);
  if (rc != QGX_OK) return rc;
  return qgx_rbm_obar(table, n, m, has_vbias, spins, r, ns, Obar, ldo, omean, scratch,
                      QGX_RBM_OBAR_STATIC_SCRATCH_BYTES, stream);
}

}  // extern "C"
