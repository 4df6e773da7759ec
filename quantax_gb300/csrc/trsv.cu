// Triangular solves with an FP32 Cholesky factor, the preconditioner of the mixed-precision
// SR solve: v <- L^-1 v, then v <- L^-T v, for L lower triangular, n x n, column-major (as
// cuSOLVER's Xpotrf leaves it; the other triangle is not read).
//
// Decoupled block substitution: 64-row blocks; a CTA takes block b in ticket order (an
// atomic counter, so block b's CTA started after the CTAs of every block it waits on) and
// folds in each earlier block k's contribution L_bk y_k as soon as block k's flag is
// published, then applies the precomputed inverse of its diagonal block and publishes y_b.
// The backward pass runs the blocks in reverse order with L^T. Every wait on a flag is bounded
// (2 s of the global timer); a wait that runs out sets the error word and the CTA goes on
// with what it has, so the caller sees a wrong residual and falls back.
#include <algorithm>

#include "qgx_common.cuh"

namespace qgx {

int64_t trsv_chol_workspace_bytes(int64_t n);
int trsv_chol_prepare(const float* L, int64_t n, void* work, cudaStream_t st);
int trsv_chol_apply(const float* L, int64_t n, float* v, void* work, uint32_t epoch, cudaStream_t st);
int trsv_chol_error(int64_t n, void* work, int* host_err, cudaStream_t st);

namespace {

constexpr int kNB = 64;            // rows per block
constexpr int kTrsvThreads = 256;  // 4 column groups x 64 rows
constexpr unsigned long long kFlagWaitNs = 2000000000ull;

struct TrsvWork {
  float* dinv;   // nblk x 64 x 64: inverses of the diagonal blocks, row-major per block
  int* flags;    // 2 x nblk: forward / backward publication epochs
  int* tickets;  // 2
  int* err;      // 1
};

inline int64_t nblocks(int64_t n) { return (n + kNB - 1) / kNB; }
inline int64_t al256(int64_t b) { return (b + 255) / 256 * 256; }

TrsvWork layout(int64_t n, void* base) {
  char* b = static_cast<char*>(base);
  const int64_t nb = nblocks(n);
  TrsvWork w;
  w.dinv = reinterpret_cast<float*>(b);
  b += al256(nb * kNB * kNB * 4);
  w.flags = reinterpret_cast<int*>(b);
  b += al256(2 * nb * 4);
  w.tickets = reinterpret_cast<int*>(b);
  w.err = w.tickets + 2;
  return w;
}

__device__ inline uint64_t gtimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ inline int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ inline void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// bounded wait of one lane for flag == epoch; false (and the error word set) on timeout
__device__ inline bool wait_flag(const int* flag, int epoch, int* err) {
  if (ld_acquire(flag) == epoch) return true;
  const uint64_t t0 = gtimer();
  while (ld_acquire(flag) != epoch) {
    if (gtimer() - t0 > kFlagWaitNs) {
      atomicExch(err, 1);
      return false;
    }
  }
  return true;
}

// inverse of every diagonal block (one CTA per block): thread c solves L_bb x = e_c by forward
// substitution; dinv[b][i][c] = x_i (rows past n: identity)
__global__ void dinv_kernel(const float* __restrict__ L, int64_t n, float* __restrict__ dinv) {
  __shared__ float D[kNB][kNB + 1];
  const int64_t b = blockIdx.x, r0 = b * kNB;
  const int nb = (int)std::min<int64_t>(kNB, n - r0);
  for (int e = threadIdx.x; e < kNB * kNB; e += blockDim.x) {
    const int i = e / kNB, j = e % kNB;  // D[i][j] = L[r0 + i][r0 + j]
    float v = 0.0f;
    if (i < nb && j < nb && j <= i) v = L[(r0 + j) * n + (r0 + i)];
    if (i >= nb && i == j) v = 1.0f;
    D[i][j] = v;
  }
  __syncthreads();
  const int c = threadIdx.x;
  if (c < kNB) {
    float x[kNB];
#pragma unroll
    for (int i = 0; i < kNB; ++i) {
      float s = (i == c) ? 1.0f : 0.0f;
      for (int j = 0; j < i; ++j) s = fmaf(-D[i][j], x[j], s);
      x[i] = s / D[i][i];
    }
    float* out = dinv + b * kNB * kNB;
#pragma unroll
    for (int i = 0; i < kNB; ++i) out[i * kNB + c] = x[i];
  }
}

// forward: v_b <- L_bb^-1 (v_b - sum_{k<b} L_bk v_k)
__global__ void __launch_bounds__(kTrsvThreads) trsv_lower_kernel(const float* __restrict__ L, int64_t n,
                                                                  float* __restrict__ v,
                                                                  const float* __restrict__ dinv, int* flags,
                                                                  int* ticket, int epoch, int* err) {
  __shared__ int sb;
  __shared__ float part[4][kNB];
  __shared__ float acc[kNB];
  __shared__ float D[kNB][kNB + 1];  // the diagonal block's inverse, padded against bank conflicts
  if (threadIdx.x == 0) sb = atomicAdd(ticket, 1);
  __syncthreads();
  const int64_t b = sb, r0 = b * kNB;
  const int nb = (int)std::min<int64_t>(kNB, n - r0);
  const int t = threadIdx.x, i = t & (kNB - 1), g = t >> 6, lane = t & 31;
  for (int e = t; e < kNB * kNB; e += blockDim.x) D[e / kNB][e % kNB] = dinv[b * kNB * kNB + e];
  float a = 0.0f;
  for (int64_t k = 0; k < b; ++k) {
    if (lane == 0) wait_flag(flags + k, epoch, err);
    __syncwarp();
    const int64_t c0 = k * kNB;
    if (i < nb) {
      const float* col = L + c0 * n + r0 + i;
#pragma unroll 4
      for (int j = g; j < kNB; j += 4) a = fmaf(col[(int64_t)j * n], __ldcg(v + c0 + j), a);
    }
  }
  part[g][i] = a;
  __syncthreads();
  if (t < kNB) acc[t] = (t < nb ? __ldcg(v + r0 + t) : 0.0f) - (part[0][t] + part[1][t] + part[2][t] + part[3][t]);
  __syncthreads();
  if (t < nb) {
    float y = 0.0f;
    for (int j = 0; j <= t; ++j) y = fmaf(D[t][j], acc[j], y);
    __stcg(v + r0 + t, y);
  }
  __threadfence();
  __syncthreads();
  if (t == 0) st_release(flags + b, epoch);
}

// backward: v_b <- L_bb^-T (v_b - sum_{k>b} L_kb^T v_k), blocks in reverse ticket order
__global__ void __launch_bounds__(kTrsvThreads) trsv_upper_kernel(const float* __restrict__ L, int64_t n,
                                                                  float* __restrict__ v,
                                                                  const float* __restrict__ dinv, int* flags,
                                                                  int* ticket, int epoch, int* err) {
  __shared__ int sb;
  __shared__ float acc[kNB];
  __shared__ float D[kNB][kNB + 1];
  const int64_t nbk = (n + kNB - 1) / kNB;
  if (threadIdx.x == 0) sb = (int)(nbk - 1) - atomicAdd(ticket, 1);
  __syncthreads();
  const int64_t b = sb, r0 = b * kNB;
  const int nb = (int)std::min<int64_t>(kNB, n - r0);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  for (int e = t; e < kNB * kNB; e += blockDim.x) D[e / kNB][e % kNB] = dinv[b * kNB * kNB + e];
  const int* bflags = flags + nbk;  // the backward pass's publications
  // warp w owns columns i = w, w + 8, ... of block b: a_i = sum_{rows j of later blocks} L[j][r0 + i] v_j
  float a[kNB / 8];
#pragma unroll
  for (int q = 0; q < kNB / 8; ++q) a[q] = 0.0f;
  for (int64_t k = nbk - 1; k > b; --k) {
    if (lane == 0) wait_flag(bflags + k, epoch, err);
    __syncwarp();
    const int64_t j0 = k * kNB;
    const int kn = (int)std::min<int64_t>(kNB, n - j0);
    const float v0 = lane < kn ? __ldcg(v + j0 + lane) : 0.0f;
    const float v1 = lane + 32 < kn ? __ldcg(v + j0 + lane + 32) : 0.0f;
#pragma unroll
    for (int q = 0; q < kNB / 8; ++q) {
      const int i = warp + 8 * q;
      if (i < nb) {
        const float* col = L + (r0 + i) * n + j0;  // column r0 + i, rows j0 ..
        float s = lane < kn ? col[lane] * v0 : 0.0f;
        if (lane + 32 < kn) s = fmaf(col[lane + 32], v1, s);
        a[q] += s;
      }
    }
  }
#pragma unroll
  for (int q = 0; q < kNB / 8; ++q) {
    const float s = warp_sum(a[q]);
    const int i = warp + 8 * q;
    if (lane == 0 && i < kNB) acc[i] = (i < nb ? __ldcg(v + r0 + i) : 0.0f) - s;
  }
  __syncthreads();
  if (t < nb) {
    // x_t = sum_j (L_bb^-T)[t][j] acc_j = sum_{j >= t} dinv[j][t] acc_j
    float x = 0.0f;
    for (int j = t; j < nb; ++j) x = fmaf(D[j][t], acc[j], x);
    __stcg(v + r0 + t, x);
  }
  __threadfence();
  __syncthreads();
  if (t == 0) st_release(flags + nbk + b, epoch);
}

}  // namespace

int64_t trsv_chol_workspace_bytes(int64_t n) {
  const int64_t nb = nblocks(n);
  return al256(nb * kNB * kNB * 4) + al256(2 * nb * 4) + al256(16);
}

// inverses of the diagonal blocks; flags, tickets and the error word cleared
int trsv_chol_prepare(const float* L, int64_t n, void* work, cudaStream_t st) {
  const TrsvWork w = layout(n, work);
  const int64_t nb = nblocks(n);
  QGX_CHECK_CUDA(cudaMemsetAsync(w.flags, 0, 2 * nb * sizeof(int), st));
  QGX_CHECK_CUDA(cudaMemsetAsync(w.tickets, 0, 3 * sizeof(int), st));
  dinv_kernel<<<(unsigned)nb, kNB, 0, st>>>(L, n, w.dinv);
  return launch_status();
}

// v <- L^-T L^-1 v; epoch: distinct positive value per apply since the last prepare
int trsv_chol_apply(const float* L, int64_t n, float* v, void* work, uint32_t epoch, cudaStream_t st) {
  const TrsvWork w = layout(n, work);
  const int64_t nb = nblocks(n);
  QGX_CHECK_CUDA(cudaMemsetAsync(w.tickets, 0, 2 * sizeof(int), st));
  trsv_lower_kernel<<<(unsigned)nb, kTrsvThreads, 0, st>>>(L, n, v, w.dinv, w.flags, w.tickets, (int)epoch, w.err);
  trsv_upper_kernel<<<(unsigned)nb, kTrsvThreads, 0, st>>>(L, n, v, w.dinv, w.flags, w.tickets + 1, (int)epoch,
                                                           w.err);
  return launch_status();
}

int trsv_chol_error(int64_t n, void* work, int* host_err, cudaStream_t st) {
  QGX_CHECK_CUDA(cudaMemcpyAsync(host_err, layout(n, work).err, sizeof(int), cudaMemcpyDeviceToHost, st));
  return QGX_OK;
}

}  // namespace qgx
