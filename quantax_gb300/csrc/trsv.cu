// Triangular solves with an FP32 Cholesky factor, the preconditioner of the mixed-precision
// SR solve: v <- L^-1 v, then v <- L^-T v, for L lower triangular, n x n, column-major (as
// cuSOLVER's Xpotrf leaves it; the other triangle is not read).
//
// Decoupled block substitution: 128-row blocks; a CTA takes block b in ticket order (an
// atomic counter, so block b's CTA started after the CTAs of every block it waits on) and
// folds in each earlier block k's contribution L_bk y_k as soon as block k's flag is
// published, then applies the precomputed inverse of its diagonal block and publishes y_b.
// The backward pass runs the blocks in reverse order with L^T. The chain of publications is
// the critical path, so the L tile of block k is loaded before its flag is awaited (it does
// not depend on the flag) and only the 128 published values are read after it. Every wait on
// a flag is bounded (2 s of the global timer); a wait that runs out sets the error word and
// the CTA goes on with what it has, so the caller sees a wrong residual and falls back.
#include <algorithm>

#include "qgx_common.cuh"

namespace qgx {

int64_t trsv_chol_workspace_bytes(int64_t n);
int trsv_chol_prepare(const float* L, int64_t n, void* work, cudaStream_t st);
int trsv_chol_apply(const float* L, int64_t n, float* v, void* work, uint32_t epoch, cudaStream_t st);
int trsv_chol_error(int64_t n, void* work, int* host_err, cudaStream_t st);
int64_t trsv64_rowmajor_workspace_bytes(int64_t n);
int trsv64_rowmajor_solve(const double* L, int64_t n, double* x, void* work, cudaStream_t st);

namespace {

constexpr int kNB = 128;                 // rows per block
constexpr int kGroups = 4;               // column groups of the off-diagonal products
constexpr int kTrsvThreads = kNB * kGroups;  // 512
constexpr int kDPitch = kNB + 1;         // padded row of a diagonal block's inverse in shared memory
constexpr unsigned long long kFlagWaitNs = 2000000000ull;

struct TrsvWork {
  float* dinv;   // nblk x 128 x 128: inverses of the diagonal blocks, row-major per block
  int* flags;    // 2 x nblk: forward / backward publication epochs
  int* tickets;  // 2
  int* err;      // 1
};

inline int64_t nblocks(int64_t n) { return (n + kNB - 1) / kNB; }
inline int64_t al256(int64_t b) { return (b + 255) / 256 * 256; }
inline size_t trsv_smem_bytes() { return (size_t)kNB * kDPitch * 4 + (size_t)(kGroups + 1) * kNB * 4; }

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

// every warp's lane 0 waits, then the warp proceeds
__device__ inline void warp_wait_flag(const int* flag, int epoch, int* err) {
  if ((threadIdx.x & 31) == 0) wait_flag(flag, epoch, err);
  __syncwarp();
}

// inverse of every diagonal block (one CTA per block): thread c solves L_bb x = e_c by forward
// substitution in shared memory; dinv[b][i][c] = x_i (rows past n: identity)
__global__ void __launch_bounds__(kNB) dinv_kernel(const float* __restrict__ L, int64_t n, float* __restrict__ dinv) {
  extern __shared__ float smem[];
  float* D = smem;                // [kNB][kDPitch]
  float* X = D + kNB * kDPitch;   // [kNB][kNB + 1]: column c of the inverse in column c
  const int64_t b = blockIdx.x, r0 = b * kNB;
  const int nb = (int)std::min<int64_t>(kNB, n - r0);
  for (int e = threadIdx.x; e < kNB * kNB; e += blockDim.x) {
    const int i = e / kNB, j = e % kNB;  // D[i][j] = L[r0 + i][r0 + j]
    float v = 0.0f;
    if (i < nb && j < nb && j <= i) v = L[(r0 + j) * n + (r0 + i)];
    if (i >= nb && i == j) v = 1.0f;
    D[i * kDPitch + j] = v;
  }
  __syncthreads();
  const int c = threadIdx.x;
  for (int i = 0; i < kNB; ++i) {
    float s = (i == c) ? 1.0f : 0.0f;
    for (int j = c; j < i; ++j) s = fmaf(-D[i * kDPitch + j], X[j * (kNB + 1) + c], s);  // x_j = 0 for j < c
    X[i * (kNB + 1) + c] = i < c ? 0.0f : s / D[i * kDPitch + i];
  }
  __syncthreads();
  float* out = dinv + b * kNB * kNB;
  for (int e = threadIdx.x; e < kNB * kNB; e += blockDim.x) out[e] = X[(e / kNB) * (kNB + 1) + (e % kNB)];
}

// forward: v_b <- L_bb^-1 (v_b - sum_{k<b} L_bk v_k)
// thread (g, i): row r0 + i, columns c0 + g + 4 jj of every earlier block
__global__ void __launch_bounds__(kTrsvThreads) trsv_lower_kernel(const float* __restrict__ L, int64_t n,
                                                                  float* __restrict__ v,
                                                                  const float* __restrict__ dinv, int* flags,
                                                                  int* ticket, int epoch, int* err) {
  extern __shared__ float smem[];
  float* D = smem;                  // the diagonal block's inverse [kNB][kDPitch]
  float* part = D + kNB * kDPitch;  // [kGroups][kNB]
  float* acc = part + kGroups * kNB;
  __shared__ int sb;
  if (threadIdx.x == 0) sb = atomicAdd(ticket, 1);
  __syncthreads();
  const int64_t b = sb, r0 = b * kNB;
  const int nb = (int)std::min<int64_t>(kNB, n - r0);
  const int t = threadIdx.x, i = t & (kNB - 1), g = t >> 7;
  for (int e = t; e < kNB * kNB; e += blockDim.x) D[(e / kNB) * kDPitch + e % kNB] = dinv[b * kNB * kNB + e];
  float a = 0.0f;
  constexpr int kPer = kNB / kGroups;  // 32 columns of each earlier block per thread
  for (int64_t k = 0; k < b; ++k) {
    const int64_t c0 = k * kNB;
    float lv[kPer];
    if (i < nb) {
      const float* col = L + (c0 + g) * n + r0 + i;
#pragma unroll
      for (int jj = 0; jj < kPer; ++jj) lv[jj] = col[(int64_t)(kGroups * jj) * n];
    }
    warp_wait_flag(flags + k, epoch, err);
    if (i < nb) {
#pragma unroll
      for (int jj = 0; jj < kPer; ++jj) a = fmaf(lv[jj], __ldcg(v + c0 + g + kGroups * jj), a);
    }
  }
  part[g * kNB + i] = a;
  __syncthreads();
  if (t < kNB) {
    float s = t < nb ? __ldcg(v + r0 + t) : 0.0f;
#pragma unroll
    for (int q = 0; q < kGroups; ++q) s -= part[q * kNB + t];
    acc[t] = s;
  }
  __syncthreads();
  // y_i = sum_{j <= i} D[i][j] acc_j, the j range split over the four groups
  {
    float y = 0.0f;
    const int j0 = g * kPer;
#pragma unroll 8
    for (int j = j0; j < j0 + kPer; ++j)
      if (j <= i) y = fmaf(D[i * kDPitch + j], acc[j], y);
    part[g * kNB + i] = y;
  }
  __syncthreads();
  if (t < nb) __stcg(v + r0 + t, part[t] + part[kNB + t] + part[2 * kNB + t] + part[3 * kNB + t]);
  __threadfence();
  __syncthreads();
  if (t == 0) st_release(flags + b, epoch);
}

// backward: v_b <- L_bb^-T (v_b - sum_{k>b} L_kb^T v_k), blocks in reverse ticket order
// warp w owns columns i = w + 16 q of block b; lane l covers rows j0 + l + 32 r of block k
__global__ void __launch_bounds__(kTrsvThreads) trsv_upper_kernel(const float* __restrict__ L, int64_t n,
                                                                  float* __restrict__ v,
                                                                  const float* __restrict__ dinv, int* flags,
                                                                  int* ticket, int epoch, int* err) {
  extern __shared__ float smem[];
  float* D = smem;
  float* part = D + kNB * kDPitch;
  float* acc = part + kGroups * kNB;
  __shared__ int sb;
  constexpr int kWarps = kTrsvThreads / 32;  // 16
  constexpr int kCols = kNB / kWarps;        // 8 columns per warp
  constexpr int kRows = kNB / 32;            // 4 rows per lane
  const int64_t nbk = (n + kNB - 1) / kNB;
  if (threadIdx.x == 0) sb = (int)(nbk - 1) - atomicAdd(ticket, 1);
  __syncthreads();
  const int64_t b = sb, r0 = b * kNB;
  const int nb = (int)std::min<int64_t>(kNB, n - r0);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  for (int e = t; e < kNB * kNB; e += blockDim.x) D[(e / kNB) * kDPitch + e % kNB] = dinv[b * kNB * kNB + e];
  const int* bflags = flags + nbk;  // the backward pass's publications
  float a[kCols];
#pragma unroll
  for (int q = 0; q < kCols; ++q) a[q] = 0.0f;
  for (int64_t k = nbk - 1; k > b; --k) {
    const int64_t j0 = k * kNB;
    const int kn = (int)std::min<int64_t>(kNB, n - j0);
    float lv[kCols][kRows];
#pragma unroll
    for (int q = 0; q < kCols; ++q) {
      const int ic = warp + kWarps * q;
      const float* col = L + (r0 + ic) * n + j0;  // column r0 + ic, rows j0 ..
#pragma unroll
      for (int r = 0; r < kRows; ++r) {
        const int row = lane + 32 * r;
        lv[q][r] = (ic < nb && row < kn) ? col[row] : 0.0f;
      }
    }
    warp_wait_flag(bflags + k, epoch, err);
    float vv[kRows];
#pragma unroll
    for (int r = 0; r < kRows; ++r) vv[r] = lane + 32 * r < kn ? __ldcg(v + j0 + lane + 32 * r) : 0.0f;
#pragma unroll
    for (int q = 0; q < kCols; ++q)
#pragma unroll
      for (int r = 0; r < kRows; ++r) a[q] = fmaf(lv[q][r], vv[r], a[q]);
  }
#pragma unroll
  for (int q = 0; q < kCols; ++q) {
    const float s = warp_sum(a[q]);
    const int ic = warp + kWarps * q;
    if (lane == 0) acc[ic] = (ic < nb ? __ldcg(v + r0 + ic) : 0.0f) - s;
  }
  __syncthreads();
  // x_i = sum_{j >= i} (L_bb^-1)[j][i] acc_j, the j range split over four groups
  {
    const int i = t & (kNB - 1), g = t >> 7;
    constexpr int kPer = kNB / kGroups;
    float x = 0.0f;
    const int j0 = g * kPer;
#pragma unroll 8
    for (int j = j0; j < j0 + kPer; ++j)
      if (j >= i) x = fmaf(D[j * kDPitch + i], acc[j], x);
    part[g * kNB + i] = x;
  }
  __syncthreads();
  if (t < nb) __stcg(v + r0 + t, part[t] + part[kNB + t] + part[2 * kNB + t] + part[3 * kNB + t]);
  __threadfence();
  __syncthreads();
  if (t == 0) st_release(flags + nbk + b, epoch);
}

// ---- FP64 solves with a row-major factor ------------------------------------------------------
// The FP64 Cholesky (chol.cu) leaves L in the row-major lower triangle of its n x n matrix (row
// stride n). x <- L^-T L^-1 x by the same decoupled block substitution, in 64-row blocks:
//   * the forward pass reads the rows of each earlier block's tile (warps over rows, lanes along
//     the contiguous columns, a warp sum per row);
//   * the backward pass reads the rows of each later block that hold L_kb (threads along the
//     contiguous columns of block b, four row groups);
//   * each diagonal block is applied through its precomputed inverse (a 64 x 64 product spread
//     over the CTA): a serial substitution in one warp runs at GB300's FP64 rate of about two
//     FMAs per clock per SM and measured slower than cuSOLVER's Xpotrs. On an ill-conditioned
//     shifted Gram (condition number 1e10) the residual equals the substitution's.
constexpr int kNB64 = 64;
constexpr int kT64 = 256;  // 8 warps
constexpr int kDP64 = kNB64 + 1;

__host__ __device__ inline int64_t nblocks64(int64_t n) { return (n + kNB64 - 1) / kNB64; }

// inverses of the 64 x 64 diagonal blocks (one CTA per block): thread c solves L_bb x = e_c by
// forward substitution in shared memory; dinv[b][i][c] = x_i (rows past n: identity)
__global__ void __launch_bounds__(kNB64) dinv64_kernel(const double* __restrict__ L, int64_t n,
                                                       double* __restrict__ dinv) {
  extern __shared__ double sm64[];
  double* D = sm64;              // [kNB64][kDP64]
  double* X = D + kNB64 * kDP64;  // [kNB64][kDP64]: column c of the inverse in column c
  const int64_t b = blockIdx.x, r0 = b * kNB64;
  const int nb = (int)std::min<int64_t>(kNB64, n - r0);
  for (int e = threadIdx.x; e < kNB64 * kNB64; e += blockDim.x) {
    const int i = e / kNB64, j = e % kNB64;
    double v = 0.0;
    if (i < nb && j <= i) v = L[(r0 + i) * n + r0 + j];
    if (i >= nb && i == j) v = 1.0;
    D[i * kDP64 + j] = v;
  }
  __syncthreads();
  const int c = threadIdx.x;
  for (int i = 0; i < kNB64; ++i) {
    double s = (i == c) ? 1.0 : 0.0;
    for (int j = c; j < i; ++j) s = fma(-D[i * kDP64 + j], X[j * kDP64 + c], s);  // x_j = 0 for j < c
    X[i * kDP64 + c] = i < c ? 0.0 : s / D[i * kDP64 + i];
  }
  __syncthreads();
  double* out = dinv + b * kNB64 * kNB64;
  for (int e = threadIdx.x; e < kNB64 * kNB64; e += blockDim.x) out[e] = X[(e / kNB64) * kDP64 + (e % kNB64)];
}

// forward: v_b <- L_bb^-1 (v_b - sum_{k<b} L_bk v_k), blocks in ticket order
__global__ void __launch_bounds__(kT64) trsv64_lower_kernel(const double* __restrict__ L, int64_t n,
                                                            double* __restrict__ v, const double* __restrict__ dinv,
                                                            int* flags, int* ticket, int epoch, int* err) {
  __shared__ double D[kNB64][kDP64];  // L_bb^-1
  __shared__ double part[kT64 / kNB64][kNB64];
  __shared__ double acc[kNB64];
  __shared__ int sb;
  if (threadIdx.x == 0) sb = atomicAdd(ticket, 1);
  __syncthreads();
  const int64_t b = sb, r0 = b * kNB64;
  const int nb = (int)std::min<int64_t>(kNB64, n - r0);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  for (int e = t; e < kNB64 * kNB64; e += blockDim.x) D[e / kNB64][e % kNB64] = dinv[b * kNB64 * kNB64 + e];
  constexpr int kRowsPerWarp = kNB64 / (kT64 / 32);  // 8: rows warp + 8 q
  double a[kRowsPerWarp];
#pragma unroll
  for (int q = 0; q < kRowsPerWarp; ++q) a[q] = 0.0;
  for (int64_t k = 0; k < b; ++k) {  // earlier blocks are whole (only the last block is short)
    const int64_t c0 = k * kNB64;
    double lv[kRowsPerWarp][2];
#pragma unroll
    for (int q = 0; q < kRowsPerWarp; ++q) {
      const int i = warp + 8 * q;
#pragma unroll
      for (int r = 0; r < 2; ++r) lv[q][r] = i < nb ? L[(r0 + i) * n + c0 + lane + 32 * r] : 0.0;
    }
    warp_wait_flag(flags + k, epoch, err);
    const double v0 = __ldcg(v + c0 + lane), v1 = __ldcg(v + c0 + lane + 32);
#pragma unroll
    for (int q = 0; q < kRowsPerWarp; ++q) a[q] = fma(lv[q][1], v1, fma(lv[q][0], v0, a[q]));
  }
#pragma unroll
  for (int q = 0; q < kRowsPerWarp; ++q) {
    const double s = warp_sum(a[q]);
    const int i = warp + 8 * q;
    if (lane == 0) acc[i] = i < nb ? __ldcg(v + r0 + i) - s : 0.0;
  }
  __syncthreads();
  {  // y_i = sum_{j <= i} D[i][j] acc_j, the j range split over four groups
    const int i = t & (kNB64 - 1), g = t / kNB64;
    constexpr int kPer = kNB64 / (kT64 / kNB64);  // 16
    double y = 0.0;
    const int j0 = g * kPer;
#pragma unroll
    for (int j = j0; j < j0 + kPer; ++j)
      if (j <= i) y = fma(D[i][j], acc[j], y);
    part[g][i] = y;
  }
  __syncthreads();
  if (t < nb) __stcg(v + r0 + t, part[0][t] + part[1][t] + part[2][t] + part[3][t]);
  __threadfence();
  __syncthreads();
  if (t == 0) st_release(flags + b, epoch);
}

// backward: v_b <- L_bb^-T (v_b - sum_{k>b} L_kb^T v_k), blocks in reverse ticket order
__global__ void __launch_bounds__(kT64) trsv64_upper_kernel(const double* __restrict__ L, int64_t n,
                                                            double* __restrict__ v, const double* __restrict__ dinv,
                                                            int* flags, int* ticket, int epoch, int* err) {
  __shared__ double D[kNB64][kDP64];  // L_bb^-1
  __shared__ double part[kT64 / kNB64][kNB64];
  __shared__ double acc[kNB64];
  __shared__ int sb;
  const int64_t nbk = nblocks64(n);
  if (threadIdx.x == 0) sb = (int)(nbk - 1) - atomicAdd(ticket, 1);
  __syncthreads();
  const int64_t b = sb, r0 = b * kNB64;
  const int nb = (int)std::min<int64_t>(kNB64, n - r0);
  const int t = threadIdx.x;
  const int i = t & (kNB64 - 1), g = t / kNB64;  // column i of block b, row group g
  constexpr int kGroups64 = kT64 / kNB64;        // 4
  constexpr int kPer64 = kNB64 / kGroups64;      // 16 rows j = g + 4 jj
  for (int e = t; e < kNB64 * kNB64; e += blockDim.x) D[e / kNB64][e % kNB64] = dinv[b * kNB64 * kNB64 + e];
  const int* bflags = flags + nbk;
  double a = 0.0;
  for (int64_t k = nbk - 1; k > b; --k) {
    const int64_t j0 = k * kNB64;
    const int kn = (int)std::min<int64_t>(kNB64, n - j0);
    double lv[kPer64];
#pragma unroll
    for (int jj = 0; jj < kPer64; ++jj) {
      const int j = g + kGroups64 * jj;
      lv[jj] = (j < kn && i < nb) ? L[(j0 + j) * n + r0 + i] : 0.0;
    }
    warp_wait_flag(bflags + k, epoch, err);
#pragma unroll
    for (int jj = 0; jj < kPer64; ++jj) {
      const int j = g + kGroups64 * jj;
      if (j < kn) a = fma(lv[jj], __ldcg(v + j0 + j), a);
    }
  }
  part[g][i] = a;
  __syncthreads();
  if (t < kNB64) acc[t] = t < nb ? __ldcg(v + r0 + t) - (part[0][t] + part[1][t] + part[2][t] + part[3][t]) : 0.0;
  __syncthreads();
  {  // x_i = sum_{j >= i} D[j][i] acc_j, the j range split over four groups
    double x = 0.0;
    const int j0 = g * kPer64;
#pragma unroll
    for (int j = j0; j < j0 + kPer64; ++j)
      if (j >= i) x = fma(D[j][i], acc[j], x);
    __syncthreads();  // every thread has read part before it is overwritten
    part[g][i] = x;
  }
  __syncthreads();
  if (t < nb) __stcg(v + r0 + t, part[0][t] + part[1][t] + part[2][t] + part[3][t]);
  __threadfence();
  __syncthreads();
  if (t == 0) st_release(flags + nbk + b, epoch);
}

// a flag wait that ran out leaves wrong values: the result becomes NaN, which the caller's
// finite check of the step turns into a skipped update
__global__ void trsv64_nan_if_err_kernel(double* __restrict__ x, int64_t n, const int* __restrict__ err) {
  if (*err == 0) return;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    x[e] = __longlong_as_double(0x7FF8000000000000LL);
}

}  // namespace

int64_t trsv64_rowmajor_workspace_bytes(int64_t n) {
  const int64_t nb = nblocks64(n);
  return al256(nb * kNB64 * kNB64 * 8) + al256(2 * nb * 4) + al256(16);
}

// x <- L^-T L^-1 x for the row-major lower factor L (n x n, row stride n)
int trsv64_rowmajor_solve(const double* L, int64_t n, double* x, void* work, cudaStream_t st) {
  const int64_t nb = nblocks64(n);
  double* dinv = static_cast<double*>(work);
  char* w = static_cast<char*>(work) + al256(nb * kNB64 * kNB64 * 8);
  int* flags = reinterpret_cast<int*>(w);
  int* tickets = reinterpret_cast<int*>(w + al256(2 * nb * 4));
  int* err = tickets + 2;
  const size_t dsmem = 2 * (size_t)kNB64 * kDP64 * 8;
  QGX_CHECK_CUDA(cudaFuncSetAttribute(dinv64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsmem));
  QGX_CHECK_CUDA(cudaMemsetAsync(w, 0, al256(2 * nb * 4) + 16, st));  // flags, tickets, error word
  dinv64_kernel<<<(unsigned)nb, kNB64, dsmem, st>>>(L, n, dinv);
  trsv64_lower_kernel<<<(unsigned)nb, kT64, 0, st>>>(L, n, x, dinv, flags, tickets, 1, err);
  trsv64_upper_kernel<<<(unsigned)nb, kT64, 0, st>>>(L, n, x, dinv, flags, tickets + 1, 1, err);
  trsv64_nan_if_err_kernel<<<(unsigned)std::min<int64_t>((n + 255) / 256, 1024), 256, 0, st>>>(x, n, err);
  return launch_status();
}

int64_t trsv_chol_workspace_bytes(int64_t n) {
  const int64_t nb = nblocks(n);
  return al256(nb * kNB * kNB * 4) + al256(2 * nb * 4) + al256(16);
}

// inverses of the diagonal blocks; flags, tickets and the error word cleared
int trsv_chol_prepare(const float* L, int64_t n, void* work, cudaStream_t st) {
  const TrsvWork w = layout(n, work);
  const int64_t nb = nblocks(n);
  const size_t dsmem = (size_t)kNB * kDPitch * 4 + (size_t)kNB * (kNB + 1) * 4;
  QGX_CHECK_CUDA(cudaFuncSetAttribute(dinv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsmem));
  QGX_CHECK_CUDA(cudaFuncSetAttribute(trsv_lower_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)trsv_smem_bytes()));
  QGX_CHECK_CUDA(cudaFuncSetAttribute(trsv_upper_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)trsv_smem_bytes()));
  QGX_CHECK_CUDA(cudaMemsetAsync(w.flags, 0, 2 * nb * sizeof(int), st));
  QGX_CHECK_CUDA(cudaMemsetAsync(w.tickets, 0, 3 * sizeof(int), st));
  dinv_kernel<<<(unsigned)nb, kNB, dsmem, st>>>(L, n, w.dinv);
  return launch_status();
}

// v <- L^-T L^-1 v; epoch: distinct positive value per apply since the last prepare
int trsv_chol_apply(const float* L, int64_t n, float* v, void* work, uint32_t epoch, cudaStream_t st) {
  const TrsvWork w = layout(n, work);
  const int64_t nb = nblocks(n);
  const size_t smem = trsv_smem_bytes();
  QGX_CHECK_CUDA(cudaMemsetAsync(w.tickets, 0, 2 * sizeof(int), st));
  trsv_lower_kernel<<<(unsigned)nb, kTrsvThreads, smem, st>>>(L, n, v, w.dinv, w.flags, w.tickets, (int)epoch,
                                                               w.err);
  trsv_upper_kernel<<<(unsigned)nb, kTrsvThreads, smem, st>>>(L, n, v, w.dinv, w.flags, w.tickets + 1, (int)epoch,
                                                               w.err);
  return launch_status();
}

int trsv_chol_error(int64_t n, void* work, int* host_err, cudaStream_t st) {
  QGX_CHECK_CUDA(cudaMemcpyAsync(host_err, layout(n, work).err, sizeof(int), cudaMemcpyDeviceToHost, st));
  return QGX_OK;
}

}  // namespace qgx
