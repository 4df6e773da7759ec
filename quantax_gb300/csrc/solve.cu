// FP64 SR / MinSR solve (quantax/optimizer/solver.py:50-201): diagonal-shifted Cholesky
// (cuSOLVER Xpotrf / Xpotrs) or the soft pseudo-inverse through an FP64 eigendecomposition
// (cuSOLVER Xsyevd), followed by the projection x = A^T y over the FP32 Obar matrix.
//
// The Gram matrix is symmetric, so the row-major buffer written by qgx_gram is also its
// own column-major image and is handed to cuSOLVER as is.
#include <cusolverDn.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "qgx_common.cuh"

namespace qgx {

int64_t trsv_chol_workspace_bytes(int64_t n);
int64_t trsv64_rowmajor_workspace_bytes(int64_t n);
int trsv64_rowmajor_solve(const double* L, int64_t n, double* x, void* work, cudaStream_t st);
int trsv_chol_prepare(const float* L, int64_t n, void* work, cudaStream_t st);
int trsv_chol_apply(const float* L, int64_t n, float* v, void* work, uint32_t epoch, cudaStream_t st);
int trsv_chol_error(int64_t n, void* work, int* host_err, cudaStream_t st);
int64_t chol_f64_workspace_bytes(int64_t n);
int chol_f64(double* A, int64_t n, int64_t lda, int* info, int32_t* status, void* work, cudaStream_t st,
             int64_t* kernels);
// chol_f64 captured once per set of buffers into a CUDA graph and replayed (chol.cu)
int chol_f64_graph(double* A, int64_t n, int64_t lda, int* info, int32_t* status, void* work, cudaStream_t st,
                   int64_t* kernels);

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_solver_mutex;
cusolverDnHandle_t g_handle[kMaxDevices] = {};
cusolverDnParams_t g_params[kMaxDevices] = {};
thread_local std::vector<char> g_host_ws;

int solver_for_current_device(cusolverDnHandle_t* h, cusolverDnParams_t* p) {
  int dev = 0;
  QGX_CHECK_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return QGX_ERR_UNSUPPORTED;
  if (!g_handle[dev]) {
    if (cusolverDnCreate(&g_handle[dev]) != CUSOLVER_STATUS_SUCCESS) return QGX_ERR_SOLVER;
    if (cusolverDnCreateParams(&g_params[dev]) != CUSOLVER_STATUS_SUCCESS) return QGX_ERR_SOLVER;
  }
  *h = g_handle[dev];
  *p = g_params[dev];
  return QGX_OK;
}

// One cuSOLVER handle per stream for the solves themselves: a handle's routines keep scratch
// memory that belongs to the handle (its internal cuBLAS workspace), so callers on different
// streams (the jobs of a serving loop) each get their own handle and never share it, with no
// ordering between their streams. At most kMaxStreamSolvers handles are kept (least recently
// used destroyed first); the handle's stream is set on every use, since a stream's address can
// be reused by a later stream. Callers hold g_solver_mutex.
struct StreamSolver {
  int dev;
  cudaStream_t st;
  cusolverDnHandle_t h;
  cusolverDnParams_t p;
  uint64_t last_use;
};
constexpr size_t kMaxStreamSolvers = 32;
std::vector<StreamSolver> g_stream_solvers;
uint64_t g_solver_clock = 0;

int solver_for_stream(cudaStream_t st, cusolverDnHandle_t* h, cusolverDnParams_t* p) {
  int dev = 0;
  QGX_CHECK_CUDA(cudaGetDevice(&dev));
  StreamSolver* hit = nullptr;
  for (auto& e : g_stream_solvers)
    if (e.dev == dev && e.st == st) hit = &e;
  if (!hit) {
    if (g_stream_solvers.size() >= kMaxStreamSolvers) {
      auto lru = std::min_element(g_stream_solvers.begin(), g_stream_solvers.end(),
                                  [](const StreamSolver& a, const StreamSolver& b) { return a.last_use < b.last_use; });
      cusolverDnDestroyParams(lru->p);
      cusolverDnDestroy(lru->h);
      g_stream_solvers.erase(lru);
    }
    StreamSolver e{dev, st, nullptr, nullptr, 0};
    if (cusolverDnCreate(&e.h) != CUSOLVER_STATUS_SUCCESS) return QGX_ERR_SOLVER;
    if (cusolverDnCreateParams(&e.p) != CUSOLVER_STATUS_SUCCESS) {
      cusolverDnDestroy(e.h);
      return QGX_ERR_SOLVER;
    }
    g_stream_solvers.push_back(e);
    hit = &g_stream_solvers.back();
  }
  hit->last_use = ++g_solver_clock;
  if (cusolverDnSetStream(hit->h, st) != CUSOLVER_STATUS_SUCCESS) return QGX_ERR_SOLVER;
  *h = hit->h;
  *p = hit->p;
  return QGX_OK;
}

// a cuSOLVER call's status as a qgx status
template <typename F>
int cus_status(F&& call) {
  return call() == CUSOLVER_STATUS_SUCCESS ? QGX_OK : QGX_ERR_SOLVER;
}

constexpr int kProjRows = 256;  // rows per partial sum of the projection x = A^T y

inline int64_t al256(int64_t b) { return (b + 255) / 256 * 256; }

// trace -> shift = rshift * tr + ashift -> added to the diagonal (single block)
__global__ void shift_diag_kernel(double* __restrict__ T, int64_t n, int64_t ldt, double rshift, double ashift,
                                  double* __restrict__ shift_out) {
  __shared__ double sh[32];
  KahanD k;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) k.add(T[i * ldt + i]);
  double v = warp_sum(k.value());
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) sh[0] = v;
  }
  __syncthreads();
  const double shift = rshift * sh[0] + ashift;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) T[i * ldt + i] += shift;
  if (threadIdx.x == 0 && shift_out) {
    shift_out[0] = shift;
    shift_out[1] = sh[0];  // trace before the shift
  }
}

// partial[chunk, col] = sum_{rows in chunk} A[s, col] y[s] to about 48 bits (the reference
// forms x = A^T y in float64, solver.py:58-61, 144-146), as float-pair sums (DSum) with
// y = yh + yl. Four columns per thread, 16-byte loads; the chunk's y split once into shared
// memory.
__global__ void project_partial_kernel(const float* __restrict__ A, int64_t nrow, int64_t ncol, int64_t lda,
                                       const double* __restrict__ y, double* __restrict__ part, bool vec4) {
  __shared__ float2 ys[kProjRows];
  const int64_t r0 = (int64_t)blockIdx.y * kProjRows;
  const int64_t r1 = min(nrow, r0 + kProjRows);
  for (int64_t s = r0 + threadIdx.x; s < r1; s += blockDim.x) {
    ys[s - r0] = split_double(y[s]);
  }
  __syncthreads();
  const int64_t c0 = 4 * (blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
  if (c0 >= ncol) return;
  DSum a0, a1, a2, a3;
  if (vec4 && c0 + 3 < ncol) {
#pragma unroll 4
    for (int64_t s = r0; s < r1; ++s) {
      const float2 yv = ys[s - r0];
      const float4 v = __ldg(reinterpret_cast<const float4*>(A + s * lda + c0));
      a0.add_prod(v.x, yv.x, yv.y);
      a1.add_prod(v.y, yv.x, yv.y);
      a2.add_prod(v.z, yv.x, yv.y);
      a3.add_prod(v.w, yv.x, yv.y);
    }
  } else {
    for (int64_t s = r0; s < r1; ++s) {
      const float2 yv = ys[s - r0];
      const float* row = A + s * lda;
      a0.add_prod(__ldg(row + c0), yv.x, yv.y);
      if (c0 + 1 < ncol) a1.add_prod(__ldg(row + c0 + 1), yv.x, yv.y);
      if (c0 + 2 < ncol) a2.add_prod(__ldg(row + c0 + 2), yv.x, yv.y);
      if (c0 + 3 < ncol) a3.add_prod(__ldg(row + c0 + 3), yv.x, yv.y);
    }
  }
  double* p = part + blockIdx.y * ncol + c0;
  p[0] = a0.value();
  if (c0 + 1 < ncol) p[1] = a1.value();
  if (c0 + 2 < ncol) p[2] = a2.value();
  if (c0 + 3 < ncol) p[3] = a3.value();
}

__global__ void sum_partials_kernel(const double* __restrict__ part, int64_t nchunk, int64_t ncol,
                                    double* __restrict__ x) {
  const int64_t col = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  KahanD k;
  for (int64_t c = 0; c < nchunk; ++c) k.add(part[c * ncol + col]);
  x[col] = k.value();
}

// soft inverse of the eigenvalues (solver.py:95-101), single block
__global__ void eigs_inv_kernel(const double* __restrict__ w, int64_t n, double rtol, double atol,
                                double* __restrict__ inv) {
  __shared__ double sh[32];
  double mx = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) mx = fmax(mx, fabs(w[i]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (threadIdx.x == 0) sh[0] = v;
  }
  __syncthreads();
  mx = sh[0];
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const double a = fabs(w[i]);
    double r = 0.0;
    if (a > 0.0) {
      const double q = (rtol * mx + atol) / a;
      const double q2 = q * q;
      r = 1.0 / (w[i] * (1.0 + q2 * q2 * q2));
    }
    inv[i] = r;
  }
}

// v_j = inv_j * rho_j, rho_j = sum_without_noise(U[:, j] * b) (solver.py:114-125, 128-149).
// U column-major (column j contiguous); one warp per column.
__global__ void rho_kernel(const double* __restrict__ U, int64_t n, const double* __restrict__ b,
                           const double* __restrict__ inv, double tol_snr, double* __restrict__ v) {
  const int64_t j = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (j >= n) return;
  const double* col = U + j * n;
  double s = 0.0;
  for (int64_t t = lane; t < n; t += 32) s += col[t] * b[t];
  s = warp_sum(s);
  double rho = s;
  if (tol_snr > 1e-6) {
    const double xm = s / (double)n;
    double q = 0.0;
    for (int64_t t = lane; t < n; t += 32) {
      const double d = col[t] * b[t] - xm;
      q += d * d;
    }
    q = warp_sum(q);
    const double xv = sqrt(q / (double)n / (double)n);
    const double snr = fabs(xm) / xv;
    const double r = tol_snr / snr;
    const double r2 = r * r;
    rho = s / (1.0 + r2 * r2 * r2);
  }
  if (lane == 0) v[j] = inv[j] * rho;
}

// y_t = sum_j U[t, j] v_j for column-major U: partials over column chunks
__global__ void uv_partial_kernel(const double* __restrict__ U, int64_t n, const double* __restrict__ v,
                                  double* __restrict__ part) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t j0 = (int64_t)blockIdx.y * kProjRows;
  const int64_t j1 = min(n, j0 + kProjRows);
  if (t >= n) return;
  double acc = 0.0;
  for (int64_t j = j0; j < j1; ++j) acc += U[j * n + t] * v[j];
  part[blockIdx.y * n + t] = acc;
}

// SR-branch noise truncation (lstsq_pinv_eig, solver.py:152-164, with _sum_without_noise,
// :114-125): the per-sample terms y[s, k] = b[s] sum_l A[s, l] V[l, k] (A FP32 row-major,
// V the FP64 eigenvectors of S, column-major) are formed tile by tile in FP64 and reduced at
// once to each 64-row chunk's mean and sum of squared deviations per column; the (ns x np)
// matrix of terms is never stored.
constexpr int kSnrRows = 64;
__global__ void __launch_bounds__(256) snr_terms_kernel(const float* __restrict__ A, int64_t ns, int64_t np,
                                                        int64_t lda, const double* __restrict__ V,
                                                        const double* __restrict__ b, double* __restrict__ part) {
  __shared__ double As[16][kSnrRows + 1];  // [l][s]
  __shared__ double Vs[16][kSnrRows + 1];  // [l][k]
  __shared__ double Ys[kSnrRows][kSnrRows + 1];
  const int64_t s0 = (int64_t)blockIdx.y * kSnrRows, k0 = (int64_t)blockIdx.x * kSnrRows;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;  // 16 x 16 threads, 4 x 4 terms each
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
  for (int64_t l0 = 0; l0 < np; l0 += 16) {
    for (int e = threadIdx.x; e < 16 * kSnrRows; e += 256) {
      const int c = e & 15, r = e >> 4;
      const int64_t srow = s0 + r, l = l0 + c, k = k0 + r;
      As[c][r] = (srow < ns && l < np) ? (double)A[srow * lda + l] : 0.0;
      Vs[c][r] = (k < np && l < np) ? V[k * np + l] : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (int c = 0; c < 16; ++c) {
      double a[4], v[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        a[i] = As[c][4 * ty + i];
        v[i] = Vs[c][4 * tx + i];
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], v[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int64_t srow = s0 + 4 * ty + i;
    const double bs = srow < ns ? b[srow] : 0.0;
#pragma unroll
    for (int j = 0; j < 4; ++j) Ys[4 * ty + i][4 * tx + j] = acc[i][j] * bs;
  }
  __syncthreads();
  if (threadIdx.x < kSnrRows) {
    const int64_t k = k0 + threadIdx.x;
    const int cnt = (int)min((int64_t)kSnrRows, ns - s0);
    if (k < np) {
      double sum = 0.0;
      for (int r = 0; r < cnt; ++r) sum += Ys[r][threadIdx.x];
      const double mean = sum / cnt;
      double m2 = 0.0;
      for (int r = 0; r < cnt; ++r) {
        const double d = Ys[r][threadIdx.x] - mean;
        m2 = fma(d, d, m2);
      }
      part[(blockIdx.y * np + k) * 2 + 0] = mean;
      part[(blockIdx.y * np + k) * 2 + 1] = m2;
    }
  }
}

// merge the chunks' (mean, M2) in chunk order (Chan, Golub and LeVeque's pairwise update),
// then x = sum, snr = |mean| / sqrt(var / ns), rho = x / (1 + (tol_snr / snr)^6), v = inv rho
__global__ void snr_rho_kernel(const double* __restrict__ part, int64_t nchunk, int64_t ns, int64_t np,
                               const double* __restrict__ inv, double tol_snr, double* __restrict__ v) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= np) return;
  double na = 0.0, mean = 0.0, m2 = 0.0;
  for (int64_t c = 0; c < nchunk; ++c) {
    const double nb = (double)min((int64_t)kSnrRows, ns - c * kSnrRows);
    const double mb = part[(c * np + k) * 2 + 0];
    const double m2b = part[(c * np + k) * 2 + 1];
    const double n = na + nb;
    const double d = mb - mean;
    mean = fma(d, nb / n, mean);
    m2 += m2b + d * d * (na * nb / n);
    na = n;
  }
  const double x = mean * (double)ns;
  double rho = x;
  if (tol_snr > 1e-6) {
    const double xv = sqrt(m2 / (double)ns / (double)ns);
    const double snr = fabs(mean) / xv;
    const double r = tol_snr / snr;
    const double r2 = r * r;
    rho = x / (1.0 + r2 * r2 * r2);
  }
  v[k] = inv[k] * rho;
}

// SHIFT_MIXED: preconditioned conjugate gradients in FP64 on (T + shift I) y = b, the
// preconditioner being the FP32 Cholesky factor of the same matrix (or of T + shift' I with
// a larger shift' when the FP32 factorisation breaks down)
constexpr int kCgMaxIters = 100;
constexpr double kCgTol = 1e-13;     // stop: recursive residual below this fraction of ||b||
constexpr double kRefineTol = 1e-10;  // accept: true residual below this fraction of ||b||
constexpr int kDotBlocks = 1024;      // fixed grid of the dot products: deterministic partial sums
enum { kScalRZ = 0, kScalAlpha, kScalBeta, kScalRR, kScalBB, kScalCount };

// FP32 copy of the shifted T, with `extra` added to the diagonal (the preconditioner's shift)
__global__ void to_f32_kernel(const double* __restrict__ in, int64_t n, float* __restrict__ out,
                              const double* __restrict__ extra) {
  const double e = extra ? *extra : 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n * n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = i / n;
    out[i] = (float)(in[i] + (i - row * n == row ? e : 0.0));
  }
}

// extra diagonal shift of the fallback preconditioner: 4 sqrt(n) 2^-24 tr(T), the size of an
// FP32 Cholesky's backward error for a matrix whose largest eigenvalue is at most tr(T)
__global__ void precond_shift_kernel(const double* __restrict__ shift_trace, int64_t n, double* __restrict__ extra) {
  *extra = 4.0 * sqrt((double)n) * 5.9604644775390625e-8 * shift_trace[1];
}

__device__ inline void block_partial(double v, double* __restrict__ part) {
  __shared__ double sh[32];
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) part[blockIdx.x] = v;
  }
}

// q = T p (warp per row, T symmetric row-major); block partials of p . q
__global__ void symv_dot_kernel(const double* __restrict__ T, int64_t n, const double* __restrict__ p,
                                double* __restrict__ q, double* __restrict__ part) {
  const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  double pq = 0.0;
  if (row < n) {
    const double* t = T + row * n;
    double s = 0.0;
    for (int64_t j = lane; j < n; j += 32) s = fma(t[j], p[j], s);
    s = warp_sum(s);
    if (lane == 0) {
      q[row] = s;
      pq = p[row] * s;
    }
  }
  block_partial(pq, part);
}

// block partials of a . b (b FP64 or FP32), fixed grid
template <typename TB>
__global__ void dot_kernel(const double* __restrict__ a, const TB* __restrict__ b, int64_t n, double* __restrict__ part) {
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s = fma(a[i], (double)b[i], s);
  block_partial(s, part);
}

// sum of the partials in a fixed order, then one scalar step of the iteration:
// 0 rz = s; 1 alpha = rz / s; 2 rr = s; 3 beta = s / rz, rz = s; 4 bb = s
__global__ void reduce_step_kernel(const double* __restrict__ part, int np, double* __restrict__ scal, int mode) {
  double s = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) s += part[i];
  __shared__ double sh[32];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
    if (mode == 0) scal[kScalRZ] = t;
    if (mode == 1) scal[kScalAlpha] = scal[kScalRZ] / t;
    if (mode == 2) scal[kScalRR] = t;
    if (mode == 3) {
      scal[kScalBeta] = t / scal[kScalRZ];
      scal[kScalRZ] = t;
    }
    if (mode == 4) scal[kScalBB] = t;
  }
}

// y += alpha p, r -= alpha q, r32 = r (the preconditioner's right-hand side); partials of r . r
__global__ void cg_update_kernel(double* __restrict__ y, double* __restrict__ r, const double* __restrict__ p,
                                 const double* __restrict__ q, float* __restrict__ r32, int64_t n,
                                 const double* __restrict__ scal, double* __restrict__ part) {
  const double alpha = scal[kScalAlpha];
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    y[i] = fma(alpha, p[i], y[i]);
    const double v = fma(-alpha, q[i], r[i]);
    r[i] = v;
    r32[i] = (float)v;
    s = fma(v, v, s);
  }
  block_partial(s, part);
}

// p = z + beta p (beta = 0: p = z)
__global__ void cg_direction_kernel(double* __restrict__ p, const float* __restrict__ z, int64_t n,
                                    const double* __restrict__ scal, int first) {
  const double beta = first ? 0.0 : scal[kScalBeta];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = first ? (double)z[i] : fma(beta, p[i], (double)z[i]);
}

__global__ void cg_init_kernel(double* __restrict__ y, double* __restrict__ r, float* __restrict__ r32,
                               const double* __restrict__ b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    y[i] = 0.0;
    r[i] = b[i];
    r32[i] = (float)b[i];
  }
}

// r = b - T y (FP64, T symmetric row-major n x n), warp per row; ||r||^2 and ||b||^2 into acc[0..1]
__global__ void residual_kernel(const double* __restrict__ T, int64_t n, const double* __restrict__ y,
                                const double* __restrict__ b, double* __restrict__ r, double* __restrict__ acc) {
  const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const double* t = T + row * n;
  double s = 0.0;
  for (int64_t j = lane; j < n; j += 32) s = fma(t[j], y[j], s);
  s = warp_sum(s);
  if (lane == 0) {
    const double v = b[row] - s;
    r[row] = v;
    atomicAdd(&acc[0], v * v);
    atomicAdd(&acc[1], b[row] * b[row]);
  }
}

__global__ void set_int_kernel(int* __restrict__ dst, int v) { *dst = v; }

// a failed factorisation (info > 0) makes the solution NaN, as the reference's Cholesky solve
// does, so the update is skipped instead of taking a step from a partial factor
__global__ void nan_if_failed_kernel(double* __restrict__ y, int64_t n, const int* __restrict__ info) {
  if (*info <= 0) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = __longlong_as_double(0x7FF8000000000000LL);
}

// info = the factorisation's info if it failed, else -1 when the final relative residual
// exceeds the tolerance, else 0
__global__ void refine_check_kernel(const double* __restrict__ acc, const int* __restrict__ fact_info,
                                    int* __restrict__ info, double tol) {
  int v = *fact_info;
  if (v == 0 && acc[1] > 0.0 && !(acc[0] <= tol * tol * acc[1])) v = -1;
  *info = v;
}

struct SolveWs {
  void* cus;
  size_t cus_bytes;
  double* y;      // n
  double* w;      // n  eigenvalues
  double* inv;    // n
  double* v;      // n
  double* f;      // n  right-hand side of the SR branch (A^T b)
  double* part;   // nchunk * max(n, np)
  double* shift;  // 2: shift, trace
  int* info;      // 2
  float* t32;     // n * n (SHIFT_MIXED)
  float* r32;     // n
  double* r;      // n
  double* acc;    // 16: iteration scalars and residual norms
  void* trsv;     // SHIFT_MIXED / SHIFT: the triangular solves' diagonal-block inverses and flags
  void* chol;     // SHIFT: the factorisation's digit slices and row exponents
};

// The FP32 factorisation of SHIFT_MIXED runs with cuSOLVER's BF16x9 emulation of FP32
// arithmetic on the tensor cores (measured on GB300 at n = 32768: 125 ms against 210 ms, the
// same |L L^T - T| on sampled entries); the FP64 iteration and its residual check follow
// unchanged. The mode is set around the FP32 calls only and the default restored after, so
// the FP64 paths that share the handle are unaffected.
struct Fp32EmulationScope {
  cusolverDnHandle_t h;
  bool on;
  Fp32EmulationScope(cusolverDnHandle_t handle, bool enable) : h(handle), on(enable) {
    if (on) cusolverDnSetMathMode(h, CUSOLVER_FP32_EMULATED_BF16X9_MATH);
  }
  ~Fp32EmulationScope() {
    if (on) cusolverDnSetMathMode(h, CUSOLVER_DEFAULT_MATH);
  }
};

int query_cusolver_bytes(int64_t n, int method, size_t* dev_bytes, size_t* host_bytes) {
  cusolverDnHandle_t h;
  cusolverDnParams_t p;
  int rc = solver_for_current_device(&h, &p);
  if (rc != QGX_OK) return rc;
  cusolverStatus_t s;
  if (method == QGX_SOLVE_SHIFT) {
    *dev_bytes = 0;
    *host_bytes = 0;
    return QGX_OK;
  }
  if (method == QGX_SOLVE_SHIFT_LIB) {
    s = cusolverDnXpotrf_bufferSize(h, p, CUBLAS_FILL_MODE_LOWER, n, CUDA_R_64F, nullptr, n, CUDA_R_64F, dev_bytes,
                                    host_bytes);
  } else if (method == QGX_SOLVE_SHIFT_MIXED) {
    Fp32EmulationScope emu(h, true);
    s = cusolverDnXpotrf_bufferSize(h, p, CUBLAS_FILL_MODE_LOWER, n, CUDA_R_32F, nullptr, n, CUDA_R_32F, dev_bytes,
                                    host_bytes);
  } else {
    s = cusolverDnXsyevd_bufferSize(h, p, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, CUDA_R_64F, nullptr, n,
                                    CUDA_R_64F, nullptr, CUDA_R_64F, dev_bytes, host_bytes);
  }
  return s == CUSOLVER_STATUS_SUCCESS ? QGX_OK : QGX_ERR_SOLVER;
}

int workspace_layout(int64_t n, int64_t np, int method, void* base, int64_t bytes, SolveWs* ws, int64_t* need) {
  size_t cb = 0, hb = 0;
  int rc = query_cusolver_bytes(n, method, &cb, &hb);
  if (rc != QGX_OK) return rc;
  const int64_t nchunk = (std::max(n, np) + kProjRows - 1) / kProjRows;
  const int64_t wide = std::max(n, np);
  int64_t off = 0;
  auto take = [&](int64_t b) {
    const int64_t o = off;
    off += al256(b);
    return o;
  };
  const int64_t o_cus = take((int64_t)cb);
  const int64_t o_y = take(n * 8);
  const int64_t o_w = take(n * 8);
  const int64_t o_inv = take(n * 8);
  const int64_t o_v = take(n * 8);
  const int64_t o_f = take(n * 8);
  // PINV on the SR branch with noise truncation: per 64-row chunk (mean, M2) of every column
  const int64_t snr_part = method == QGX_SOLVE_PINV
                               ? (std::max(n, np) + kSnrRows - 1) / kSnrRows * std::min(n, np) * 16
                               : 0;
  const int64_t o_part = take(std::max(nchunk * wide * 8, snr_part));
  const int64_t o_shift = take(16);
  const int64_t o_info = take(8);
  const bool mixed = method == QGX_SOLVE_SHIFT_MIXED;
  const int64_t o_t32 = take(mixed ? n * n * 4 : 0);
  const int64_t o_r32 = take(mixed ? n * 4 : 0);
  const int64_t o_r = take(mixed ? n * 8 : 0);
  const int64_t o_acc = take(mixed ? 16 * 8 : 0);
  const int64_t o_trsv = take(mixed ? trsv_chol_workspace_bytes(n)
                                    : (method == QGX_SOLVE_SHIFT ? trsv64_rowmajor_workspace_bytes(n) : 0));
  const int64_t o_chol = take(method == QGX_SOLVE_SHIFT ? chol_f64_workspace_bytes(n) : 0);
  *need = off;
  if (!base) return QGX_OK;
  if (bytes < off) return QGX_ERR_ARG;
  char* b = static_cast<char*>(base);
  ws->cus = b + o_cus;
  ws->cus_bytes = cb;
  ws->y = reinterpret_cast<double*>(b + o_y);
  ws->w = reinterpret_cast<double*>(b + o_w);
  ws->inv = reinterpret_cast<double*>(b + o_inv);
  ws->v = reinterpret_cast<double*>(b + o_v);
  ws->f = reinterpret_cast<double*>(b + o_f);
  ws->part = reinterpret_cast<double*>(b + o_part);
  ws->shift = reinterpret_cast<double*>(b + o_shift);
  ws->info = reinterpret_cast<int*>(b + o_info);
  ws->t32 = reinterpret_cast<float*>(b + o_t32);
  ws->r32 = reinterpret_cast<float*>(b + o_r32);
  ws->r = reinterpret_cast<double*>(b + o_r);
  ws->acc = reinterpret_cast<double*>(b + o_acc);
  ws->trsv = b + o_trsv;
  ws->chol = b + o_chol;
  if (hb > g_host_ws.size()) g_host_ws.resize(hb);
  return QGX_OK;
}

thread_local int64_t g_kernels = 0;  // qgx kernels launched by the current solve call

// x (ncol) = A^T y for A (nrow x ncol, lda)
int project(const float* A, int64_t nrow, int64_t ncol, int64_t lda, const double* y, double* part, double* x,
            cudaStream_t st) {
  const int64_t nchunk = (nrow + kProjRows - 1) / kProjRows;
  if (nchunk > 65535) return QGX_ERR_UNSUPPORTED;
  const bool vec4 = ((reinterpret_cast<uintptr_t>(A) & 15) == 0) && (lda % 4 == 0);
  ++g_kernels;
  project_partial_kernel<<<dim3((unsigned)((ncol + 1023) / 1024), (unsigned)nchunk), 256, 0, st>>>(
      A, nrow, ncol, lda, y, part, vec4);
  ++g_kernels;
  sum_partials_kernel<<<(unsigned)((ncol + 255) / 256), 256, 0, st>>>(part, nchunk, ncol, x);
  return launch_status();
}

// y = T^-1 b (SHIFT) or U diag(inv) rho (PINV), T n x n (overwritten)
int solve_gram(double* T, int64_t n, const double* b, int method, double rshift, double ashift, double rtol, double atol,
               double tol_snr, const SolveWs& ws, int32_t* info, cudaStream_t st) {
  cusolverDnHandle_t h;
  cusolverDnParams_t p;
  int rc = solver_for_stream(st, &h, &p);
  if (rc != QGX_OK) return rc;
  int* dinfo = info ? info : ws.info;
  void* hws = g_host_ws.empty() ? nullptr : g_host_ws.data();
  if (method == QGX_SOLVE_SHIFT || method == QGX_SOLVE_SHIFT_LIB) {
    ++g_kernels;
    shift_diag_kernel<<<1, 1024, 0, st>>>(T, n, n, rshift, ashift, ws.shift);
    if ((rc = launch_status()) != QGX_OK) return rc;
    cublasFillMode_t fill = CUBLAS_FILL_MODE_LOWER;
    if (method == QGX_SOLVE_SHIFT) {
      // this library's factorisation: L in the row-major lower triangle = the column-major
      // upper factor cuSOLVER's potrs takes
      if ((rc = chol_f64_graph(T, n, n, dinfo, nullptr, ws.chol, st, &g_kernels)) != QGX_OK) return rc;
      fill = CUBLAS_FILL_MODE_UPPER;
    } else if ((rc = cus_status([&] {
                  return cusolverDnXpotrf(h, p, CUBLAS_FILL_MODE_LOWER, n, CUDA_R_64F, T, n, CUDA_R_64F, ws.cus,
                                          ws.cus_bytes, hws, g_host_ws.size(), dinfo);
                })) != QGX_OK) {
      return rc;
    }
    QGX_CHECK_CUDA(cudaMemcpyAsync(ws.y, b, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    if (method == QGX_SOLVE_SHIFT) {
      // this library's decoupled block substitution on the row-major factor (trsv.cu), where
      // Xpotrs's FP64 substitution took 3.4 ms at n = 8192
      g_kernels += 4;
      if ((rc = trsv64_rowmajor_solve(T, n, ws.y, ws.trsv, st)) != QGX_OK) return rc;
    } else if ((rc = cus_status([&] {
                  // Xpotrs reports only argument errors; it writes its own word so that the
                  // factorisation's info (> 0: leading minor not positive definite) reaches the caller
                  return cusolverDnXpotrs(h, p, fill, n, 1, CUDA_R_64F, T, n, CUDA_R_64F, ws.y, n, ws.info + 1);
                })) != QGX_OK) {
      return rc;
    }
    ++g_kernels;
    nan_if_failed_kernel<<<(unsigned)std::min<int64_t>((n + 255) / 256, 1024), 256, 0, st>>>(ws.y, n, dinfo);
    return launch_status();
  }
  if (method == QGX_SOLVE_SHIFT_MIXED) {
    // host-synchronous: the factorisation's outcome and the convergence are read on the host
    ++g_kernels;
    shift_diag_kernel<<<1, 1024, 0, st>>>(T, n, n, rshift, ashift, ws.shift);
    const unsigned g = (unsigned)std::min<int64_t>((n * n + 255) / 256, 8192);
    double* extra = ws.acc + 8;
    int hinfo = 0;
    for (int attempt = 0; attempt < 2; ++attempt) {
      if (attempt == 1) {
        ++g_kernels;
        precond_shift_kernel<<<1, 1, 0, st>>>(ws.shift, n, extra);
      }
      ++g_kernels;
      to_f32_kernel<<<g, 256, 0, st>>>(T, n, ws.t32, attempt == 1 ? extra : nullptr);
      if ((rc = launch_status()) != QGX_OK) return rc;
      {
        Fp32EmulationScope emu(h, true);
        if ((rc = cus_status([&] {
               return cusolverDnXpotrf(h, p, CUBLAS_FILL_MODE_LOWER, n, CUDA_R_32F, ws.t32, n, CUDA_R_32F, ws.cus,
                                       ws.cus_bytes, hws, g_host_ws.size(), ws.info);
             })) != QGX_OK)
          return rc;
      }
      QGX_CHECK_CUDA(cudaMemcpyAsync(&hinfo, ws.info, sizeof(int), cudaMemcpyDeviceToHost, st));
      QGX_CHECK_CUDA(cudaStreamSynchronize(st));
      if (hinfo == 0) break;
    }
    if (hinfo != 0) {  // even the more shifted FP32 factor broke down
      ++g_kernels;
      set_int_kernel<<<1, 1, 0, st>>>(dinfo, hinfo);
      ++g_kernels;
      nan_if_failed_kernel<<<(unsigned)std::min<int64_t>((n + 255) / 256, 1024), 256, 0, st>>>(ws.y, n, dinfo);
      return launch_status();
    }
    double* scal = ws.acc;
    double* pv = ws.w;   // search direction
    double* qv = ws.inv; // T p
    const unsigned gr = (unsigned)((n * 32 + 255) / 256);
    const unsigned gd = (unsigned)std::min<int64_t>((n + 255) / 256, kDotBlocks);
    // r32 <- M^-1 r32 = L^-T L^-1 r32 with the decoupled block triangular solves (trsv.cu)
    ++g_kernels;
    if ((rc = trsv_chol_prepare(ws.t32, n, ws.trsv, st)) != QGX_OK) return rc;
    uint32_t epoch = 0;
    auto precondition = [&]() -> int {
      g_kernels += 2;
      return trsv_chol_apply(ws.t32, n, ws.r32, ws.trsv, ++epoch, st);
    };
    ++g_kernels;
    cg_init_kernel<<<gd, 256, 0, st>>>(ws.y, ws.r, ws.r32, b, n);
    ++g_kernels;
    dot_kernel<double><<<gd, 256, 0, st>>>(b, b, n, ws.part);
    ++g_kernels;
    reduce_step_kernel<<<1, 256, 0, st>>>(ws.part, (int)gd, scal, 4);
    if ((rc = precondition()) != QGX_OK) return rc;
    ++g_kernels;
    cg_direction_kernel<<<gd, 256, 0, st>>>(pv, ws.r32, n, scal, 1);
    ++g_kernels;
    dot_kernel<float><<<gd, 256, 0, st>>>(ws.r, ws.r32, n, ws.part);
    ++g_kernels;
    reduce_step_kernel<<<1, 256, 0, st>>>(ws.part, (int)gd, scal, 0);
    if ((rc = launch_status()) != QGX_OK) return rc;
    double host[2];
    int trsv_err = 0;
    for (int it = 0; it < kCgMaxIters; ++it) {
      ++g_kernels;
      symv_dot_kernel<<<gr, 256, 0, st>>>(T, n, pv, qv, ws.part);
      ++g_kernels;
      reduce_step_kernel<<<1, 256, 0, st>>>(ws.part, (int)gr, scal, 1);
      ++g_kernels;
      cg_update_kernel<<<gd, 256, 0, st>>>(ws.y, ws.r, pv, qv, ws.r32, n, scal, ws.part);
      ++g_kernels;
      reduce_step_kernel<<<1, 256, 0, st>>>(ws.part, (int)gd, scal, 2);
      QGX_CHECK_CUDA(cudaMemcpyAsync(host, scal + kScalRR, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
      if ((rc = trsv_chol_error(n, ws.trsv, &trsv_err, st)) != QGX_OK) return rc;
      QGX_CHECK_CUDA(cudaStreamSynchronize(st));
      if (trsv_err) break;  // a triangular solve timed out: the residual check below fails
      if (!(host[0] > kCgTol * kCgTol * host[1])) break;  // converged (or NaN: caught by the check below)
      if ((rc = precondition()) != QGX_OK) return rc;
      ++g_kernels;
      dot_kernel<float><<<gd, 256, 0, st>>>(ws.r, ws.r32, n, ws.part);
      ++g_kernels;
      reduce_step_kernel<<<1, 256, 0, st>>>(ws.part, (int)gd, scal, 3);
      ++g_kernels;
      cg_direction_kernel<<<gd, 256, 0, st>>>(pv, ws.r32, n, scal, 0);
    }
    // the true residual of the result decides
    double* last = ws.acc + 10;
    QGX_CHECK_CUDA(cudaMemsetAsync(last, 0, 2 * sizeof(double), st));
    ++g_kernels;
    residual_kernel<<<gr, 256, 0, st>>>(T, n, ws.y, b, ws.r, last);
    ++g_kernels;
    refine_check_kernel<<<1, 1, 0, st>>>(last, ws.info, dinfo, kRefineTol);
    if (trsv_err) {  // a triangular solve timed out
      ++g_kernels;
      set_int_kernel<<<1, 1, 0, st>>>(dinfo, -1);
    }
    return launch_status();
  }
  if ((rc = cus_status([&] {
         return cusolverDnXsyevd(h, p, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, CUDA_R_64F, T, n,
                                 CUDA_R_64F, ws.w, CUDA_R_64F, ws.cus, ws.cus_bytes, hws, g_host_ws.size(), dinfo);
       })) != QGX_OK)
    return rc;
  ++g_kernels;
  eigs_inv_kernel<<<1, 1024, 0, st>>>(ws.w, n, rtol, atol, ws.inv);
  ++g_kernels;
  rho_kernel<<<(unsigned)((n * 32 + 255) / 256), 256, 0, st>>>(T, n, b, ws.inv, tol_snr, ws.v);
  const int64_t nchunk = (n + kProjRows - 1) / kProjRows;
  ++g_kernels;
  uv_partial_kernel<<<dim3((unsigned)((n + 255) / 256), (unsigned)nchunk), 256, 0, st>>>(T, n, ws.v, ws.part);
  ++g_kernels;
  sum_partials_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(ws.part, nchunk, n, ws.y);
  return launch_status();
}

}  // namespace
}  // namespace qgx

using namespace qgx;

extern "C" {

int qgx_solve_workspace_bytes(int64_t n, int64_t np, int32_t method, int64_t* bytes) {
  QGX_CHECK_ARG(n > 0 && np > 0 && bytes && method >= QGX_SOLVE_SHIFT && method <= QGX_SOLVE_SHIFT_LIB);
  std::lock_guard<std::mutex> lock(g_solver_mutex);
  SolveWs ws;
  return workspace_layout(n, np, method, nullptr, 0, &ws, bytes);
}

int64_t qgx_last_solve_kernels(void) { return g_kernels; }

int qgx_minsr_solve(double* T, int64_t n, const float* A, int64_t np, int64_t lda, const double* b, int32_t method,
                    double rshift, double ashift, double rtol, double atol, double tol_snr, double* x, int32_t* info,
                    void* workspace, int64_t workspace_bytes, qgx_stream_t stream) {
  QGX_CHECK_ARG(n > 0 && np > 0 && lda >= np && T && A && b && x && workspace);
  QGX_CHECK_ARG(method == QGX_SOLVE_SHIFT || method == QGX_SOLVE_PINV || method == QGX_SOLVE_SHIFT_MIXED ||
                method == QGX_SOLVE_SHIFT_LIB);
  QGX_CHECK_ARG((reinterpret_cast<uintptr_t>(workspace) & 255) == 0);
  std::lock_guard<std::mutex> lock(g_solver_mutex);
  g_kernels = 0;
  SolveWs ws;
  int64_t need = 0;
  int rc = workspace_layout(n, np, method, workspace, workspace_bytes, &ws, &need);
  if (rc != QGX_OK) return rc;
  cudaStream_t st = as_cuda(stream);
  if ((rc = solve_gram(T, n, b, method, rshift, ashift, rtol, atol, tol_snr, ws, info, st)) != QGX_OK) return rc;
  return project(A, n, np, lda, ws.y, ws.part, x, st);
}

int qgx_sr_solve(double* S, int64_t np, const float* A, int64_t n, int64_t lda, const double* b, int32_t method,
                 double rshift, double ashift, double rtol, double atol, double tol_snr, double* x, int32_t* info,
                 void* workspace, int64_t workspace_bytes, qgx_stream_t stream) {
  QGX_CHECK_ARG(n > 0 && np > 0 && lda >= np && S && A && b && x && workspace);
  QGX_CHECK_ARG(method == QGX_SOLVE_SHIFT || method == QGX_SOLVE_PINV || method == QGX_SOLVE_SHIFT_LIB);
  QGX_CHECK_ARG((reinterpret_cast<uintptr_t>(workspace) & 255) == 0);
  std::lock_guard<std::mutex> lock(g_solver_mutex);
  g_kernels = 0;
  SolveWs ws;
  int64_t need = 0;
  int rc = workspace_layout(np, n, method, workspace, workspace_bytes, &ws, &need);
  if (rc != QGX_OK) return rc;
  cudaStream_t st = as_cuda(stream);
  if (method == QGX_SOLVE_PINV && tol_snr > 1e-6) {
    // lstsq_pinv_eig with noise truncation: S = V diag(l) V^T, rho_k from the per-sample
    // terms b[s] (A V)[s, k], x = V diag(l+) rho
    cusolverDnHandle_t h;
    cusolverDnParams_t p;
    if ((rc = solver_for_stream(st, &h, &p)) != QGX_OK) return rc;
    void* hws = g_host_ws.empty() ? nullptr : g_host_ws.data();
    if ((rc = cus_status([&] {
           return cusolverDnXsyevd(h, p, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, np, CUDA_R_64F, S, np,
                                   CUDA_R_64F, ws.w, CUDA_R_64F, ws.cus, ws.cus_bytes, hws, g_host_ws.size(),
                                   info ? info : ws.info);
         })) != QGX_OK)
      return rc;
    ++g_kernels;
    eigs_inv_kernel<<<1, 1024, 0, st>>>(ws.w, np, rtol, atol, ws.inv);
    const int64_t nchunk = (n + kSnrRows - 1) / kSnrRows;
    if (nchunk > 65535) return QGX_ERR_UNSUPPORTED;
    ++g_kernels;
    snr_terms_kernel<<<dim3((unsigned)((np + kSnrRows - 1) / kSnrRows), (unsigned)nchunk), 256, 0, st>>>(
        A, n, np, lda, S, b, ws.part);
    ++g_kernels;
    snr_rho_kernel<<<(unsigned)((np + 255) / 256), 256, 0, st>>>(ws.part, nchunk, n, np, ws.inv, tol_snr, ws.v);
    const int64_t vchunk = (np + kProjRows - 1) / kProjRows;
    ++g_kernels;
    uv_partial_kernel<<<dim3((unsigned)((np + 255) / 256), (unsigned)vchunk), 256, 0, st>>>(S, np, ws.v, ws.part);
    ++g_kernels;
    sum_partials_kernel<<<(unsigned)((np + 255) / 256), 256, 0, st>>>(ws.part, vchunk, np, x);
    return launch_status();
  }
  // F = A^T b into ws.f, then S x = F
  if ((rc = project(A, n, np, lda, b, ws.part, ws.f, st)) != QGX_OK) return rc;
  if ((rc = solve_gram(S, np, ws.f, method, rshift, ashift, rtol, atol, 0.0, ws, info, st)) != QGX_OK) return rc;
  QGX_CHECK_CUDA(cudaMemcpyAsync(x, ws.y, np * sizeof(double), cudaMemcpyDeviceToDevice, st));
  return QGX_OK;
}

// F = A^T b with the solve's deterministic two-pass projection (TimeEvol.get_SF,
// quantax/optimizer/time_evol.py:63-68)
int qgx_obar_rmatvec_workspace_bytes(int64_t rows, int64_t cols, int64_t* bytes) {
  QGX_CHECK_ARG(rows >= 0 && cols >= 0 && bytes);
  *bytes = al256(std::max<int64_t>(1, (rows + kProjRows - 1) / kProjRows) * std::max<int64_t>(cols, 1) * 8);
  return QGX_OK;
}

int qgx_obar_rmatvec(const float* A, int64_t rows, int64_t cols, int64_t lda, const double* b, double* y,
                     void* workspace, int64_t workspace_bytes, qgx_stream_t stream) {
  QGX_CHECK_ARG(rows > 0 && cols > 0 && lda >= cols && A && b && y && workspace);
  int64_t need = 0;
  qgx_obar_rmatvec_workspace_bytes(rows, cols, &need);
  QGX_CHECK_ARG(workspace_bytes >= need);
  return project(A, rows, cols, lda, b, static_cast<double*>(workspace), y, as_cuda(stream));
}

// x = S^-1 f for a given symmetric S (n x n FP64, overwritten): pinvh_solve
// (quantax/optimizer/solver.py:104-111) or the shifted Cholesky solve
int qgx_sym_solve(double* S, int64_t n, const double* f, int32_t method, double rshift, double ashift, double rtol,
                  double atol, double* x, int32_t* info, void* workspace, int64_t workspace_bytes,
                  qgx_stream_t stream) {
  QGX_CHECK_ARG(n > 0 && S && f && x && workspace);
  QGX_CHECK_ARG(method == QGX_SOLVE_SHIFT || method == QGX_SOLVE_PINV || method == QGX_SOLVE_SHIFT_LIB);
  QGX_CHECK_ARG((reinterpret_cast<uintptr_t>(workspace) & 255) == 0);
  std::lock_guard<std::mutex> lock(g_solver_mutex);
  g_kernels = 0;
  SolveWs ws;
  int64_t need = 0;
  int rc = workspace_layout(n, 1, method, workspace, workspace_bytes, &ws, &need);
  if (rc != QGX_OK) return rc;
  cudaStream_t st = as_cuda(stream);
  if ((rc = solve_gram(S, n, f, method, rshift, ashift, rtol, atol, 0.0, ws, info, st)) != QGX_OK) return rc;
  QGX_CHECK_CUDA(cudaMemcpyAsync(x, ws.y, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
  return QGX_OK;
}

}  // extern "C"
