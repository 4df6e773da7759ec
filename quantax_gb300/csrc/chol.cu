// FP64 Cholesky factorisation A = L L^T for the diagonal-shifted MinSR / SR solves
// (quantax/optimizer/solver.py:50-62: jax.scipy.linalg.solve(T + shift, b, assume_a="pos")).
//
// A is n x n, symmetric, row-major with leading dimension lda. L overwrites the lower triangle
// (L[i][j] at A[i lda + j], i >= j); the strict upper triangle is not touched, so it still
// holds the matrix by symmetry. Read as column-major, the factor is the upper triangle
// U = L^T with A = U^T U.
//
// FP64 arithmetic runs at about two FMAs per clock per SM on GB300, so only the O(n^2 b) part
// of the work runs on the FP64 pipe: right-looking, 256-column panels, each factored as four
// 64-column blocks (potrf of the 64 x 64 diagonal block and the 64-wide triangular solve of
// every row below it, in FP64). Every update of the form C -= P P^T runs on the tensor cores
// as an exact integer product (the Ozaki scheme: Ozaki, Ogita, Oishi and Rump, "Error-free
// transformations of matrix multiplication by using fast routines of matrix multiplication and
// its applications", Numer. Algorithms 59, 2012):
//   * each row r of the panel P (K <= 256 columns) is scaled by 2^-e_r, e_r the exponent with
//     max_k |P_rk| < 2^e_r, and rounded to the integer F = round(P 2^(56 - e_r)), |F| <= 2^56;
//   * F is written as 8 balanced base-128 digits S_0 .. S_7 (|S_0| <= 128, S_t in [-64, 64)
//     for t >= 1), each exact in BF16; P_rk = 2^e_r sum_t S_t[r][k] 2^(-7(t+1)) up to 2^(e_r-57);
//   * for each level l = t + u <= 7 the tensor core accumulates I_l = sum_(t+u=l) S_t S_u^T
//     over K in FP32: every product is an integer below 2^14 in magnitude and every partial
//     sum an integer below 2^24 (at most 8 pairs, K <= 256), so the FP32 accumulation is exact;
//   * the epilogue forms V = sum_l I_l 2^(38 - 7 l) exactly in int64 (levels 6 and 7 rounded
//     to 2^-38), converts once to FP64 and subtracts 2^(e_i + e_j - 52) V from C_ij.
// The products with t + u >= 8 are dropped: with the digits' own truncation the update's error
// is a few 2^-56 K 2^(e_i + e_j), below FP64's own rounding of a K-term dot product.
//
// The tensor-core kernel: one CTA per 128 x 32 tile of C on or below the diagonal, two CTAs
// per SM (one CTA's epilogue overlaps the other's MMAs). Warp 4 loads the 8 digit slices of the
// tile's 128 A rows and 32 B rows, 32 K-elements per stage (3D TMA box, 64-byte swizzle, one
// stage); warp 5 issues, per 16-element K step, one tcgen05.mma per A slice t (M 128,
// N = 32 (8 - t), K 16, BF16 -> FP32) against the B slices 0 .. 7 - t side by side, so the
// eight 32-column level accumulators (256 TMEM columns) each collect their level's products;
// warps 0-3 read the levels back and fold them in int64 into a shared-memory tile of FP64
// deltas, and all six warps apply the update to C in coalesced rows. Every mbarrier wait is
// bounded (2 s); a wait that runs out records QGX_ERR_TIMEOUT, the CTA frees its TMEM and
// leaves C alone.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "qgx_common.cuh"
#include "qgx_tc.cuh"

namespace qgx {
namespace {

constexpr int kPanel = 256;                     // columns of one tensor-core trailing update
constexpr int kBlk = 64;                        // columns of one FP64 diagonal block
constexpr int kSlices = 8;                      // BF16 digits per element
constexpr int kFixBits = 56;                    // kSlices * 7 fraction bits of the sliced rows
constexpr int kOzM = 128, kOzN = 32, kOzKB = 32;  // tile rows, tile columns, K per stage
constexpr int kOzStages = 1;  // two CTAs per SM: one CTA's epilogue overlaps the other's MMAs
constexpr int kOzABytes = kSlices * kOzM * kOzKB * 2;  // 64 KB
constexpr int kOzBBytes = kSlices * kOzN * kOzKB * 2;  // 16 KB
constexpr int kOzStageBytes = kOzABytes + kOzBBytes;
constexpr int kOzThreads = 192;
constexpr size_t kOzSmem = 1024 + (size_t)kOzStages * kOzStageBytes + 256;
constexpr uint32_t kOzTmemCols = kSlices * kOzN;  // eight 32-column FP32 level accumulators
constexpr int kOzDLd = kOzN + 1;       // doubles per row of the epilogue's transpose tile

inline int64_t al256(int64_t b) { return (b + 255) / 256 * 256; }

// ---- digit slices ---------------------------------------------------------------------------
// Rows [0, m) of a K-column panel (row r at A + (row0 + r) lda + col0): exponent e_r and the
// 8 BF16 digit slices S[t][r][k] (slice-major, row stride K). One warp per row.
__global__ void slice_rows_kernel(const double* __restrict__ A, int64_t lda, int64_t row0, int64_t col0, int64_t m,
                                  int K, __nv_bfloat16* __restrict__ S, int* __restrict__ ex) {
  const int64_t r = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= m) return;  // whole warps
  const double* a = A + (row0 + r) * lda + col0;
  double mx = 0.0;
  for (int k = lane; k < K; k += 32) mx = fmax(mx, fabs(a[k]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  int e = 0;
  if (mx > 0.0) frexp(mx, &e);  // mx = f 2^e, f in [0.5, 1): every |a_k| < 2^e
  if (lane == 0) ex[r] = e;
  for (int k = lane; k < K; k += 32) {
    long long F = __double2ll_rn(ldexp(a[k], kFixBits - e));  // exact scaling, |F| <= 2^56
#pragma unroll
    for (int t = kSlices - 1; t >= 1; --t) {
      const long long d = ((F + 64) & 127) - 64;  // balanced digit in [-64, 64)
      S[((int64_t)t * m + r) * K + k] = __float2bfloat16_rn((float)d);
      F = (F - d) >> 7;                           // exact
    }
    S[(int64_t)r * K + k] = __float2bfloat16_rn((float)F);  // |S_0| <= 128
  }
}

// ---- FP64 diagonal block and triangular solve -----------------------------------------------
// Cholesky of the nb x nb (nb <= 64) diagonal block at (c, c), in place. The first pivot that is
// not positive sets *info = c + k + 1 (the order of the failing leading minor, as LAPACK and
// cuSOLVER report it); the factorisation carries on with a NaN pivot. 256 threads as a 16 x 16
// grid over the trailing block (no index division in the update loop); the pivot's inverse
// square root scales its column.
__global__ void __launch_bounds__(256) potrf_block_kernel(double* __restrict__ A, int64_t lda, int64_t c, int nb,
                                                          int* __restrict__ info) {
  __shared__ double a[kBlk][kBlk + 1];
  __shared__ double piv[2];  // sqrt and inverse sqrt of the current pivot
  const int ti = threadIdx.x >> 4, tj = threadIdx.x & 15;
  for (int i = ti; i < nb; i += 16)
    for (int j = tj; j <= i; j += 16) a[i][j] = A[(c + i) * lda + c + j];
  __syncthreads();
  for (int k = 0; k < nb; ++k) {
    if (threadIdx.x == 0) {
      double d = a[k][k];
      if (!(d > 0.0)) {
        atomicCAS(info, 0, (int)(c + k + 1));
        d = __longlong_as_double(0x7FF8000000000000LL);
      }
      const double r = rsqrt(d);
      piv[0] = d * r;  // sqrt(d)
      piv[1] = r;
    }
    __syncthreads();
    const double r = piv[1];
    if (threadIdx.x == 0) a[k][k] = piv[0];
    for (int i = k + 1 + threadIdx.x; i < nb; i += blockDim.x) a[i][k] *= r;
    __syncthreads();
    for (int i = k + 1 + ti; i < nb; i += 16) {
      const double aik = a[i][k];
      for (int j = k + 1 + tj; j <= i; j += 16) a[i][j] = fma(-aik, a[j][k], a[i][j]);
    }
    __syncthreads();
  }
  for (int i = ti; i < nb; i += 16)
    for (int j = tj; j <= i; j += 16) A[(c + i) * lda + c + j] = a[i][j];
}

// rows [r0, n) of the 64 columns at c: x L_cc^T = a with L_cc the factored diagonal block, in
// place (reference BLAS dtrsm 'R','L','T','N' order: scale by the pivot's reciprocal, then
// update the later columns). Eight lanes per row, lane l holding columns l, l + 8, ..., l + 56:
// at step k the owner of column k scales it and an 8-lane shuffle hands it to the others, which
// update their later columns. 16 rows per 128-thread CTA, so even a short panel's rows spread
// over every SM (the SMs' FP64 pipes bound the work).
constexpr int kTrsmThreads = 128;
constexpr int kTrsmRows = kTrsmThreads / 8;
__global__ void __launch_bounds__(kTrsmThreads) trsm_block_kernel(double* __restrict__ A, int64_t lda, int64_t c,
                                                                  int64_t r0, int64_t n) {
  __shared__ double l[kBlk][kBlk + 1];
  __shared__ double dinv[kBlk];
  for (int e = threadIdx.x; e < kBlk * kBlk; e += blockDim.x) {
    const int i = e / kBlk, j = e % kBlk;
    l[i][j] = j <= i ? A[(c + i) * lda + c + j] : 0.0;
  }
  for (int i = threadIdx.x; i < kBlk; i += blockDim.x) dinv[i] = 1.0 / A[(c + i) * lda + c + i];
  __syncthreads();
  const int sub = threadIdx.x & 7;  // lane within the row's group of eight
  const int64_t r = r0 + (int64_t)blockIdx.x * kTrsmRows + (threadIdx.x >> 3);
  const bool live = r < n;  // whole 8-lane groups share a row; dead groups keep shuffling zeros
  double* row = A + (live ? r : r0) * lda + c;
  double x[kBlk / 8];
#pragma unroll
  for (int q = 0; q < kBlk / 8; ++q) x[q] = live ? row[8 * q + sub] : 0.0;
#pragma unroll
  for (int k = 0; k < kBlk; ++k) {
    const int qk = k >> 3;
    double xk = 0.0;
    if (sub == (k & 7)) {
      x[qk] *= dinv[k];
      xk = x[qk];
    }
    xk = __shfl_sync(0xffffffffu, xk, k & 7, 8);
#pragma unroll
    for (int q = 0; q < kBlk / 8; ++q)
      if (8 * q + sub > k) x[q] = fma(-xk, l[8 * q + sub][k], x[q]);
  }
  if (live) {
#pragma unroll
    for (int q = 0; q < kBlk / 8; ++q) row[8 * q + sub] = x[q];
  }
}

// ---- tensor-core update C -= P P^T (lower part) ----------------------------------------------
// K-major BF16 operand rows of 64 bytes, 64-byte swizzle: 8-row groups 512 bytes apart
__device__ inline uint64_t desc_sw64(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);  // start address
  d |= (uint64_t)1 << 16;                   // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(512 >> 4) << 32;          // stride byte offset: 8 rows x 64 bytes
  d |= (uint64_t)1 << 46;                   // descriptor version of tcgen05
  d |= (uint64_t)4 << 61;                   // 64-byte swizzle
  return d;
}

// BF16 x BF16 -> FP32, K-major A and B, M = 128, N = n (a multiple of 16, at most 256)
constexpr uint32_t oz_idesc(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kOzM >> 4) << 24);
}

__device__ inline void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ inline void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], "
      "[%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(z)
      : "memory");
}

// 16 columns of this warp's 32 TMEM lanes into registers, without waiting (tmem_wait_ld makes
// them usable): several loads can be in flight behind one wait
__device__ inline void tmem_ld_16cols_nowait(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

__device__ inline void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// level l's integer, scaled to 2^(38 - 7 l) (levels 6 and 7 rounded to the nearest 2^-38)
template <int L>
__device__ inline long long level_term(int v) {
  constexpr int s = 38 - 7 * L;
  if constexpr (s >= 0) {
    return (long long)v << s;
  } else {
    return ((long long)v + (1LL << (-s - 1))) >> (-s);
  }
}

// 2^x for any exponent an FP64 update can take
__device__ inline double pow2(int x) {
  if (x >= -1022 && x <= 1023) return __hiloint2double((x + 1023) << 20, 0);
  return ldexp(1.0, x);
}

// C[i][j] -= sum_k P[a0 + i][k] P[b0 + j][k] for the m x ncols region at C (ldc), where slice
// row r is the panel's row r; only entries with a0 + i >= b0 + j (on or below the diagonal of the
// whole matrix) are updated
__global__ void __launch_bounds__(kOzThreads, 2)
    ozaki_syrk_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
                      const int* __restrict__ ex, int64_t m, int64_t ncols, int a0, int b0, int nkb,
                      double* __restrict__ C, int64_t ldc, int32_t* __restrict__ status) {
  const int64_t row0 = (int64_t)blockIdx.x * kOzM, col0 = (int64_t)blockIdx.y * kOzN;
  if (a0 + row0 + kOzM - 1 < b0 + col0) return;  // the tile lies above the diagonal: nothing to update
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + kOzStages * kOzStageBytes);
  uint64_t* empty = full + kOzStages;
  uint64_t* acc_full = empty + kOzStages;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(acc_full + 1);
  volatile int* fail = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kOzStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(acc_full, 1);
    *fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kOzTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  int issued = 0;  // producer: stage loads issued
  if (warp == 4) {
    if (lane == 0) {
      for (int kb = 0; kb < nkb && !*fail; ++kb, ++issued) {
        const int s = kb % kOzStages;
        const uint32_t ph = (uint32_t)((kb / kOzStages) & 1);
        if (!mbar_wait(&empty[s], ph ^ 1u)) {
          *fail = 1;
          break;
        }
        uint8_t* a = smem + s * kOzStageBytes;
        mbar_expect_tx(&full[s], kOzStageBytes);
        tma_load_3d(a, &map_a, &full[s], kb * kOzKB, a0 + (int)row0, 0);
        tma_load_3d(a + kOzABytes, &map_b, &full[s], kb * kOzKB, b0 + (int)col0, 0);
      }
    }
  } else if (warp == 5) {
    if (lane == 0) {
      for (int kb = 0; kb < nkb && !*fail; ++kb) {
        const int s = kb % kOzStages;
        const uint32_t ph = (uint32_t)((kb / kOzStages) & 1);
        if (!mbar_wait(&full[s], ph)) {
          *fail = 1;
          break;
        }
        tc_fence_after();
        const uint32_t base = smem_u32(smem + s * kOzStageBytes);
#pragma unroll 1
        for (int kk = 0; kk < kOzKB / 16; ++kk) {  // 32 bytes of K per instruction
          // one MMA per A slice t: B is the slices u = 0 .. 7 - t of the column rows, contiguous
          // in shared memory (slice u at rows kOzN u ..), so D's column block u is S_t S_u^T and
          // lands in the accumulator of level t + u (columns kOzN (t + u) ..): levels t .. 7
          // are one contiguous N = kOzN (8 - t) range. Every level sum stays an integer below
          // 2^24, so the FP32 accumulation is exact in any order.
          const uint64_t db = desc_sw64(base + kOzABytes + kk * 32);
#pragma unroll
          for (int t = 0; t < kSlices; ++t) {
            const uint64_t da = desc_sw64(base + t * (kOzM * kOzKB * 2) + kk * 32);
            mma_bf16(tmem + (uint32_t)(kOzN * t), da, db, oz_idesc(kOzN * (kSlices - t)),
                     (kb == 0 && kk == 0 && t == 0) ? 0u : 1u);
          }
        }
        mma_commit(&empty[s]);
      }
      mma_commit(acc_full);  // also after a failed wait: tracks every MMA issued so far
    }
  }

  // epilogue warps 0..3: fold the eight levels of each row (TMEM lane) into FP64 deltas
  double* dt = reinterpret_cast<double*>(smem);  // 128 x 65 doubles over the (finished) stages
  const int q = warp & 3;
  if (warp < 4) {
    // while the MMAs run: pull this tile's rows of C into L2 for the read-modify-write below
    for (int rr = q; rr < kOzM; rr += 4) {
      const int64_t i = row0 + rr;
      if (i >= m) break;
      // lanes 0-3: the cache lines holding columns 16 lane .. of the row (every address lies in C)
      if (lane < kOzN / 16 && col0 + 16 * lane < ncols)
        asm volatile("prefetch.global.L2 [%0];" ::"l"(C + i * ldc + col0 + 16 * lane));
    }
    if (!mbar_wait(acc_full, 0)) *fail = 1;
    if (!*fail) {
      tc_fence_after();
      const int rl = 32 * q + lane;
      const uint32_t lane_addr = tmem + ((uint32_t)(32 * q) << 16);
#pragma unroll 1
      for (int g = 0; g < kOzN / 16; ++g) {
        long long v[16];
        // four levels in flight behind one wait, twice
#pragma unroll
        for (int half = 0; half < 2; ++half) {
          uint32_t r[4][16];
#pragma unroll
          for (int l4 = 0; l4 < 4; ++l4)
            tmem_ld_16cols_nowait(lane_addr + (uint32_t)(kOzN * (4 * half + l4) + 16 * g), r[l4]);
          tmem_wait_ld();
#define QGX_OZ_LEVEL(L)                                                                   \
  _Pragma("unroll") for (int j = 0; j < 16; ++j) {                                        \
    const long long tv = level_term<L>(__float2int_rn(__uint_as_float(r[(L) & 3][j])));  \
    v[j] = (L) == 0 ? tv : v[j] + tv;                                                     \
  }
          if (half == 0) {
            QGX_OZ_LEVEL(0)
            QGX_OZ_LEVEL(1)
            QGX_OZ_LEVEL(2)
            QGX_OZ_LEVEL(3)
          } else {
            QGX_OZ_LEVEL(4)
            QGX_OZ_LEVEL(5)
            QGX_OZ_LEVEL(6)
            QGX_OZ_LEVEL(7)
          }
#undef QGX_OZ_LEVEL
        }
#pragma unroll
        for (int j = 0; j < 16; ++j) dt[rl * kOzDLd + 16 * g + j] = (double)v[j];
      }
    }
  }
  tc_fence_before();
  __syncthreads();  // deltas complete; every role has left its loop
  if (*fail) {
    if (threadIdx.x == 0 && status) atomicExch(status, QGX_ERR_TIMEOUT);
  } else {
    // C[i][j] -= 2^(e_i + e_j - 52) V_ij on or below the diagonal, by all six warps (the
    // producer and MMA warps are idle by now): warp w takes rows w, w + 6, ..., eight rows at a
    // time with all their loads of C issued before the first update, so the loads' latencies
    // overlap (lane l holds column l of each row)
    constexpr int kBatch = 8, kRmwWarps = kOzThreads / 32;
    int ej[kOzN / 32];
    bool jin[kOzN / 32];
#pragma unroll
    for (int h = 0; h < kOzN / 32; ++h) {
      const int64_t j = col0 + 32 * h + lane;
      jin[h] = j < ncols;
      ej[h] = jin[h] ? ex[b0 + j] : 0;
    }
#pragma unroll 1
    for (int rb = warp; rb < kOzM; rb += kRmwWarps * kBatch) {
      double cv[kBatch][kOzN / 32];
      bool ok[kBatch][kOzN / 32];
#pragma unroll
      for (int r = 0; r < kBatch; ++r) {
        const int rr = rb + kRmwWarps * r;  // a row of this tile (rr < kOzM) and of the matrix
        const int64_t i = row0 + rr;
#pragma unroll
        for (int h = 0; h < kOzN / 32; ++h) {
          const int64_t j = col0 + 32 * h + lane;
          ok[r][h] = rr < kOzM && i < m && jin[h] && b0 + j <= a0 + i;
          cv[r][h] = ok[r][h] ? C[i * ldc + j] : 0.0;
        }
      }
#pragma unroll
      for (int r = 0; r < kBatch; ++r) {
        const int rr = rb + kRmwWarps * r;
        const int64_t i = row0 + rr;
        const int ei = rr < kOzM && i < m ? ex[a0 + i] : 0;
#pragma unroll
        for (int h = 0; h < kOzN / 32; ++h) {
          if (!ok[r][h]) continue;
          const int cl = 32 * h + lane;
          C[i * ldc + col0 + cl] = fma(-dt[rr * kOzDLd + cl], pow2(ei + ej[h] - 52), cv[r][h]);
        }
      }
    }
  }
  if (*fail && warp == 4 && lane == 0) {
    // no copy may land in shared memory after the CTA has left: wait (bounded) for the loads
    // of the last stages issued
    for (int kb = std::max(0, issued - kOzStages); kb < issued; ++kb)
      mbar_wait(&full[kb % kOzStages], (uint32_t)((kb / kOzStages) & 1));
  }
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kOzTmemCols) : "memory");
  }
}

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
  static std::once_flag once;
  static EncodeTiled fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiled>(p);
  });
  return fn;
}

// slices S[8][m][K] as a 3D tensor (K, m, 8); box 32 x box_rows x 8, 64-byte swizzle, rows past
// m read as zeros
int encode_slices(CUtensorMap* map, const __nv_bfloat16* S, int64_t m, int K, int box_rows) {
  EncodeTiled enc = encode_fn();
  if (!enc) return QGX_ERR_UNSUPPORTED;
  const cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)m, (cuuint64_t)kSlices};
  const cuuint64_t strides[2] = {(cuuint64_t)K * 2, (cuuint64_t)(m * K * 2)};
  const cuuint32_t box[3] = {(cuuint32_t)kOzKB, (cuuint32_t)box_rows, (cuuint32_t)kSlices};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult cr = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<__nv_bfloat16*>(S), dims, strides, box,
                          estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return cr == CUDA_SUCCESS ? QGX_OK : QGX_ERR_UNSUPPORTED;
}

struct CholWs {
  __nv_bfloat16* s_panel[2];  // 8 x n x 256 digits of a trailing panel (two panels in flight)
  __nv_bfloat16* s_block;     // 8 x n x 64 digits of a diagonal block's column strip
  int* e_panel[2];            // n row exponents each
  int* e_block;               // n row exponents
};

int64_t chol_layout(int64_t n, void* base, CholWs* ws) {
  int64_t off = 0;
  auto take = [&](int64_t b) {
    const int64_t o = off;
    off += al256(b);
    return o;
  };
  const int64_t o_sp0 = take(kSlices * n * kPanel * 2), o_sp1 = take(kSlices * n * kPanel * 2);
  const int64_t o_sb = take(kSlices * n * kBlk * 2);
  const int64_t o_ep0 = take(n * 4), o_ep1 = take(n * 4), o_eb = take(n * 4);
  if (base && ws) {
    char* b = static_cast<char*>(base);
    ws->s_panel[0] = reinterpret_cast<__nv_bfloat16*>(b + o_sp0);
    ws->s_panel[1] = reinterpret_cast<__nv_bfloat16*>(b + o_sp1);
    ws->s_block = reinterpret_cast<__nv_bfloat16*>(b + o_sb);
    ws->e_panel[0] = reinterpret_cast<int*>(b + o_ep0);
    ws->e_panel[1] = reinterpret_cast<int*>(b + o_ep1);
    ws->e_block = reinterpret_cast<int*>(b + o_eb);
  }
  return off;
}

// digit slices of the K-column panel at A[row0 .., col0 ..] (m rows)
int slice_panel(const double* A, int64_t lda, int64_t row0, int64_t col0, int64_t m, int K, __nv_bfloat16* S,
                int* ex, cudaStream_t st, int64_t* kernels) {
  if (m <= 0) return QGX_OK;
  slice_rows_kernel<<<(unsigned)((m + 7) / 8), 256, 0, st>>>(A, lda, row0, col0, m, K, S, ex);
  ++*kernels;
  return launch_status();
}

// C -= P P^T over the region of rows [r0, r0 + m) x columns [q0, q0 + ncols) of A, P the panel
// sliced into S (ms rows, slice row r = matrix row s0 + r)
int ozaki_region(double* A, int64_t lda, const __nv_bfloat16* S, const int* ex, int64_t ms, int64_t s0, int K,
                 int64_t r0, int64_t m, int64_t q0, int64_t ncols, int32_t* status, cudaStream_t st,
                 int64_t* kernels) {
  if (m <= 0 || ncols <= 0) return QGX_OK;
  if (ms > 0x7fffffffLL || (m + kOzM - 1) / kOzM > 0x7fffffffLL || (ncols + kOzN - 1) / kOzN > 65535)
    return QGX_ERR_UNSUPPORTED;
  CUtensorMap ma, mb;
  int rc = encode_slices(&ma, S, ms, K, kOzM);
  if (rc == QGX_OK) rc = encode_slices(&mb, S, ms, K, kOzN);
  if (rc != QGX_OK) return rc;
  QGX_CHECK_CUDA(cudaFuncSetAttribute(ozaki_syrk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kOzSmem));
  const dim3 grid((unsigned)((m + kOzM - 1) / kOzM), (unsigned)((ncols + kOzN - 1) / kOzN));
  ozaki_syrk_kernel<<<grid, kOzThreads, kOzSmem, st>>>(ma, mb, ex, m, ncols, (int)(r0 - s0), (int)(q0 - s0),
                                                      K / kOzKB, A + r0 * lda + q0, lda, status);
  ++*kernels;
  return launch_status();
}

// Per device: the look-ahead stream (highest priority) and the events that order it against the
// caller's stream. One factorisation at a time per device (the mutex is held while enqueueing).
struct LookAhead {
  std::mutex mu;
  cudaStream_t aux = nullptr;
  cudaEvent_t start = nullptr, end = nullptr, strip_done[2] = {}, rest_done[2] = {};
};
constexpr int kMaxCholDevices = 64;
LookAhead g_look[kMaxCholDevices];
std::mutex g_look_init;

int look_ahead_for_current_device(LookAhead** out) {
  int dev = 0;
  QGX_CHECK_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxCholDevices) return QGX_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_look_init);
  LookAhead& la = g_look[dev];
  if (!la.aux) {
    int lo = 0, hi = 0;
    QGX_CHECK_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    QGX_CHECK_CUDA(cudaStreamCreateWithPriority(&la.aux, cudaStreamNonBlocking, hi));
    cudaEvent_t* evs[6] = {&la.start, &la.end, &la.strip_done[0], &la.strip_done[1], &la.rest_done[0],
                           &la.rest_done[1]};
    for (cudaEvent_t* e : evs) QGX_CHECK_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  }
  *out = &la;
  return QGX_OK;
}

}  // namespace

int64_t chol_f64_workspace_bytes(int64_t n) { return n > 0 ? chol_layout(n, nullptr, nullptr) : 0; }

// A = L L^T in place (see the file comment). info: 0, or the order of the first leading minor
// that is not positive definite. status (may be NULL): QGX_ERR_TIMEOUT if a tensor-core wait ran
// out. Adds the number of kernels launched to *kernels.
//
// Look-ahead: panel k's trailing update is split into the next panel's 256 columns (the strip)
// and the rest. The panel chain (FP64 diagonal blocks, triangular solves, the in-panel updates),
// the panel's slicing and the strip run on a high-priority internal stream; the rest runs on the
// caller's stream, so the next panel's FP64 chain overlaps the large tensor-core update. Panel
// k's chain waits for the rest update of panel k - 2, and panel k's strip for the rest update of
// panel k - 1: every update of a column block is ordered after the previous one (the strip and
// the previous panel's rest both update the next panel's columns below its diagonal). Two slice
// buffers alternate between panels. The caller's stream waits for the internal one at the end,
// so the factor is complete in stream order.
int chol_f64(double* A, int64_t n, int64_t lda, int* info, int32_t* status, void* work, cudaStream_t st,
             int64_t* kernels) {
  if ((reinterpret_cast<uintptr_t>(work) & 255) != 0) return QGX_ERR_ARG;
  LookAhead* la = nullptr;
  int rc = look_ahead_for_current_device(&la);
  if (rc != QGX_OK) return rc;
  std::lock_guard<std::mutex> lock(la->mu);
  CholWs ws;
  chol_layout(n, work, &ws);
  cudaStream_t aux = la->aux;
  QGX_CHECK_CUDA(cudaMemsetAsync(info, 0, sizeof(int), st));
  if (status) QGX_CHECK_CUDA(cudaMemsetAsync(status, 0, sizeof(int32_t), st));
  QGX_CHECK_CUDA(cudaEventRecord(la->start, st));
  QGX_CHECK_CUDA(cudaStreamWaitEvent(aux, la->start, 0));
  int64_t k = 0;
  for (int64_t c0 = 0; c0 < n; c0 += kPanel, ++k) {
    const int64_t pe = std::min<int64_t>(c0 + kPanel, n);
    if (k >= 2) QGX_CHECK_CUDA(cudaStreamWaitEvent(aux, la->rest_done[k & 1], 0));
    // the panel chain
    for (int64_t cj = c0; cj < pe; cj += kBlk) {
      const int nb = (int)std::min<int64_t>(kBlk, n - cj);
      potrf_block_kernel<<<1, 256, 0, aux>>>(A, lda, cj, nb, info);
      ++*kernels;
      const int64_t rb = cj + kBlk;  // first row below the block
      if (rb >= n) break;
      trsm_block_kernel<<<(unsigned)((n - rb + kTrsmRows - 1) / kTrsmRows), kTrsmThreads, 0, aux>>>(A, lda, cj, rb,
                                                                                                      n);
      ++*kernels;
      if ((rc = launch_status()) != QGX_OK) return rc;
      if (rb < pe) {  // the block's columns update the rest of the panel (K = 64)
        if ((rc = slice_panel(A, lda, rb, cj, n - rb, kBlk, ws.s_block, ws.e_block, aux, kernels)) != QGX_OK ||
            (rc = ozaki_region(A, lda, ws.s_block, ws.e_block, n - rb, rb, kBlk, rb, n - rb, rb, pe - rb, status,
                               aux, kernels)) != QGX_OK)
          return rc;
      }
    }
    if (pe >= n) break;
    // the panel's trailing update (K = 256): the strip on the internal stream, the rest on st
    const int b = (int)(k & 1);
    const int64_t ms = n - pe, pe2 = std::min<int64_t>(pe + kPanel, n);
    if ((rc = slice_panel(A, lda, pe, c0, ms, kPanel, ws.s_panel[b], ws.e_panel[b], aux, kernels)) != QGX_OK)
      return rc;
    // the strip updates the next panel's columns, which the previous panel's rest update (on st)
    // also updates: both read-modify-write the same entries, so the strip waits for it
    if (k >= 1) QGX_CHECK_CUDA(cudaStreamWaitEvent(aux, la->rest_done[(k - 1) & 1], 0));
    if ((rc = ozaki_region(A, lda, ws.s_panel[b], ws.e_panel[b], ms, pe, kPanel, pe, ms, pe, pe2 - pe, status, aux,
                           kernels)) != QGX_OK)
      return rc;
    if (pe2 < n) {
      QGX_CHECK_CUDA(cudaEventRecord(la->strip_done[b], aux));
      QGX_CHECK_CUDA(cudaStreamWaitEvent(st, la->strip_done[b], 0));
      if ((rc = ozaki_region(A, lda, ws.s_panel[b], ws.e_panel[b], ms, pe, kPanel, pe2, n - pe2, pe2, n - pe2, status,
                             st, kernels)) != QGX_OK)
        return rc;
      QGX_CHECK_CUDA(cudaEventRecord(la->rest_done[b], st));
    }
  }
  QGX_CHECK_CUDA(cudaEventRecord(la->end, aux));
  QGX_CHECK_CUDA(cudaStreamWaitEvent(st, la->end, 0));
  return launch_status();
}

// ---- factorisation graphs ------------------------------------------------------------
// A factorisation is a long launch sequence (about 2000 kernels and event operations at
// n = 32768). Enqueued one by one it fills the device's queue of pending launches, after which
// every further launch waits for the GPU: the caller's thread is held for the whole
// factorisation, and callers on other streams (the jobs of a serving loop) cannot get their
// work queued meanwhile. The sequence is therefore captured once per set of buffers into a
// CUDA graph (on a private stream, relaxed capture mode; the look-ahead stream joins the capture
// through its events, which become edges of the graph) and replayed with one launch. Two
// replays share no stream or event, so factorisations on different streams can overlap.
namespace {

struct CholKey {
  double* A;
  int64_t n, lda;
  int* info;
  int32_t* status;
  void* work;
  int device;
  bool operator==(const CholKey& o) const {
    return A == o.A && n == o.n && lda == o.lda && info == o.info && status == o.status && work == o.work &&
           device == o.device;
  }
};

struct CholGraph {
  CholKey key;
  cudaGraphExec_t exec;
  int64_t kernels;
  uint64_t last_use;
};

constexpr int kMaxCholGraphs = 16;
std::mutex g_chol_graph_mutex;
std::vector<CholGraph> g_chol_graphs;
uint64_t g_chol_clock = 0;
cudaStream_t g_chol_capture[kMaxCholDevices] = {};

}  // namespace

int chol_f64_graph(double* A, int64_t n, int64_t lda, int* info, int32_t* status, void* work, cudaStream_t st,
                   int64_t* kernels) {
  int dev = 0;
  QGX_CHECK_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxCholDevices) return QGX_ERR_UNSUPPORTED;
  const CholKey key{A, n, lda, info, status, work, dev};
  std::lock_guard<std::mutex> lock(g_chol_graph_mutex);
  CholGraph* hit = nullptr;
  for (auto& e : g_chol_graphs)
    if (e.key == key) hit = &e;
  if (!hit) {
    if (!g_chol_capture[dev]) QGX_CHECK_CUDA(cudaStreamCreateWithFlags(&g_chol_capture[dev], cudaStreamNonBlocking));
    cudaStream_t cs = g_chol_capture[dev];
    QGX_CHECK_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed));
    int64_t count = 0;
    const int rc = chol_f64(A, n, lda, info, status, work, cs, &count);
    cudaGraph_t graph = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(cs, &graph);
    if (rc != QGX_OK) {
      if (graph) cudaGraphDestroy(graph);
      cudaGetLastError();
      return rc;
    }
    QGX_CHECK_CUDA(ce);
    cudaGraphExec_t exec = nullptr;
    // the look-ahead chain keeps the priority of the stream it was captured from
    const cudaError_t ie = cudaGraphInstantiateWithFlags(&exec, graph, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(graph);
    QGX_CHECK_CUDA(ie);
    if ((int)g_chol_graphs.size() >= kMaxCholGraphs) {  // evict the least recently used (an
      // executable graph still running is freed when it completes)
      auto lru = std::min_element(g_chol_graphs.begin(), g_chol_graphs.end(),
                                  [](const CholGraph& a, const CholGraph& b) { return a.last_use < b.last_use; });
      cudaGraphExecDestroy(lru->exec);
      g_chol_graphs.erase(lru);
    }
    g_chol_graphs.push_back(CholGraph{key, exec, count, 0});
    hit = &g_chol_graphs.back();
  }
  hit->last_use = ++g_chol_clock;
  QGX_CHECK_CUDA(cudaGraphLaunch(hit->exec, st));
  *kernels += hit->kernels;
  return QGX_OK;
}

}  // namespace qgx

using namespace qgx;

extern "C" {

int64_t qgx_cholesky_workspace_bytes(int64_t n) { return chol_f64_workspace_bytes(n); }

int qgx_cholesky(double* A, int64_t n, int64_t lda, int32_t* info, int32_t* status, void* workspace,
                 int64_t workspace_bytes, qgx_stream_t stream) {
  QGX_CHECK_ARG(n > 0 && lda >= n && A && info && workspace);
  QGX_CHECK_ARG(workspace_bytes >= chol_f64_workspace_bytes(n));
  QGX_CHECK_ARG((reinterpret_cast<uintptr_t>(workspace) & 255) == 0);
  int64_t kernels = 0;
  return chol_f64_graph(A, n, lda, info, status, workspace, as_cuda(stream), &kernels);
}

}  // extern "C"
