// Tensor-core Gram matrix T = A A^T on sm_103a with tcgen05 (quantax/optimizer/solver.py:139).
//
// One CTA computes one 128 x 128 tile of T on or below the diagonal (tiles taken in 8 x 8
// super-blocks, so that concurrently resident CTAs share operand panels in L2):
//   warp 4 / lane 0  TMA producer: 128 x 128-byte K-major tiles of the row block and of the
//                    column block, 128B-swizzled, into a ring of kStages shared-memory stages;
//   warp 5 / lane 0  MMA issuer: tcgen05.mma M=128 N=128 (K = 8 for tf32, 16 for bf16; four
//                    per 128-byte k-block); tcgen05.commit frees a stage when its MMAs are done;
//   warps 6-9        (split tf32 only) write the low parts lo = x - tf32(x) of the staged
//                    operands beside them;
//   warps 0-3        epilogue (warp w owns TMEM lanes 32w..32w+31, i.e. tile rows).
// K is accumulated in chunks of kChunkElems elements, alternately in two 128-column TMEM
// accumulators, each chunk starting from zero. The epilogue adds every finished chunk into
// FP32 registers (round to nearest) while the next chunk is computed, then stores the tile and
// its mirror in FP64, both coalesced (the direct tile goes through a shared-memory transpose).
// The tensor core's FP32 accumulation of one long K loses up to ~k 2^-25 relative with a
// systematic sign; with chunks that bias is bounded by the chunk length, and the rounding of
// the chunk sums is unbiased: T stays accurate enough for a diagonal shift of 1e-6 tr(T).
// Every mbarrier wait is bounded by a wall-clock limit; a wait that runs out records
// QGX_ERR_TIMEOUT in the optional status word, the CTA releases its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>

#include "qgx_common.cuh"
#include "qgx_tc.cuh"

namespace qgx {
namespace {

constexpr int kTile = 128;          // rows / columns of a T tile
constexpr int kGroup = 8;           // tiles per side of a rasterisation super-block
constexpr int kRowBytes = 128;      // bytes of one operand row per k-block (one swizzle atom)
constexpr int kBlockBytes = kTile * kRowBytes;  // one operand block of a stage
// KIND 0: tf32, 1: bf16, 2: split tf32 (hi*hi + hi*lo + lo*hi, FP32-class accuracy)
constexpr int kChunkElems = 256;  // K elements accumulated in TMEM before the epilogue takes them
template <int KIND>
struct GramCfg {
  static constexpr int kStageBytes = (KIND == 2 ? 4 : 2) * kBlockBytes;  // A, B (+ A lo, B lo)
  static constexpr int kStages = 3;
  static constexpr int kThreads = KIND == 2 ? 320 : 192;  // epilogue 0-3, producer 4, MMA 5, split 6-9
  static constexpr size_t kSmem = 1024 + (size_t)kStages * kStageBytes + 256;
  static constexpr int kElems = KIND == 1 ? 64 : 32;      // elements per 128-byte k-block
  static constexpr int kChunkBlocks = kChunkElems / kElems;
};
constexpr uint32_t kTmemCols = 256;  // two chunk accumulators

// K-major operand tile, 128-byte rows, 128B swizzle: 8-row core groups 1024 bytes apart
__device__ inline uint64_t smem_desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);  // start address
  d |= (uint64_t)1 << 16;                   // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;         // stride byte offset: 8 rows x 128 bytes
  d |= (uint64_t)1 << 46;                   // descriptor version of tcgen05
  d |= (uint64_t)2 << 61;                   // 128-byte swizzle
  return d;
}

// instruction descriptor: FP32 accumulator, K-major A and B, M = N = 128
template <int KIND>
constexpr uint32_t instr_desc() {
  // operand format: tf32 = 2 (kind::tf32), bf16 = 1 (kind::f16)
  return (1u << 4) | ((KIND == 1 ? 1u : 2u) << 7) | ((KIND == 1 ? 1u : 2u) << 10) | ((uint32_t)(kTile >> 3) << 17) |
         ((uint32_t)(kTile >> 4) << 24);
}

template <int KIND>
__device__ inline void mma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t accumulate) {
  if (KIND != 1) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(instr_desc<KIND>()), "r"(accumulate));
  } else {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(instr_desc<KIND>()), "r"(accumulate));
  }
}

// the TF32 value the tensor core takes from an FP32 operand: the 10 leading explicit mantissa
// bits, the 13 below them ignored
__device__ inline float tf32_hi(float x) { return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u); }

__device__ inline void record_status(int32_t* status, int code) {
  if (status) atomicExch(status, code);
}

template <int KIND>
__global__ void __launch_bounds__(GramCfg<KIND>::kThreads, 1)
    gram_tc_kernel(const __grid_constant__ CUtensorMap tmap, int64_t n, int64_t nkb, double* __restrict__ T,
                   int64_t ldt, int32_t* __restrict__ status) {
  using Cfg = GramCfg<KIND>;
  constexpr int kStages = Cfg::kStages;
  constexpr int kStageBytes = Cfg::kStageBytes;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + kStages * kStageBytes);
  uint64_t* empty = full + kStages;
  uint64_t* split = empty + kStages;  // KIND 2: operands split into hi / lo
  uint64_t* acc_full = split + kStages;   // two: a chunk accumulator is complete
  uint64_t* acc_empty = acc_full + 2;     // two: the epilogue has taken a chunk accumulator
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(acc_empty + 2);
  volatile int* fail = reinterpret_cast<volatile int*>(tmem_slot + 1);

  // block index -> tile (bi, bj), bi >= bj, grouped: kGroup x kGroup super-blocks in lower-
  // triangular order, row-major inside, so that the CTAs resident at once share a few row and
  // column panels of the operand in L2; blocks past the matrix or above the diagonal exit
  const int64_t sb = blockIdx.x / (kGroup * kGroup), w = blockIdx.x % (kGroup * kGroup);
  int64_t si = (int64_t)((sqrt(8.0 * (double)sb + 1.0) - 1.0) * 0.5);
  while ((si + 1) * (si + 2) / 2 <= sb) ++si;
  while (si * (si + 1) / 2 > sb) --si;
  const int64_t sj = sb - si * (si + 1) / 2;
  const int64_t bi = si * kGroup + w / kGroup, bj = sj * kGroup + w % kGroup;
  if (bi * kTile >= n || bj > bi) return;
  const int row0 = (int)(bi * kTile), col0 = (int)(bj * kTile);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
      mbar_init(&split[s], 128);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], 4);  // one arrival per epilogue warp
    }
    *fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  constexpr int kElems = Cfg::kElems;
  constexpr int kChunkBlocks = Cfg::kChunkBlocks;
  const int64_t nchunk = (nkb + kChunkBlocks - 1) / kChunkBlocks;

  if (warp == 4) {
    if (lane == 0) {
      for (int64_t kb = 0; kb < nkb && !*fail; ++kb) {
        const int s = (int)(kb % kStages);
        const uint32_t ph = (uint32_t)((kb / kStages) & 1);
        if (!mbar_wait(&empty[s], ph ^ 1u)) {
          *fail = 1;
          break;
        }
        uint8_t* a = smem + s * kStageBytes;
        uint8_t* b = a + kBlockBytes;
        mbar_expect_tx(&full[s], 2 * kBlockBytes);
        tma_load_2d(a, &tmap, &full[s], (int)(kb * kElems), row0);
        tma_load_2d(b, &tmap, &full[s], (int)(kb * kElems), col0);
      }
    }
  } else if (warp == 5) {
    if (lane == 0) {
      for (int64_t kb = 0; kb < nkb && !*fail; ++kb) {
        const int64_t c = kb / kChunkBlocks;
        const bool first = kb % kChunkBlocks == 0;
        const bool last = kb % kChunkBlocks == kChunkBlocks - 1 || kb == nkb - 1;
        const uint32_t acc = tmem + (uint32_t)(128 * (c & 1));
        // the accumulator of chunk c - 2 must have been taken by the epilogue
        if (first && c >= 2 && !mbar_wait(&acc_empty[c & 1], (uint32_t)((c >> 1) - 1) & 1)) {
          *fail = 1;
          break;
        }
        const int s = (int)(kb % kStages);
        const uint32_t ph = (uint32_t)((kb / kStages) & 1);
        if (!mbar_wait(KIND == 2 ? &split[s] : &full[s], ph)) {
          *fail = 1;
          break;
        }
        tc_fence_after();
        const uint32_t base = smem_u32(smem + s * kStageBytes);
        const uint64_t da = smem_desc_sw128(base);
        const uint64_t db = smem_desc_sw128(base + kBlockBytes);
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)  // 32 bytes of K per instruction
          mma<KIND>(acc, da + 2 * kk, db + 2 * kk, (first && kk == 0) ? 0u : 1u);
        if (KIND == 2) {
          const uint64_t la = smem_desc_sw128(base + 2 * kBlockBytes);
          const uint64_t lb = smem_desc_sw128(base + 3 * kBlockBytes);
#pragma unroll
          for (int kk = 0; kk < 4; ++kk) {
            mma<KIND>(acc, da + 2 * kk, lb + 2 * kk, 1u);
            mma<KIND>(acc, la + 2 * kk, db + 2 * kk, 1u);
          }
        }
        mma_commit(&empty[s]);
        if (last) mma_commit(&acc_full[c & 1]);
      }
    }
  } else if (KIND == 2 && warp >= 6) {
    // split x = hi + lo: the tensor core reads an FP32 operand as TF32 by ignoring its 13
    // low mantissa bits, so the staged x itself is hi; lo = x - hi is exact and goes to a
    // second buffer in the same swizzled layout (the tensor core reads lo truncated too)
    const int t = threadIdx.x - 192;
    for (int64_t kb = 0; kb < nkb && !*fail; ++kb) {
      const int s = (int)(kb % kStages);
      const uint32_t ph = (uint32_t)((kb / kStages) & 1);
      if (!mbar_wait(&full[s], ph)) {
        *fail = 1;
        break;
      }
      const float4* x = reinterpret_cast<const float4*>(smem + s * kStageBytes);
      float4* lo = reinterpret_cast<float4*>(smem + s * kStageBytes + 2 * kBlockBytes);
#pragma unroll 4
      for (int e = t; e < 2 * kBlockBytes / 16; e += 128) {
        const float4 v = x[e];
        lo[e] = make_float4(v.x - tf32_hi(v.x), v.y - tf32_hi(v.y), v.z - tf32_hi(v.z), v.w - tf32_hi(v.w));
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&split[s])) : "memory");
    }
  }

  // epilogue warps 0..3: take every chunk accumulator into the running sums
  float sum[kTile];
#pragma unroll
  for (int j = 0; j < kTile; ++j) sum[j] = 0.0f;
  const int q = warp & 3;
  if (warp < 4) {
    for (int64_t c = 0; c < nchunk; ++c) {
      if (*fail || !mbar_wait(&acc_full[c & 1], (uint32_t)(c >> 1) & 1)) {
        *fail = 1;
        break;
      }
      tc_fence_after();
#pragma unroll
      for (int g = 0; g < kTile / 32; ++g) {
        float v[32];
        tmem_ld_32cols(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(128 * (c & 1) + 32 * g), v);
#pragma unroll
        for (int j = 0; j < 32; ++j) sum[32 * g + j] += v[j];
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&acc_empty[c & 1])) : "memory");
    }
  }
  __syncthreads();  // every role has finished: the stage memory is free for the transpose
  if (*fail) {
    if (threadIdx.x == 0) record_status(status, QGX_ERR_TIMEOUT);
  } else if (warp < 4) {
    float* tr = reinterpret_cast<float*>(smem) + q * 32 * 33;
    const int r_local = 32 * q + lane;
#pragma unroll
    for (int g = 0; g < kTile / 32; ++g) {
      // mirror: T[col][row], consecutive lanes -> consecutive rows of T's column
      const int64_t r = row0 + r_local;
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int64_t cc = col0 + 32 * g + j;
        if (r < n && cc < n) T[cc * ldt + r] = (double)sum[32 * g + j];
      }
      if (bi != bj) {
#pragma unroll
        for (int j = 0; j < 32; ++j) tr[lane * 33 + j] = sum[32 * g + j];
        __syncwarp();
        const int64_t cc = col0 + 32 * g + lane;
        for (int j = 0; j < 32; ++j) {
          const int64_t rr = row0 + 32 * q + j;
          if (rr < n && cc < n) T[rr * ldt + cc] = (double)tr[j * 33 + lane];
        }
        __syncwarp();
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
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

template <int KIND>
int launch_gram_tc(const void* A, int64_t rows, int64_t k, int64_t lda, double* T, int64_t ldt, int32_t* status,
                   cudaStream_t st) {
  const int esize = KIND == 1 ? 2 : 4;
  const int elems = KIND == 1 ? 64 : 32;
  // TMA: 16-byte aligned base and row stride
  if ((reinterpret_cast<uintptr_t>(A) & 15) || ((lda * esize) & 15)) return QGX_ERR_UNSUPPORTED;
  if (rows > 0x7fffffffLL || k > 0x7fffffffLL) return QGX_ERR_UNSUPPORTED;
  EncodeTiled enc = encode_fn();
  if (!enc) return QGX_ERR_UNSUPPORTED;
  CUtensorMap map;
  const cuuint64_t dims[2] = {(cuuint64_t)k, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)(lda * esize)};
  const cuuint32_t box[2] = {(cuuint32_t)elems, (cuuint32_t)kTile};
  const cuuint32_t estr[2] = {1, 1};
  CUresult cr = enc(&map, KIND == 1 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                    const_cast<void*>(A), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (cr != CUDA_SUCCESS) return QGX_ERR_UNSUPPORTED;
  const int64_t nb = (rows + kTile - 1) / kTile;
  const int64_t ns = (nb + kGroup - 1) / kGroup;  // super-blocks per side
  const int64_t tiles = ns * (ns + 1) / 2 * kGroup * kGroup;
  if (tiles > 0x7fffffffLL) return QGX_ERR_UNSUPPORTED;
  const int64_t nkb = (k + elems - 1) / elems;
  auto kern = gram_tc_kernel<KIND>;
  constexpr size_t smem = GramCfg<KIND>::kSmem;
  QGX_CHECK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (status) QGX_CHECK_CUDA(cudaMemsetAsync(status, 0, sizeof(int32_t), st));
  kern<<<(unsigned)tiles, GramCfg<KIND>::kThreads, smem, st>>>(map, rows, nkb, T, ldt, status);
  return launch_status();
}

__global__ void to_bf16_kernel(const float* __restrict__ in, int64_t rows, int64_t k, int64_t ldi,
                               __nv_bfloat16* __restrict__ out, int64_t ldo) {
  const int64_t r = blockIdx.y;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < k; c += (int64_t)gridDim.x * blockDim.x)
    out[r * ldo + c] = __float2bfloat16_rn(in[r * ldi + c]);
}

// out[c][r] = in[r][c] through a 32 x 33 shared tile (coalesced reads and writes); OUT_BF16
// rounds to nearest even
template <bool OUT_BF16>
__global__ void transpose_kernel(const float* __restrict__ in, int64_t rows, int64_t cols, int64_t ldi,
                                 void* __restrict__ out, int64_t ldo) {
  __shared__ float tile[32][33];
  const int64_t r0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
  for (int i = ty; i < 32; i += 8) {
    const int64_t r = r0 + i, c = c0 + tx;
    tile[i][tx] = (r < rows && c < cols) ? in[r * ldi + c] : 0.0f;
  }
  __syncthreads();
  for (int i = ty; i < 32; i += 8) {
    const int64_t c = c0 + i, r = r0 + tx;
    if (c < cols && r < rows) {
      if (OUT_BF16)
        reinterpret_cast<__nv_bfloat16*>(out)[c * ldo + r] = __float2bfloat16_rn(tile[tx][i]);
      else
        reinterpret_cast<float*>(out)[c * ldo + r] = tile[tx][i];
    }
  }
}

}  // namespace

int gram_tc(const float* A, int64_t rows, int64_t k, int64_t lda, double* T, int64_t ldt, int mode, cudaStream_t st) {
  if (mode == QGX_GRAM_TF32 && k > 0) return launch_gram_tc<0>(A, rows, k, lda, T, ldt, nullptr, st);
  if (mode == QGX_GRAM_3XTF32 && k > 0) return launch_gram_tc<2>(A, rows, k, lda, T, ldt, nullptr, st);
  return QGX_ERR_UNSUPPORTED;
}

}  // namespace qgx

using namespace qgx;

extern "C" {

int qgx_gram_tc(const void* A, int32_t a_dtype, int64_t rows, int64_t k, int64_t lda, double* T, int64_t ldt,
                int32_t* status, qgx_stream_t stream) {
  QGX_CHECK_ARG(rows >= 0 && k > 0 && lda >= k && ldt >= rows && a_dtype >= 0 && a_dtype <= 2);
  if (rows == 0) return QGX_OK;
  QGX_CHECK_ARG(A && T);
  if (a_dtype == 0) return launch_gram_tc<0>(A, rows, k, lda, T, ldt, status, as_cuda(stream));
  if (a_dtype == 2) return launch_gram_tc<2>(A, rows, k, lda, T, ldt, status, as_cuda(stream));
  return launch_gram_tc<1>(A, rows, k, lda, T, ldt, status, as_cuda(stream));
}

int qgx_transpose(const float* in, int64_t rows, int64_t cols, int64_t ldi, void* out, int64_t ldo, int32_t out_dtype,
                  qgx_stream_t stream) {
  QGX_CHECK_ARG(rows >= 0 && cols >= 0 && ldi >= cols && ldo >= rows && (out_dtype == 0 || out_dtype == 1));
  if (rows == 0 || cols == 0) return QGX_OK;
  QGX_CHECK_ARG(in && out);
  const int64_t gy = (rows + 31) / 32, gx = (cols + 31) / 32;
  QGX_CHECK_ARG(gy <= 65535 && gx <= 2147483647LL);
  if (out_dtype == 1)
    transpose_kernel<true><<<dim3((unsigned)gx, (unsigned)gy), 256, 0, as_cuda(stream)>>>(in, rows, cols, ldi, out, ldo);
  else
    transpose_kernel<false><<<dim3((unsigned)gx, (unsigned)gy), 256, 0, as_cuda(stream)>>>(in, rows, cols, ldi, out, ldo);
  return launch_status();
}

int qgx_f32_to_bf16(const float* in, int64_t rows, int64_t k, int64_t ldi, uint16_t* out, int64_t ldo,
                    qgx_stream_t stream) {
  QGX_CHECK_ARG(rows >= 0 && k >= 0 && ldi >= k && ldo >= k);
  if (rows == 0 || k == 0) return QGX_OK;
  QGX_CHECK_ARG(in && out && rows <= 2147483647LL);
  const unsigned gx = (unsigned)std::min<int64_t>((k + 255) / 256, 64);
  to_bf16_kernel<<<dim3(gx, (unsigned)std::min<int64_t>(rows, 65535)), 256, 0, as_cuda(stream)>>>(
      in, std::min<int64_t>(rows, 65535), k, ldi, reinterpret_cast<__nv_bfloat16*>(out), ldo);
  for (int64_t r0 = 65535; r0 < rows; r0 += 65535) {
    const int64_t rr = std::min<int64_t>(65535, rows - r0);
    to_bf16_kernel<<<dim3(gx, (unsigned)rr), 256, 0, as_cuda(stream)>>>(
        in + r0 * ldi, rr, k, ldi, reinterpret_cast<__nv_bfloat16*>(out) + r0 * ldo, ldo);
  }
  return launch_status();
}

}  // extern "C"
