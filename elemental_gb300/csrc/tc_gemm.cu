// K5 on the 5th-generation tensor cores: the trailing Schur update
//   C[m x n] -= A[m x K] * B[K x n]      (C FP32, column-major, in place)
// of the low-precision factorizations (El::LU's Gemm(NORMAL, NORMAL, -1,
// A21, A12, 1, A22), src/lapack_like/factor/LU.cpp:134) and the blocked TRSM
// updates, written for sm_103a with tcgen05 + TMEM + TMA in inline PTX.
//
// Operands are first packed (pack_a / pack_b) into K-major tiles of the
// operand precision: BF16 (tcgen05.mma kind::f16) or TF32 (kind::tf32, FP32
// storage rounded to TF32).  One CTA computes a 128 x 256 tile of C:
//   warp 0 / lane 0  TMA producer: 128-byte-swizzled A and B k-blocks into a
//                    2-stage shared-memory ring (mbarrier full/empty);
//   warp 1 / lane 0  MMA issuer: 4 tcgen05.mma (K = 128 bytes) per k-block
//                    into a 128 x 256 FP32 accumulator in TMEM, commits free
//                    the stage and finally signal the epilogue;
//   warps 0-7        epilogue: tcgen05.ld 32 lanes x 32 columns, C -= acc
//                    with coalesced loads/stores (lane = row of the column-
//                    major C), the C loads issued before the accumulator is
//                    ready.
// ~97 KB of shared memory and 256 TMEM columns per CTA, so two CTAs share an
// SM and one's epilogue (HBM-bound) overlaps the other's MMA.  Every wait is
// bounded (globaltimer); a timeout records an error and the CTA still frees
// its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp8.h>
#include <cudaTypedefs.h>

#include "kernels.h"
#include "tc_gemm.h"
#include "tcgen05.cuh"

namespace elgb {

namespace {

using namespace tc;

constexpr int kBM = 128;
constexpr int kBN = 256;
constexpr int kBKBytes = 128;  // one 128-byte swizzle row of K per stage
constexpr int kStages = 2;
constexpr int kStageA = kBM * kBKBytes;  // 16 KB
constexpr int kStageB = kBN * kBKBytes;  // 32 KB
constexpr int kTmemCols = 256;
constexpr int kGemmThreads = 256;

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// Instruction descriptor: D FP32, A/B BF16 (kind::f16) or TF32, both
// K-major, M = 128, N = 256.
template <int KIND>
__host__ __device__ constexpr uint32_t idesc_m128n256() {
  // operand formats: kind::f16 BF16 = 1, kind::tf32 TF32 = 2, kind::f8f6f4 E4M3 = 0
  constexpr uint32_t fmt = KIND == kTcBF16 ? 1u : KIND == kTcFP8 ? 0u : 2u;
  return (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(kBN >> 3) << 17) |
         ((uint32_t)(kBM >> 4) << 24);
}

// Power-of-two scale mapping an operand whose largest magnitude is amax to
// at most the E4M3 maximum 448 (1 for an all-zero operand).
__host__ __device__ __forceinline__ float fp8_scale(float amax) {
  if (!(amax > 0.f) || !(amax < 3.0e38f)) return 1.f;
  return ldexpf(1.f, ilogbf(448.f / amax));
}

// passes = 1: C -= A B.  passes = 3 (TF32 split, ~FP32 accuracy):
// C -= Ahi Bhi + Ahi Blo + Alo Bhi, one accumulator, the three products
// streamed through the same pipeline one after the other.
template <int KIND>
__global__ void __launch_bounds__(kGemmThreads, 2)
tc_gemm_sub_kernel(const __grid_constant__ CUtensorMap tmA,
                   const __grid_constant__ CUtensorMap tmB,
                   const __grid_constant__ CUtensorMap tmAlo,
                   const __grid_constant__ CUtensorMap tmBlo, float* __restrict__ C, long ldc,
                   int m, int n, int num_kb, int passes, const float* __restrict__ amax,
                   DevStatus* st) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1024-byte alignment for the swizzled tiles
  unsigned char* base = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* sA = base;
  unsigned char* sB = base + kStages * kStageA;
  __shared__ __align__(8) uint64_t full_bar[kStages];
  __shared__ __align__(8) uint64_t empty_bar[kStages];
  __shared__ __align__(8) uint64_t accum_bar;
  __shared__ uint32_t s_tmem;
  __shared__ int s_abort;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * kBN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(&accum_bar, 1);
    s_abort = 0;
    fence_mbar_init();
  }
  if (warp == 1) tmem_alloc(&s_tmem, kTmemCols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = s_tmem;

  const int total_kb = num_kb * passes;
  if (warp == 0 && lane == 0) {
    // TMA producer
    for (int kb = 0; kb < total_kb; ++kb) {
      const int s = kb % kStages;
      if (kb >= kStages) {
        if (!mbar_wait(&empty_bar[s], ((kb / kStages) & 1) ^ 1, st, 10)) {
          s_abort = 1;
          break;
        }
      }
      const int pass = kb / num_kb;
      mbar_arrive_expect_tx(&full_bar[s], kStageA + kStageB);
      const int xk = (kb - pass * num_kb) * (kBKBytes / (KIND == kTcBF16 ? 2 : KIND == kTcFP8 ? 1 : 4));
      tma_load_2d(sA + s * kStageA, pass == 2 ? &tmAlo : &tmA, &full_bar[s], xk, m0);
      tma_load_2d(sB + s * kStageB, pass == 1 ? &tmBlo : &tmB, &full_bar[s], xk, n0);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    constexpr uint32_t idesc = idesc_m128n256<KIND>();
    bool ok = true;
    for (int kb = 0; kb < total_kb && ok; ++kb) {
      const int s = kb % kStages;
      if (!mbar_wait(&full_bar[s], (kb / kStages) & 1, st, 11)) {
        s_abort = 1;
        ok = false;
        break;
      }
      tc_fence_after();
      const uint64_t adesc = sdesc_sw128(smem_u32(sA + s * kStageA));
      const uint64_t bdesc = sdesc_sw128(smem_u32(sB + s * kStageB));
#pragma unroll
      for (int kk = 0; kk < 4; ++kk)  // 4 x 32 bytes of K per 128-byte row
        umma<KIND>(tmem, adesc + 2 * kk, bdesc + 2 * kk, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
      umma_commit(&empty_bar[s]);
    }
    umma_commit(&accum_bar);
  }
  __syncwarp();

  // Epilogue: all 8 warps.  Warp w reads TMEM lanes 32*(w%4).. (rows) and
  // the column half w/4.
  const int wl = warp & 3, half = warp >> 2;
  const int row = m0 + 32 * wl + lane;
  const bool row_ok = row < m;
  float* crow = C + row;
  // FP8: the products carry the operands' scales (exact powers of two)
  const float unscale = KIND == kTcFP8 ? 1.f / (fp8_scale(amax[0]) * fp8_scale(amax[1])) : 1.f;
  bool ready = false;
  for (int cc = 0; cc < 4; ++cc) {
    const int cbase = half * 128 + cc * 32;
    float cv[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const int col = n0 + cbase + j;
      cv[j] = (row_ok && col < n) ? crow[(long)col * ldc] : 0.f;
    }
    if (!ready) {
      // warp-uniform decision: tcgen05.ld below is a whole-warp instruction
      ready = __all_sync(0xffffffffu, mbar_wait(&accum_bar, 0, st, 12));
      tc_fence_after();
      if (!ready) break;
    }
    uint32_t acc[32];
    tmem_ld32(tmem + ((uint32_t)(32 * wl) << 16) + (uint32_t)cbase, acc);
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const int col = n0 + cbase + j;
      if (row_ok && col < n) crow[(long)col * ldc] = cv[j] - __uint_as_float(acc[j]) * unscale;
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, kTmemCols);
  }
}

// ---------------------------------------------------------------------------
// Operand packing: FP32 column-major -> K-major BF16 / TF32 rows, K padded
// ---------------------------------------------------------------------------
__device__ __forceinline__ float to_tf32(float v) {
  uint32_t t;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(v));
  return __uint_as_float(t);
}

// Writes the operand value (and, for the split form, the TF32 remainder
// v - tf32(v) to `lo`).
template <int KIND>
__device__ __forceinline__ void store_op(void* out, void* lo, size_t idx, float v, float scale) {
  if (KIND == kTcFP8) {
    reinterpret_cast<__nv_fp8_storage_t*>(out)[idx] =
        __nv_cvt_float_to_fp8(v * scale, __NV_SATFINITE, __NV_E4M3);
  } else if (KIND == kTcBF16) {
    reinterpret_cast<__nv_bfloat16*>(out)[idx] = __float2bfloat16_rn(v);
  } else {
    const float hi = to_tf32(v);
    reinterpret_cast<float*>(out)[idx] = hi;
    if (lo) reinterpret_cast<float*>(lo)[idx] = to_tf32(v - hi);
  }
}

// A (m x K, column-major) -> out[i * Kp + k]; 32 x 32 tiles through shared
// memory so both the read and the write are coalesced.
template <int KIND>
__global__ void pack_a_kernel(const float* __restrict__ A, long lda, int m, int K, int Kp,
                              void* __restrict__ out, void* __restrict__ lo,
                              const float* __restrict__ amax) {
  __shared__ float t[32][33];
  const float scale = KIND == kTcFP8 ? fp8_scale(amax[0]) : 1.f;
  const int i0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  for (int q = 0; q < 32; q += 8) {
    const int i = i0 + tx, k = k0 + ty + q;
    t[ty + q][tx] = (i < m && k < K) ? A[i + (long)k * lda] : 0.f;
  }
  __syncthreads();
  for (int q = 0; q < 32; q += 8) {
    const int i = i0 + ty + q, k = k0 + tx;
    if (i < m && k < Kp) store_op<KIND>(out, lo, (size_t)i * Kp + k, t[tx][ty + q], scale);
  }
}

// B (K x n, column-major) -> out[j * Kp + k]: already K-contiguous.
template <int KIND>
__global__ void pack_b_kernel(const float* __restrict__ B, long ldb, int K, int n, int Kp,
                              void* __restrict__ out, void* __restrict__ lo,
                              const float* __restrict__ amax) {
  const float scale = KIND == kTcFP8 ? fp8_scale(amax[1]) : 1.f;
  for (int j = blockIdx.y; j < n; j += gridDim.y)
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < Kp; k += gridDim.x * blockDim.x)
      store_op<KIND>(out, lo, (size_t)j * Kp + k, k < K ? B[k + (long)j * ldb] : 0.f, scale);
}

// amax[0] = max |A| (m x K), amax[1] = max |B| (K x n), both column-major;
// amax zeroed beforehand.  Non-negative floats order as their bit patterns.
__global__ void absmax_kernel(const float* __restrict__ A, long lda, int m, int K,
                              const float* __restrict__ B, long ldb, int n,
                              float* __restrict__ amax) {
  float a = 0.f, b = 0.f;
  const long na = (long)m * K, nb = (long)K * n;
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < na; i += stride)
    a = fmaxf(a, fabsf(A[(i % m) + (i / m) * lda]));
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < nb; i += stride)
    b = fmaxf(b, fabsf(B[(i % K) + (i / K) * ldb]));
  for (int o = 16; o > 0; o >>= 1) {
    a = fmaxf(a, __shfl_xor_sync(0xffffffffu, a, o));
    b = fmaxf(b, __shfl_xor_sync(0xffffffffu, b, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(reinterpret_cast<int*>(amax), __float_as_int(a));
    atomicMax(reinterpret_cast<int*>(amax) + 1, __float_as_int(b));
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                         cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// 2-D K-major operand map: inner dim K (padded, Kp), outer dim rows; box of
// one 128-byte K row by `box_rows` rows, 128-byte swizzle.
bool make_operand_map(CUtensorMap* map, void* gptr, int kind, int Kp, int rows, int box_rows) {
  auto fn = encode_fn();
  if (!fn) return false;
  const int esz = kind == kTcBF16 ? 2 : kind == kTcFP8 ? 1 : 4;
  cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)Kp * esz};
  cuuint32_t box[2] = {(cuuint32_t)(kBKBytes / esz), (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, kind == kTcBF16  ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16
                       : kind == kTcFP8 ? CU_TENSOR_MAP_DATA_TYPE_UINT8
                                        : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                  2, gptr, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

}  // namespace

static size_t rup1k(size_t b) { return (b + 1023) / 1024 * 1024; }

static int op_esz(int kind) { return kind == kTcBF16 ? 2 : kind == kTcFP8 ? 1 : 4; }

size_t tc_gemm_workspace_bytes(int kind, int m, int n, int K) {
  const int esz = op_esz(kind);
  const int kbe = kBKBytes / esz;
  const size_t Kp = (size_t)((K + kbe - 1) / kbe) * kbe;
  const size_t copies = kind == kTcTF32x3 ? 2 : 1;
  return copies * (rup1k((size_t)m * Kp * esz) + rup1k((size_t)n * Kp * esz)) + 1024;
}

cudaError_t launch_tc_gemm_sub(int kind, int m, int n, int K, const float* A, long lda,
                               const float* B, long ldb, float* C, long ldc, void* ws,
                               DevStatus* st, cudaStream_t stream, int* nlaunch,
                               cudaEvent_t ev0, cudaEvent_t ev1) {
  if (nlaunch) *nlaunch = 0;
  if (m <= 0 || n <= 0 || K <= 0) return cudaSuccess;
  const bool split = kind == kTcTF32x3;
  const int esz = op_esz(kind);
  const int kbe = kBKBytes / esz;
  const int Kp = (K + kbe - 1) / kbe * kbe;
  char* Abuf = static_cast<char*>(ws);
  char* Bbuf = Abuf + rup1k((size_t)m * Kp * esz);
  char* Alo = split ? Bbuf + rup1k((size_t)n * Kp * esz) : nullptr;
  char* Blo = split ? Alo + rup1k((size_t)m * Kp * esz) : nullptr;
  // FP8 operand maxima (per call, i.e. per panel) after the packed operands
  float* amax = reinterpret_cast<float*>(
      Abuf + (split ? 2 : 1) * (rup1k((size_t)m * Kp * esz) + rup1k((size_t)n * Kp * esz)));
  dim3 pg((m + 31) / 32, (Kp + 31) / 32);
  int nl = 2;
  if (kind == kTcFP8) {
    cudaError_t e0 = cudaMemsetAsync(amax, 0, 2 * sizeof(float), stream);
    if (e0 != cudaSuccess) return e0;
    absmax_kernel<<<1024, 256, 0, stream>>>(A, lda, m, K, B, ldb, n, amax);
    pack_a_kernel<kTcFP8><<<pg, dim3(32, 8), 0, stream>>>(A, lda, m, K, Kp, Abuf, nullptr, amax);
    pack_b_kernel<kTcFP8><<<dim3((Kp + 255) / 256, grid_y(n)), 256, 0, stream>>>(B, ldb, K, n, Kp,
                                                                        Bbuf, nullptr, amax);
    nl = 3;
  } else if (kind == kTcBF16) {
    pack_a_kernel<kTcBF16><<<pg, dim3(32, 8), 0, stream>>>(A, lda, m, K, Kp, Abuf, nullptr,
                                                           amax);
    pack_b_kernel<kTcBF16><<<dim3((Kp + 255) / 256, grid_y(n)), 256, 0, stream>>>(B, ldb, K, n, Kp,
                                                                         Bbuf, nullptr, amax);
  } else {
    pack_a_kernel<kTcTF32><<<pg, dim3(32, 8), 0, stream>>>(A, lda, m, K, Kp, Abuf, Alo, amax);
    pack_b_kernel<kTcTF32><<<dim3((Kp + 255) / 256, grid_y(n)), 256, 0, stream>>>(B, ldb, K, n, Kp,
                                                                         Bbuf, Blo, amax);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int mk = kind == kTcTF32x3 ? kTcTF32 : kind;
  CUtensorMap tmA, tmB, tmAlo, tmBlo;
  if (!make_operand_map(&tmA, Abuf, mk, Kp, m, kBM) ||
      !make_operand_map(&tmB, Bbuf, mk, Kp, n, kBN))
    return cudaErrorInvalidValue;
  if (split) {
    if (!make_operand_map(&tmAlo, Alo, mk, Kp, m, kBM) ||
        !make_operand_map(&tmBlo, Blo, mk, Kp, n, kBN))
      return cudaErrorInvalidValue;
  } else {
    tmAlo = tmA;
    tmBlo = tmB;
  }
  const size_t smem = kStages * (kStageA + kStageB) + 1024;
  dim3 grid((m + kBM - 1) / kBM, (n + kBN - 1) / kBN);
  const int num_kb = Kp / kbe;
  const int passes = split ? 3 : 1;
  if (ev0) cudaEventRecord(ev0, stream);
  auto kern = kind == kTcBF16  ? tc_gemm_sub_kernel<kTcBF16>
              : kind == kTcFP8 ? tc_gemm_sub_kernel<kTcFP8>
                               : tc_gemm_sub_kernel<kTcTF32>;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  kern<<<grid, kGemmThreads, smem, stream>>>(tmA, tmB, tmAlo, tmBlo, C, ldc, m, n, num_kb,
                                             passes, amax, st);
  if (ev1) cudaEventRecord(ev1, stream);
  if (nlaunch) *nlaunch = nl + 1;
  return cudaGetLastError();
}

}  // namespace elgb
