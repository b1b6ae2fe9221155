// K5 on the 5th-generation tensor cores: the trailing Schur update
//   C[m x n] -= A[m x K] * B[K x n]      (C FP32, column-major, in place)
// of the low-precision factorizations (El::LU's Gemm(NORMAL, NORMAL, -1,
// A21, A12, 1, A22), src/lapack_like/factor/LU.cpp:134) and the blocked TRSM
// updates, written for sm_103a with tcgen05 + TMEM + TMA in inline PTX.
//
// Operands are first packed (pack_a / pack_b) into K-major tiles of the
// operand precision: BF16 (tcgen05.mma kind::f16), TF32 (kind::tf32, FP32
// storage rounded to TF32, optionally split hi + lo for three products) or
// E4M3 (kind::f8f6f4, scaled per call).  tc_gemm_persistent_kernel then walks
// the 128 x 256 C tiles with one CTA per SM of a bounded grid; its layout is
// described above the kernel.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
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
constexpr int kStageA = kBM * kBKBytes;  // 16 KB
constexpr int kStageB = kBN * kBKBytes;  // 32 KB

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

// ---------------------------------------------------------------------------
// Persistent form: one CTA per SM (of a bounded grid) walks the 128 x 256
// tiles in groups of `group_n` tile columns, n fastest within a group (see
// tile_origin).  Each stage of the shared-memory ring holds a
// k-block of every operand copy at once -- for TF32x3 the hi and lo tiles of
// A and of B (96 KB), from which the three products are issued, instead of
// streaming the operands three times -- and two 256-column TMEM
// accumulators let the epilogue of tile t overlap the MMAs of tile t + 1.
//   warp 0 / lane 0  TMA producer over (tile, k-block), 2-stage ring (4 for
//                    the single-product kinds);
//   warp 1 / lane 0  MMA issuer; commits free a stage, and a finished
//                    accumulator is signalled on tfull[b];
//   warps 2..5       epilogue (warp w reads TMEM lanes 32 (w % 4) ..), C -=
//                    acc, then one arrive per warp on tempty[b].
// 197 KB of shared memory: one CTA per SM, so the grid bounds the SMs the
// kernel holds (the look-ahead panel of the factorization keeps the rest).
// Every wait is bounded; a timeout records an error and the CTA still frees
// its TMEM.
constexpr int kPThreads = 192;
constexpr int kPRing = 192 * 1024;
constexpr int kPTmemCols = 512;

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Origin (m0, n0) of tile t.  The tile columns are taken `group_n` at a time
// and, within a group, the tiles run n fastest: the CTAs of one wave share a
// few rows of A tiles and the group's B tiles, which stay in L2 from wave to
// wave, so A streams from DRAM once per group instead of once per tile
// column (m fastest re-read all of A for every column of tiles).
__device__ __forceinline__ void tile_origin(int t, int tiles_m, int tiles_n, int group_n,
                                            int& m0, int& n0) {
  const int per_group = group_n * tiles_m;
  const int g = t / per_group, idx = t - g * per_group;
  const int gn = min(group_n, tiles_n - g * group_n);
  m0 = (idx / gn) * kBM;
  n0 = (g * group_n + idx % gn) * kBN;
}

template <int KIND, bool SPLIT>
__global__ void __launch_bounds__(kPThreads, 1)
tc_gemm_persistent_kernel(const __grid_constant__ CUtensorMap tmA,
                          const __grid_constant__ CUtensorMap tmB,
                          const __grid_constant__ CUtensorMap tmAlo,
                          const __grid_constant__ CUtensorMap tmBlo, float* __restrict__ C,
                          long ldc, int m, int n, int num_kb, int group_n,
                          const float* __restrict__ amax, DevStatus* st) {
  constexpr int kStageBytes = (SPLIT ? 2 : 1) * (kStageA + kStageB);
  constexpr int kS = kPRing / kStageBytes;  // 2 (split) or 4 stages
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ __align__(8) uint64_t full_bar[kS];
  __shared__ __align__(8) uint64_t empty_bar[kS];
  __shared__ __align__(8) uint64_t tfull[2];
  __shared__ __align__(8) uint64_t tempty[2];
  __shared__ __align__(8) uint64_t drain_bar;
  __shared__ uint32_t s_tmem;
  __shared__ volatile int s_abort;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tiles_m = (m + kBM - 1) / kBM, tiles_n = (n + kBN - 1) / kBN;
  const int ntiles = tiles_m * tiles_n;
  pdl_launch_dependents();  // a leaf panel after it may be scheduled now
  // stage s: A hi | B hi | A lo | B lo
  auto sA = [&](int s) { return base + (size_t)s * kStageBytes; };
  auto sB = [&](int s) { return base + (size_t)s * kStageBytes + kStageA; };
  auto sAl = [&](int s) { return base + (size_t)s * kStageBytes + kStageA + kStageB; };
  auto sBl = [&](int s) { return base + (size_t)s * kStageBytes + 2 * kStageA + kStageB; };

  if (threadIdx.x == 0) {
    for (int s = 0; s < kS; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], 4);
    }
    mbar_init(&drain_bar, 1);
    s_abort = 0;
    fence_mbar_init();
  }
  if (warp == 1) tmem_alloc(&s_tmem, kPTmemCols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = s_tmem;

  uint32_t it_issued = 0;  // producer: k-blocks whose loads were issued
  if (warp == 0 && lane == 0) {
    // TMA producer
    uint32_t it = 0;
    for (int t = blockIdx.x; t < ntiles && !s_abort; t += gridDim.x) {
      int m0, n0;
      tile_origin(t, tiles_m, tiles_n, group_n, m0, n0);
      for (int kb = 0; kb < num_kb; ++kb, ++it) {
        const int s = it % kS;
        if (it >= (uint32_t)kS && !mbar_wait(&empty_bar[s], ((it / kS) & 1) ^ 1, st, 20)) {
          s_abort = 1;
          break;
        }
        mbar_arrive_expect_tx(&full_bar[s], kStageBytes);
        const int xk = kb * (kBKBytes / (KIND == kTcBF16 ? 2 : KIND == kTcFP8 ? 1 : 4));
        tma_load_2d(sA(s), &tmA, &full_bar[s], xk, m0);
        tma_load_2d(sB(s), &tmB, &full_bar[s], xk, n0);
        if (SPLIT) {
          tma_load_2d(sAl(s), &tmAlo, &full_bar[s], xk, m0);
          tma_load_2d(sBl(s), &tmBlo, &full_bar[s], xk, n0);
        }
        it_issued = it + 1;
      }
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    constexpr uint32_t idesc = idesc_m128n256<KIND>();
    uint32_t it = 0, lt = 0;
    for (int t = blockIdx.x; t < ntiles && !s_abort; t += gridDim.x, ++lt) {
      const int b = lt & 1;
      const uint32_t u = lt >> 1;
      if (lt >= 2 && !mbar_wait(&tempty[b], (u - 1) & 1, st, 21)) {
        s_abort = 1;
        break;
      }
      tc_fence_after();
      const uint32_t d = tmem + (uint32_t)(b * kBN);
      bool ok = true;
      for (int kb = 0; kb < num_kb; ++kb, ++it) {
        const int s = it % kS;
        if (!mbar_wait(&full_bar[s], (it / kS) & 1, st, 22)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint64_t ah = sdesc_sw128(smem_u32(sA(s))), bh = sdesc_sw128(smem_u32(sB(s)));
        const uint64_t al = sdesc_sw128(smem_u32(sAl(s))), bl = sdesc_sw128(smem_u32(sBl(s)));
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {  // 4 x 32 bytes of K per 128-byte row
          umma<KIND>(d, ah + 2 * kk, bh + 2 * kk, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
          if (SPLIT) {
            umma<KIND>(d, ah + 2 * kk, bl + 2 * kk, idesc, 1u);
            umma<KIND>(d, al + 2 * kk, bh + 2 * kk, idesc, 1u);
          }
        }
        umma_commit(&empty_bar[s]);
      }
      if (!ok) {
        s_abort = 1;
        break;
      }
      umma_commit(&tfull[b]);
    }
  } else if (warp >= 2) {
    // epilogue: warp w reads TMEM lanes 32 * (w % 4) .. (rows of the tile)
    const int q = warp & 3;
    const float unscale =
        KIND == kTcFP8 ? 1.f / (fp8_scale(amax[0]) * fp8_scale(amax[1])) : 1.f;
    uint32_t lt = 0;
    for (int t = blockIdx.x; t < ntiles && !s_abort; t += gridDim.x, ++lt) {
      const int b = lt & 1;
      const uint32_t u = lt >> 1;
      int m0, n0;
      tile_origin(t, tiles_m, tiles_n, group_n, m0, n0);
      const int row = m0 + 32 * q + lane;
      const bool row_ok = row < m;
      float* crow = C + row;
      float cv[32];
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int col = n0 + j;
        cv[j] = (row_ok && col < n) ? crow[(long)col * ldc] : 0.f;
      }
      // warp-uniform: tcgen05.ld below is a whole-warp instruction
      const bool ready = __all_sync(0xffffffffu, mbar_wait(&tfull[b], u & 1, st, 23));
      tc_fence_after();
      if (!ready) {
        s_abort = 1;
        break;
      }
      for (int cc = 0; cc < kBN / 32; ++cc) {
        uint32_t acc[32];
        tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * kBN + cc * 32), acc);
        float nx[32];
        if (cc + 1 < kBN / 32) {
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int col = n0 + (cc + 1) * 32 + j;
            nx[j] = (row_ok && col < n) ? crow[(long)col * ldc] : 0.f;
          }
        }
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int col = n0 + cc * 32 + j;
          if (row_ok && col < n) crow[(long)col * ldc] = cv[j] - __uint_as_float(acc[j]) * unscale;
        }
        if (cc + 1 < kBN / 32) {
#pragma unroll
          for (int j = 0; j < 32; ++j) cv[j] = nx[j];
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty[b]);
    }
  }
  __syncwarp();  // lanes 1..31 of the producer and MMA warps wait for lane 0
  __syncthreads();
  if (s_abort) {
    // a wait gave up: let this CTA's own asynchronous work land (bounded)
    // before its shared memory and TMEM go away
    if (warp == 0 && lane == 0) {
      const uint32_t first = it_issued > (uint32_t)kS ? it_issued - kS : 0;
      for (uint32_t i = first; i < it_issued; ++i)
        mbar_wait(&full_bar[i % kS], (i / kS) & 1, st, 24);
    } else if (warp == 1 && lane == 0) {
      umma_commit(&drain_bar);
      mbar_wait(&drain_bar, 0, st, 25);
    }
    __syncwarp();
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, kPTmemCols);
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

// SMs of the current device (cached per device).
static int num_sms() {
  static int cache[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return 148;
  if (!cache[dev]) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    cache[dev] = v > 0 ? v : 148;
  }
  return cache[dev];
}

// How many 16-CTA clusters of the persistent kernel `kern` fit the device at
// once (one per GPC with 16 SMs to spare); 0 if clusters of 16 are
// unavailable.  Cached per device and kernel variant (0..3); the non-portable
// cluster size is allowed on the kernel at the first query.
template <typename K>
static int clusters16(K kern, int variant, size_t smem) {
  static int cache[64][4] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  const bool cached = dev >= 0 && dev < 64 && variant >= 0 && variant < 4;
  if (cached && cache[dev][variant]) return cache[dev][variant] > 0 ? cache[dev][variant] : 0;
  int r = -1;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
      cudaSuccess) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(16);
    cfg.blockDim = dim3(kPThreads);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 16;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nc = 0;
    if (cudaOccupancyMaxActiveClusters(&nc, (void*)kern, &cfg) == cudaSuccess && nc > 0) r = nc;
  }
  cudaGetLastError();
  if (cached) cache[dev][variant] = r;
  return r > 0 ? r : 0;
}

cudaError_t launch_tc_gemm_sub(int kind, int m, int n, int K, const float* A, long lda,
                               const float* B, long ldb, float* C, long ldc, void* ws,
                               DevStatus* st, cudaStream_t stream, int* nlaunch,
                               cudaEvent_t ev0, cudaEvent_t ev1, int grid_mode, bool a_packed) {
  if (nlaunch) *nlaunch = 0;
  if (m <= 0 || n <= 0 || K <= 0) return cudaSuccess;
  const bool split = kind == kTcTF32x3;
  const int esz = op_esz(kind);
  const int kbe = kBKBytes / esz;
  const int Kp = (K + kbe - 1) / kbe * kbe;
  // the packed A words first (their place depends on m and K only, so a
  // caller may reuse them: a_packed), then B's
  const size_t asz = rup1k((size_t)m * Kp * esz), bsz = rup1k((size_t)n * Kp * esz);
  char* Abuf = static_cast<char*>(ws);
  char* Alo = split ? Abuf + asz : nullptr;
  char* Bbuf = Abuf + (split ? 2 : 1) * asz;
  char* Blo = split ? Bbuf + bsz : nullptr;
  // FP8 operand maxima (per call, i.e. per panel) after the packed operands
  float* amax = reinterpret_cast<float*>(Abuf + (split ? 2 : 1) * (asz + bsz));
  if (kind == kTcFP8) a_packed = false;  // its scale is taken over A and B per call
  dim3 pg((m + 31) / 32, (Kp + 31) / 32);
  int nl = a_packed ? 1 : 2;
  if (kind == kTcFP8) {
    cudaError_t e0 = cudaMemsetAsync(amax, 0, 2 * sizeof(float), stream);
    if (e0 != cudaSuccess) return e0;
    absmax_kernel<<<1024, 256, 0, stream>>>(A, lda, m, K, B, ldb, n, amax);
    pack_a_kernel<kTcFP8><<<pg, dim3(32, 8), 0, stream>>>(A, lda, m, K, Kp, Abuf, nullptr, amax);
    pack_b_kernel<kTcFP8><<<dim3((Kp + 255) / 256, grid_y(n)), 256, 0, stream>>>(B, ldb, K, n, Kp,
                                                                        Bbuf, nullptr, amax);
    nl = 3;
  } else if (kind == kTcBF16) {
    if (!a_packed)
      pack_a_kernel<kTcBF16><<<pg, dim3(32, 8), 0, stream>>>(A, lda, m, K, Kp, Abuf, nullptr,
                                                             amax);
    pack_b_kernel<kTcBF16><<<dim3((Kp + 255) / 256, grid_y(n)), 256, 0, stream>>>(B, ldb, K, n, Kp,
                                                                         Bbuf, nullptr, amax);
  } else {
    if (!a_packed)
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
  const int num_kb = Kp / kbe;
  const int tiles = ((m + kBM - 1) / kBM) * ((n + kBN - 1) / kBN);
  const int sms = num_sms();
  auto kern = kind == kTcBF16  ? tc_gemm_persistent_kernel<kTcBF16, false>
              : kind == kTcFP8 ? tc_gemm_persistent_kernel<kTcFP8, false>
              : split          ? tc_gemm_persistent_kernel<kTcTF32, true>
                               : tc_gemm_persistent_kernel<kTcTF32, false>;
  const int variant = kind == kTcBF16 ? 0 : kind == kTcFP8 ? 1 : split ? 2 : 3;
  const size_t smem = kPRing + 1024;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.blockDim = dim3(kPThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  int grid = std::min(tiles, sms);
  if (grid_mode == kGridSmall) grid = std::min(tiles, kSmallGrid);
  if (grid_mode == kGridTiles) grid = tiles;
  if (grid_mode == kGridSpareGpc) {
    // 16-CTA clusters (one per GPC: a GPC has fewer than 32 SMs) on all GPCs
    // but one, which stays free for the kernels of the other stream
    const int gpcs = clusters16(kern, variant, smem);
    if (gpcs >= 2) {
      grid = std::min(16 * (gpcs - 1), (tiles + 15) / 16 * 16);
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = 16;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
    } else {
      grid = std::min(tiles, std::max(1, sms - kSmallGrid - 8));
    }
  }
  cfg.gridDim = dim3(grid);
  // tile columns per group: the group's B tiles (every operand copy) take
  // ~16 MB of the 129 MB L2, beside a wave's C tiles (~40 MB read and written)
  const int tiles_n = (n + kBN - 1) / kBN;
  const size_t btile = (size_t)kBN * Kp * esz * (split ? 2 : 1);
  const int group_n = (int)std::max<size_t>(1, std::min<size_t>(tiles_n, (16u << 20) / btile));
  if (ev0) cudaEventRecord(ev0, stream);
  e = cudaLaunchKernelEx(&cfg, kern, tmA, tmB, tmAlo, tmBlo, C, ldc, m, n, num_kb, group_n,
                         (const float*)amax, st);
  if (e != cudaSuccess) return e;
  if (ev1) cudaEventRecord(ev1, stream);
  if (nlaunch) *nlaunch = nl + 1;
  return cudaGetLastError();
}

}  // namespace elgb
