// Added form 2: thousands of independent, uneven-size solves A_i X_i = B_i in
// ONE persistent launch (replayed from a CUDA graph).
//
// Each CTA draws systems from an atomic ticket over a largest-first order
// (longest-processing-time scheduling) and solves each one alone:
//   * general systems: LU with partial pivoting (El::LU's blocked
//     right-looking schedule, src/lapack_like/factor/LU.cpp:104-138, with
//     lu::Panel's column steps, LU/Panel.hpp:15-59) + lu::SolveAfter;
//   * SPD systems: lower Cholesky (LowerVariant3Blocked,
//     src/lapack_like/factor/Cholesky/LowerVariant3.hpp:43-68) +
//     cholesky::SolveAfter;
// in a chosen factorization precision (FP32 or FP64), followed -- for FP32
// factors -- by refinement with an FP64 residual (Refined.hpp:44-119 rule:
// keep an update only if the backward error drops) and an FP64
// refactorization of the same system when refinement stalls.
//
// The working copy of the matrix lives in a per-CTA global workspace (it is
// L2-resident for the sizes this form targets); each nb-column panel is
// staged in shared memory, the trailing update is register-tiled FMA with
// both operands staged in shared memory.  nb is per system (autotuned per
// size bucket, capped so the panel fits in shared memory).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "../../include/elgb300.h"
#include "batched.h"
#include "driver.h"
#include "mlp_device.cuh"
#include "tcgen05.cuh"

namespace elgb {

namespace {

constexpr int kBT = 256;               // threads per CTA
constexpr int kBQ = 8;                 // max right-hand sides
constexpr int kPhases = 10;            // per-system timing slots
constexpr int kSmemPanel = 144 * 1024; // panel staging budget (bytes)
// tensor-core trailing update (FP32 / BF16 factors): operand tiles after the
// panel budget, 1024-byte aligned for the 128-byte swizzle
constexpr int kTcM = 128, kTcN = 128;             // C tile per MMA round
constexpr int kTcTileA = kTcM * 128;              // one 128-byte K row per M row
constexpr int kTcTileB = kTcN * 128;
constexpr int kTcSmem = 2 * kTcTileA + 2 * kTcTileB;  // hi and lo of each: 64 KB
constexpr int kTcCols = 256;                      // TMEM columns (2 FP32 accumulators)
constexpr int kDynSmem = kSmemPanel + kTcSmem + 1024;
static_assert(kSmemPanel >= 2 * kTcM * kTcN * 4, "C staging of the tensor-core update");

struct SysDesc {
  int n, kind, nb, prec;  // kind 0 LU, 1 Cholesky; prec 0 FP64, 1 FP32 + IR
  long a_off, b_off;      // into A (FP64, ld n) and B / X (FP64, ld n)
  int ib, pad;            // inner panel width (the shared-memory panel), <= nb
};

struct Shared {
  // per-system device time by phase (thread 0 accumulates, globaltimer ns):
  // 0 panel, 1 row swaps, 2 U12 solve, 3 trailing update, 4 LU-IR,
  // 5 FGMRES-IR, 6 FP64 path, 7 features; within 4-5: 8 FP64 residuals and
  // products, 9 low-precision triangular solves
  unsigned long long ph[kPhases];
  float feat[16];                     // the selector's features of the system
  unsigned long long mma_bar;         // tcgen05 commit barrier
  unsigned mma_phase;                 // its next parity
  unsigned tmem;                      // TMEM accumulator base
  int tc_err;                         // a tensor-core wait timed out
  float h1[64], h2[64], lg[4];        // the selector network's activations
  double red[kBT / 32][kBQ + 1];
  double colv[kBQ + 1];
  int ival[4];
  int piv[64];
  int pairs[4 * 64 + 4];
  int top[64];
  int keys[256];
  int vals[256];
  int order[64];
};

template <typename T>
__device__ __forceinline__ T tabs(T x) { return x < T(0) ? -x : x; }

// Operand rounding of the BF16 factorization: products of BF16-rounded
// operands accumulated in FP32 (what a BF16 tensor-core update computes).
__device__ __forceinline__ float rnd(float x, bool lowp) {
  return lowp ? __bfloat162float(__float2bfloat16_rn(x)) : x;
}
__device__ __forceinline__ double rnd(double x, bool) { return x; }

// ---- block reductions ------------------------------------------------------
__device__ __forceinline__ void block_argmax_abs(float& v, int& r, Shared& sh, float* fv,
                                                 int* fr) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  warp_argmax(v, r);
  __syncthreads();
  if (lane == 0) {
    fv[warp] = v;
    fr[warp] = r;
  }
  __syncthreads();
  if (warp == 0) {
    float wv = lane < kBT / 32 ? fv[lane] : -1.f;
    int wr = lane < kBT / 32 ? fr[lane] : -1;
    warp_argmax(wv, wr);
    if (lane == 0) {
      fv[8] = wv;
      fr[8] = wr;
    }
  }
  __syncthreads();
  v = fv[8];
  r = fr[8];
  (void)sh;
}

__device__ __forceinline__ void block_argmax_abs(double& v, int& r, Shared& sh, double* fv,
                                                 int* fr) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  warp_argmax(v, r);
  __syncthreads();
  if (lane == 0) {
    fv[warp] = v;
    fr[warp] = r;
  }
  __syncthreads();
  if (warp == 0) {
    double wv = lane < kBT / 32 ? fv[lane] : -1.0;
    int wr = lane < kBT / 32 ? fr[lane] : -1;
    warp_argmax(wv, wr);
    if (lane == 0) {
      fv[8] = wv;
      fr[8] = wr;
    }
  }
  __syncthreads();
  v = fv[8];
  r = fr[8];
  (void)sh;
}

// Per-column sums over `n` rows of f(row, col) for q columns: out[c].
template <typename F>
__device__ __forceinline__ void block_colsum(int n, int q, F f, Shared& sh, double* out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double acc[kBQ];
#pragma unroll
  for (int c = 0; c < kBQ; ++c) acc[c] = 0.0;
  for (int r = threadIdx.x; r < n; r += kBT)
#pragma unroll
    for (int c = 0; c < kBQ; ++c)
      if (c < q) acc[c] += f(r, c);
#pragma unroll
  for (int c = 0; c < kBQ; ++c) {
    double v = acc[c];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) sh.red[warp][c] = v;
  }
  __syncthreads();
  if (threadIdx.x < q) {
    double v = 0.0;
    for (int w = 0; w < kBT / 32; ++w) v += sh.red[w][threadIdx.x];
    out[threadIdx.x] = v;
  }
  __syncthreads();
}

// ---- LU --------------------------------------------------------------------
// (dst, src) list of the rows changed by the panel's interchanges (rows
// k + i <-> sh.piv[i], i < jb, in order): after them row dst holds what row
// src held.  Label replay by thread 0 on the top rows plus a small hash
// table of the outside rows; cnt in sh.ival[0], dst in sh.pairs[0..),
// src in sh.pairs[128..).
__device__ void cta_build_pairs(int k, int jb, Shared& sh) {
  if (threadIdx.x == 0) {
    // replay on labels (top rows + up to jb outside rows in a small table)
    int nk = 0;
    for (int i = 0; i < jb; ++i) sh.top[i] = k + i;
    for (int i = 0; i < 256; ++i) sh.keys[i] = -1;
    for (int i = 0; i < jb; ++i) {
      const int p = sh.piv[i];
      if (p < k + jb) {
        const int t = sh.top[i];
        sh.top[i] = sh.top[p - k];
        sh.top[p - k] = t;
      } else {
        int h = (int)(((unsigned)p * 2654435761u) >> 8) & 255;
        while (sh.keys[h] != -1 && sh.keys[h] != p) h = (h + 1) & 255;
        if (sh.keys[h] == p) {
          const int t = sh.vals[h];
          sh.vals[h] = sh.top[i];
          sh.top[i] = t;
        } else {
          sh.keys[h] = p;
          sh.vals[h] = sh.top[i];
          sh.top[i] = p;
          sh.order[nk++] = h;
        }
      }
    }
    int c = 0;
    for (int i = 0; i < jb; ++i)
      if (sh.top[i] != k + i) {
        sh.pairs[c] = k + i;
        sh.pairs[128 + c] = sh.top[i];
        ++c;
      }
    for (int t = 0; t < nk; ++t) {
      const int h = sh.order[t];
      if (sh.vals[h] != sh.keys[h]) {
        sh.pairs[c] = sh.keys[h];
        sh.pairs[128 + c] = sh.vals[h];
        ++c;
      }
    }
    sh.ival[0] = c;
  }
  __syncthreads();
}

// The row interchanges listed by cta_build_pairs on the columns [c_lo, c_hi).
template <typename T>
__device__ void cta_swap_cols(T* W, int ld, Shared& sh, T* stage, int stage_elems, int c_lo,
                              int c_hi) {
  const int cnt = sh.ival[0];
  if (cnt == 0 || c_hi <= c_lo) return;
  const int ncols_out = c_hi - c_lo;
  const int chunk = max(1, stage_elems / cnt);
  for (int c0 = 0; c0 < ncols_out; c0 += chunk) {
    const int cw = min(chunk, ncols_out - c0);
#pragma unroll 8
    for (int idx = threadIdx.x; idx < cw * cnt; idx += kBT) {
      const int e = idx % cnt, cc = c0 + idx / cnt;
      const int col = c_lo + cc;
      stage[idx] = W[sh.pairs[128 + e] + (long)col * ld];
    }
    __syncthreads();
#pragma unroll 8
    for (int idx = threadIdx.x; idx < cw * cnt; idx += kBT) {
      const int e = idx % cnt, cc = c0 + idx / cnt;
      const int col = c_lo + cc;
      W[sh.pairs[e] + (long)col * ld] = stage[idx];
    }
    __syncthreads();
  }
}

// C[m x nc] -= P[m x jb] * Q[jb x nc]: P in shared memory (ld = ldp), Q in
// global (ld = ldq, staged in kGC-column chunks into `qs`), C in global.
// Tiles of 128 x kGC: lane l of warp w owns rows r0 + l + 32 i (i < 4) and
// columns c0 + w + 8 j (j < kGC / 8), so a warp's C accesses are 128-byte
// rows of one column and its Q reads are shared-memory broadcasts.  The C
// tile is loaded into registers before the k loop (the loads are in flight
// during the FMAs).
template <typename T>
struct GemmShape {
  static constexpr int kGC = 64;  // FP32: 4 x 8 per thread
};
template <>
struct GemmShape<double> {
  static constexpr int kGC = 32;  // FP64: 4 x 4 per thread
};

template <typename T>
__device__ __forceinline__ void gemm_tile_load(const T* C, int ldc, int m, int cw, int r0,
                                               int lane, int w, T (&v)[4][GemmShape<T>::kGC / 8]) {
  constexpr int kTC = GemmShape<T>::kGC / 8;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = r0 + lane + 32 * i;
#pragma unroll
    for (int j = 0; j < kTC; ++j) {
      const int cc = w + 8 * j;
      v[i][j] = (r < m && cc < cw) ? C[r + (long)cc * ldc] : T(0);
    }
  }
}

template <typename T>
__device__ __noinline__ void cta_gemm_update(const T* P, int ldp, const T* Q, int ldq, T* C,
                                             int ldc, int m, int nc, int jb, T* qs, bool lowp) {
  constexpr int kGC = GemmShape<T>::kGC, kTC = kGC / 8;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int c0 = 0; c0 < nc; c0 += kGC) {
    const int cw = min(kGC, nc - c0);
    T* Cc = C + (long)c0 * ldc;
    __syncthreads();
    for (int idx = threadIdx.x; idx < jb * kGC; idx += kBT) {
      const int kk = idx % jb, cc = idx / jb;
      qs[kk + cc * jb] = cc < cw ? rnd(Q[kk + (long)(c0 + cc) * ldq], lowp) : T(0);
    }
    __syncthreads();
    // software pipeline over the 128-row tiles: the next tile's C is loaded
    // while this tile's FMAs run
    T cv[4][kTC], cn[4][kTC];
    gemm_tile_load<T>(Cc, ldc, m, cw, 0, lane, w, cv);
    for (int r0 = 0; r0 < m; r0 += 128) {
      if (r0 + 128 < m) gemm_tile_load<T>(Cc, ldc, m, cw, r0 + 128, lane, w, cn);
      T acc[4][kTC];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < kTC; ++j) acc[i][j] = T(0);
#pragma unroll 4
      for (int kk = 0; kk < jb; ++kk) {
        T a[4], b[kTC];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int r = r0 + lane + 32 * i;
          a[i] = r < m ? rnd(P[r + kk * ldp], lowp) : T(0);
        }
#pragma unroll
        for (int j = 0; j < kTC; ++j) b[j] = qs[kk + (w + 8 * j) * jb];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < kTC; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int r = r0 + lane + 32 * i;
#pragma unroll
        for (int j = 0; j < kTC; ++j) {
          const int cc = w + 8 * j;
          if (r < m && cc < cw) Cc[r + (long)cc * ldc] = cv[i][j] - acc[i][j];
          cv[i][j] = cn[i][j];
        }
      }
    }
  }
  __syncthreads();
}

// U12 := L11^{-1} U12 (L11 unit lower, jb x jb in the shared panel, ld mp),
// one thread per column with the column held in registers.
template <typename T, int JB>
__device__ __noinline__ void cta_trsm_cols(const T* L, int mp, T* W0, int ld, int n2, bool lowp) {
  for (int c = threadIdx.x; c < n2; c += kBT) {
    T* col = W0 + (long)c * ld;
    T x[JB];
#pragma unroll
    for (int i = 0; i < JB; ++i) x[i] = col[i];
#pragma unroll
    for (int i = 1; i < JB; ++i) {
      T s = x[i];
#pragma unroll
      for (int l = 0; l < i; ++l) s = fma(-rnd(L[i + l * mp], lowp), rnd(x[l], lowp), s);
      x[i] = s;
    }
#pragma unroll
    for (int i = 1; i < JB; ++i) col[i] = x[i];
  }
}

template <typename T>
__device__ void cta_trsm_u12(const T* L, int mp, T* W0, int ld, int jb, int n2, bool lowp) {
  switch (jb) {
    case 8: cta_trsm_cols<T, 8>(L, mp, W0, ld, n2, lowp); break;
    case 16: cta_trsm_cols<T, 16>(L, mp, W0, ld, n2, lowp); break;
    case 32:
      if (sizeof(T) == 4) {  // 32 doubles per thread would spill
        cta_trsm_cols<T, 32>(L, mp, W0, ld, n2, lowp);
        break;
      }
      [[fallthrough]];
    default:
      for (int c = threadIdx.x; c < n2; c += kBT) {
        T* col = W0 + (long)c * ld;
        for (int i = 1; i < jb; ++i) {
          T s = col[i];
          for (int l = 0; l < i; ++l) s = fma(-rnd(L[i + l * mp], lowp), rnd(col[l], lowp), s);
          col[i] = s;
        }
      }
  }
  __syncthreads();
}

// ---- tensor-core trailing update ----------------------------------------------
// C[m x nc] -= P[m x jb] * Q[jb x nc] on the 5th-generation tensor cores,
// inside one CTA: P is A21 and Q = U12, C = A22, all in the CTA's global
// workspace (ld ldp / ldq / ldc).  For each 128 x 128 C tile the CTA writes
// the operands into 128-byte-swizzled K-major tiles (the layout TMA's
// SWIZZLE_128B produces: 8-row groups of 1024 bytes, the 16-byte chunk c of
// row r stored at chunk c ^ (r & 7)), thread 0 issues tcgen05.mma into one of
// two 128 x 128 FP32 accumulators in TMEM and commits to an mbarrier, and all
// 8 warps read the accumulator back (tcgen05.ld, warp w owns TMEM lanes
// 32 (w % 4).. and column half w / 4) and subtract it from C, staged in
// shared memory by cp.async one tile ahead (pipeline in cta_gemm_update_tc).
//   FP32 factors: TF32 split, C -= Ahi Bhi + Ahi Blo + Alo Bhi (~FP32);
//   BF16 factors: one kind::f16 pass on BF16 operands (FP32 accumulation).
// K = jb <= 32 (TF32) or <= 64 (BF16): one 128-byte K row per operand row.
__device__ __forceinline__ int sw128(int r, int chunk) {
  return (r >> 3) * 1024 + (r & 7) * 128 + ((chunk ^ (r & 7)) << 4);
}

__device__ __forceinline__ float tf32_rna(float v) {
  uint32_t t;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(v));
  return __uint_as_float(t);
}

// 16 bytes of K for operand row r: 4 FP32 (TF32 hi / lo) or 8 BF16 values
// taken from get(k), zero past jb.
template <typename G>
__device__ __forceinline__ void tc_put_chunk(unsigned char* hi, unsigned char* lo, int r,
                                             int c, int jb, bool bf16, G get) {
  const int off = sw128(r, c);
  if (bf16) {
    __nv_bfloat162 h[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int k = 8 * c + 2 * e;
      h[e] = __floats2bfloat162_rn(k < jb ? get(k) : 0.f, k + 1 < jb ? get(k + 1) : 0.f);
    }
    *reinterpret_cast<uint4*>(hi + off) = *reinterpret_cast<uint4*>(h);
  } else {
    float4 vh, vl;
    float* ph = &vh.x;
    float* pl = &vl.x;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int k = 4 * c + e;
      const float v = k < jb ? get(k) : 0.f;
      ph[e] = tf32_rna(v);
      pl[e] = tf32_rna(v - ph[e]);
    }
    *reinterpret_cast<float4*>(hi + off) = vh;
    *reinterpret_cast<float4*>(lo + off) = vl;
  }
}

__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(tc::smem_u32(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Software-pipelined over the 128 x 128 C tiles t (row blocks outer):
//   * C(t+1) streams into a shared-memory buffer by cp.async (no registers
//     held) while tile t's epilogue runs, so ~64 KB of C is always in flight;
//   * the accumulator is double-buffered in TMEM (2 x 128 columns): the MMAs
//     of tile t+1 run while the epilogue of tile t reads tile t's columns;
//   * tile t+1's U12 values are loaded into registers before waiting for
//     tile t's MMAs and converted into the operand tile after it.
// cs: 2 x 128 x 128 floats of shared memory (the panel's staging area, free
// during the trailing update).  A thread copies and updates the same C
// elements (row 32 (w % 4) + lane, columns 64 (w / 4) + j), so its own
// cp.async.wait_group is the only wait the C buffer needs.
__device__ __noinline__ void cta_gemm_update_tc(const float* P, int ldp, const float* Q,
                                                int ldq, float* C, int ldc, int m, int nc,
                                                int jb, bool bf16, Shared& sh,
                                                unsigned char* tiles, float* cs) {
  unsigned char* sAh = tiles;
  unsigned char* sAl = tiles + kTcTileA;
  unsigned char* sBh = tiles + 2 * kTcTileA;
  unsigned char* sBl = sBh + kTcTileB;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wl = warp & 3, half = warp >> 2;
  const int kstep = bf16 ? 16 : 8;
  const int nk = (jb + kstep - 1) / kstep;     // MMAs per pass (32 bytes of K each)
  const int nchunk = bf16 ? (jb + 7) / 8 : (jb + 3) / 4;
  const int per = bf16 ? 8 : 4;                // K values per 16-byte chunk
  const uint32_t idesc = (1u << 4) | ((bf16 ? 1u : 2u) << 7) | ((bf16 ? 1u : 2u) << 10) |
                         ((uint32_t)(kTcN >> 3) << 17) | ((uint32_t)(kTcM >> 4) << 24);
  const int nct = (nc + kTcN - 1) / kTcN;
  const int T = ((m + kTcM - 1) / kTcM) * nct;
  uint32_t phase = sh.mma_phase;
  const uint32_t tmem = sh.tmem;
  constexpr int kItems = kTcN * 8 / kBT;       // (column, chunk) items per thread
  static_assert(kItems * kBT == kTcN * 8 && kTcM * 8 == kItems * kBT, "tile items");

  auto load_c = [&](int t) {  // C(t) -> cs[t & 1]; one commit group per call
    if (t < T) {
      const int r0 = (t / nct) * kTcM, c0 = (t % nct) * kTcN;
      const int row = r0 + 32 * wl + lane;
      const int cb = c0 + 64 * half;
      if (row < m) {
        float* dst = cs + (t & 1) * (kTcM * kTcN) + (64 * half) * kTcM + 32 * wl + lane;
        const float* src = C + row + (long)cb * ldc;
        const int ncol = min(64, nc - cb);
#pragma unroll 8
        for (int j = 0; j < ncol; ++j) cp_async4(dst + j * kTcM, src + (long)j * ldc);
      }
    }
    cp_async_commit();
  };
  float qv[kItems][8];
  auto fetch_b = [&](int t) {  // tile t's U12 values into registers
    const int c0 = (t % nct) * kTcN;
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
      const int idx = threadIdx.x + it * kBT;
      const int j = idx >> 3, c = idx & 7;
      const bool ok = c0 + j < nc && c < nchunk;
      const float* qc = Q + (long)(c0 + j) * ldq;
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const int k = per * c + e;
        qv[it][e] = (ok && e < per && k < jb) ? qc[k] : 0.f;
      }
    }
  };
  auto put_b = [&]() {  // qv is zero past jb and outside the tile
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
      const int idx = threadIdx.x + it * kBT;
      const int off = sw128(idx >> 3, idx & 7);
      if (bf16) {
        __nv_bfloat162 h[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) h[e] = __floats2bfloat162_rn(qv[it][2 * e], qv[it][2 * e + 1]);
        *reinterpret_cast<uint4*>(sBh + off) = *reinterpret_cast<uint4*>(h);
      } else {
        float4 vh, vl;
        float* ph = &vh.x;
        float* pl = &vl.x;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          ph[e] = tf32_rna(qv[it][e]);
          pl[e] = tf32_rna(qv[it][e] - ph[e]);
        }
        *reinterpret_cast<float4*>(sBh + off) = vh;
        *reinterpret_cast<float4*>(sBl + off) = vl;
      }
    }
  };
  auto build_a = [&](int t) {  // rows r0.. of P
    const int r0 = (t / nct) * kTcM;
    for (int idx = threadIdx.x; idx < kTcM * 8; idx += kBT) {
      const int r = idx >> 3, c = idx & 7;
      const bool ok = r0 + r < m && c < nchunk;
      const float* pr = P + r0 + r;
      tc_put_chunk(sAh, sAl, r, c, ok ? jb : 0, bf16, [&](int k) { return pr[(long)k * ldp]; });
    }
  };
  auto issue = [&](int t) {  // thread 0: tile t's MMAs into TMEM buffer t & 1
    const uint64_t ah = tc::sdesc_sw128(tc::smem_u32(sAh));
    const uint64_t al = tc::sdesc_sw128(tc::smem_u32(sAl));
    const uint64_t bh = tc::sdesc_sw128(tc::smem_u32(sBh));
    const uint64_t bl = tc::sdesc_sw128(tc::smem_u32(sBl));
    const uint32_t d = tmem + (uint32_t)((t & 1) * kTcN);
    const int passes = bf16 ? 1 : 3;
    uint32_t acc = 0;
    for (int ps = 0; ps < passes; ++ps) {
      const uint64_t ad = ps == 2 ? al : ah;
      const uint64_t bd = ps == 1 ? bl : bh;
      for (int kk = 0; kk < nk; ++kk) {
        if (bf16)
          tc::umma<kTcBF16>(d, ad + 2 * kk, bd + 2 * kk, idesc, acc);
        else
          tc::umma<kTcTF32>(d, ad + 2 * kk, bd + 2 * kk, idesc, acc);
        acc = 1;
      }
    }
    tc::umma_commit(reinterpret_cast<uint64_t*>(&sh.mma_bar));
  };

  __syncthreads();  // the callers' use of cs and the operand tiles is over
  if (sh.tc_err || T == 0) {
    __syncthreads();
    return;
  }
  load_c(0);
  fetch_b(0);
  build_a(0);
  put_b();
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  if (threadIdx.x == 0) issue(0);
  for (int t = 0; t < T; ++t) {
    load_c(t + 1);
    const bool more = t + 1 < T;
    if (more) fetch_b(t + 1);
    // tile t's MMAs done: its TMEM buffer is final and the operand tiles free
    bool ok = tc::mbar_try_wait(reinterpret_cast<uint64_t*>(&sh.mma_bar), phase);
    if (!__all_sync(0xffffffffu, ok)) {
      const unsigned long long t0 = globaltimer_ns();
      while (true) {
        ok = tc::mbar_try_wait(reinterpret_cast<uint64_t*>(&sh.mma_bar), phase);
        if (__all_sync(0xffffffffu, ok)) break;
        if (globaltimer_ns() - t0 > kSpinLimitNs) {
          if (lane == 0) sh.tc_err = 1;
          break;
        }
      }
    }
    phase ^= 1u;
    tc::tc_fence_after();
    if (more) {
      if ((t + 1) % nct == 0) build_a(t + 1);
      put_b();
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    cp_async_wait<1>();  // this thread's copies of C(t) have landed
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const bool err = sh.tc_err != 0;  // uniform: written only before the barrier
    if (!err) {
      if (more && threadIdx.x == 0) issue(t + 1);
      const int r0 = (t / nct) * kTcM, c0 = (t % nct) * kTcN;
      const int row = r0 + 32 * wl + lane;
      const int cb = c0 + 64 * half;
      const float* src = cs + (t & 1) * (kTcM * kTcN) + (64 * half) * kTcM + 32 * wl + lane;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        uint32_t a[32];
        tc::tmem_ld32(tmem + ((uint32_t)(32 * wl) << 16) +
                          (uint32_t)((t & 1) * kTcN + 64 * half + 32 * h),
                      a);
        if (row < m) {
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int col = cb + 32 * h + j;
            if (col < nc)
              C[row + (long)col * ldc] = src[(32 * h + j) * kTcM] - __uint_as_float(a[j]);
          }
        }
      }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (err) break;
  }
  cp_async_wait<0>();
  if (threadIdx.x == 0) sh.mma_phase = phase;
  __syncthreads();
}

// In-CTA LU with partial pivoting of the n x n matrix W (ld), blocked by nb.
// piv_out[0..n) receives the swap destinations; returns info (0 ok, j+1 at
// the first zero pivot).
template <typename T>
__device__ __noinline__ int cta_lu(T* W, int n, int ld, int nb, int ib, int* piv_out, Shared& sh,
                                   T* smem, int smem_elems, bool lowp,
                                   unsigned char* tc_tiles) {
  __shared__ T fv[9];
  __shared__ int fr[9];
  int info = 0;
  unsigned long long t0 = threadIdx.x == 0 ? globaltimer_ns() : 0ull;
  auto phase = [&](int i) {  // closes phase i (after a block barrier)
    if (threadIdx.x == 0) {
      const unsigned long long t = globaltimer_ns();
      sh.ph[i] += t - t0;
      t0 = t;
    }
  };
  // Two levels when the shared-memory panel is narrower than the block:
  // sub-panels of ib columns are factored in shared memory and update only
  // the rest of their nb-column block; the block then updates the trailing
  // matrix once with K = nb (half the trailing traffic of K = ib).
  ib = max(1, min(ib, nb));
  const bool one_level = ib == nb;
  for (int k = 0; k < n; k += nb) {
    const int nbk = min(nb, n - k);
    T* panel = smem;
    int mp = n - k, jb = nbk;
    for (int ks = k; ks < k + nbk; ks += ib) {
      jb = min(ib, k + nbk - ks);
      mp = n - ks;
      panel = smem;  // mp x jb, ld mp
      for (int idx = threadIdx.x; idx < mp * jb; idx += kBT) {
        const int r = idx % mp, c = idx / mp;
        panel[idx] = W[(ks + r) + (long)(ks + c) * ld];
      }
      __syncthreads();
      for (int j = 0; j < jb; ++j) {
        T bv = T(-1);
        int br = -1;
        for (int r = j + threadIdx.x; r < mp; r += kBT) {
          const T v = tabs(panel[r + j * mp]);
          if (argmax_better(v, r, bv, br)) {
            bv = v;
            br = r;
          }
        }
        block_argmax_abs(bv, br, sh, fv, fr);
        const int p = br < 0 ? j : br;
        if (threadIdx.x == 0) sh.piv[j] = ks + p;
        if (p != j)
          for (int c = threadIdx.x; c < jb; c += kBT) {
            const T t = panel[j + c * mp];
            panel[j + c * mp] = panel[p + c * mp];
            panel[p + c * mp] = t;
          }
        __syncthreads();
        const T alpha = panel[j + j * mp];
        if (alpha == T(0)) {
          if (info == 0) info = ks + j + 1;
        } else {
          const T inv = T(1) / alpha;
          for (int r = j + 1 + threadIdx.x; r < mp; r += kBT) {
            const T l = panel[r + j * mp] * inv;
            panel[r + j * mp] = l;
            const T lr = rnd(l, lowp);
            // columns in groups of eight: the loads issued together, then the
            // fmas and stores (same arithmetic, one latency per group)
            int c = j + 1;
            for (; c + 7 < jb; c += 8) {
              T u[8], v[8];
#pragma unroll
              for (int e = 0; e < 8; ++e) {
                u[e] = panel[j + (c + e) * mp];
                v[e] = panel[r + (c + e) * mp];
              }
#pragma unroll
              for (int e = 0; e < 8; ++e) panel[r + (c + e) * mp] = fma(-lr, rnd(u[e], lowp), v[e]);
            }
            for (; c < jb; ++c)
              panel[r + c * mp] = fma(-lr, rnd(panel[j + c * mp], lowp), panel[r + c * mp]);
          }
        }
        __syncthreads();
      }
      for (int idx = threadIdx.x; idx < mp * jb; idx += kBT) {
        const int r = idx % mp, c = idx / mp;
        W[(ks + r) + (long)(ks + c) * ld] = panel[idx];
      }
      for (int j = threadIdx.x; j < jb; j += kBT) piv_out[ks + j] = sh.piv[j];
      __syncthreads();
      phase(0);
      const int nin = k + nbk - ks - jb;  // block columns right of the sub-panel
      if (!one_level) {
        // the sub-panel's interchanges on the rest of its block (left and
        // right of it), so the block's L and U12 are consistently permuted
        cta_build_pairs(ks, jb, sh);
        cta_swap_cols(W, ld, sh, smem + mp * jb, smem_elems - mp * jb, k, ks);
        cta_swap_cols(W, ld, sh, smem + mp * jb, smem_elems - mp * jb, ks + jb, k + nbk);
        phase(1);
      }
      if (nin > 0) {
        cta_trsm_u12<T>(panel, mp, W + ks + (long)(ks + jb) * ld, ld, jb, nin, lowp);
        phase(2);
        cta_gemm_update<T>(panel + jb, mp, W + ks + (long)(ks + jb) * ld, ld,
                           W + (ks + jb) + (long)(ks + jb) * ld, ld, mp - jb, nin, jb,
                           smem + mp * jb, lowp);
        phase(3);
      }
    }
    // the block's interchanges on the trailing columns, U12, A22 update
    const int n2 = n - k - nbk;
    if (n2 > 0) {
      T* stage = one_level ? smem + mp * jb : smem;
      const int stage_elems = one_level ? smem_elems - mp * jb : smem_elems;
      if (!one_level) {
        for (int j = threadIdx.x; j < nbk; j += kBT) sh.piv[j] = piv_out[k + j];
        __syncthreads();
      }
      // right of the block at once; left of it deferred to the end
      cta_build_pairs(k, nbk, sh);
      cta_swap_cols(W, ld, sh, stage, stage_elems, k + nbk, n);
      phase(1);
      // one level: L11 and A21 still in the shared panel; two: from W
      const T* L11 = one_level ? panel : W + k + (long)k * ld;
      const int ldl = one_level ? mp : ld;
      const T* A21 = one_level ? panel + nbk : W + (k + nbk) + (long)k * ld;
      cta_trsm_u12<T>(L11, ldl, W + k + (long)(k + nbk) * ld, ld, nbk, n2, lowp);
      phase(2);
      bool done_tc = false;
      if constexpr (sizeof(T) == 4) {
        if (tc_tiles && n2 >= 32 && nbk <= (lowp ? 64 : 32)) {
          // A21 from W (written back with the panel): the panel's shared
          // memory stages C
          cta_gemm_update_tc(W + (k + nbk) + (long)k * ld, ld, W + k + (long)(k + nbk) * ld, ld,
                             W + (k + nbk) + (long)(k + nbk) * ld, ld, n2, n2, nbk, lowp, sh,
                             tc_tiles, reinterpret_cast<float*>(smem));
          done_tc = true;
        }
      }
      if (!done_tc)
        cta_gemm_update<T>(A21, ldl, W + k + (long)(k + nbk) * ld, ld,
                           W + (k + nbk) + (long)(k + nbk) * ld, ld, n2, n2, nbk,
                           stage, lowp);
    }
    __syncthreads();
    phase(3);
  }
  // Left columns: each block column b = [kb, kb + jbb) takes the
  // interchanges of every later panel, composed into one row relabelling
  // lab (rows >= kb + jbb; the content of row i comes from row lab[i]) and
  // applied as a gather through shared memory -- coalesced reads and writes
  // instead of per-panel scattered row swaps.  lab is built from the last
  // panel backwards: lab <- lambda_b o lab, lambda_b the relabelling of
  // panel b's own interchanges.
  {
    int* lab = reinterpret_cast<int*>(smem);
    int* pmap = lab + n;
    T* buf = reinterpret_cast<T*>(pmap + n);  // 2n ints: 8-byte aligned
    const int cap = (int)((smem_elems * (long)sizeof(T) - 2 * (long)n * sizeof(int)) /
                          (long)sizeof(T));
    for (int i = threadIdx.x; i < n; i += kBT) {
      lab[i] = i;
      pmap[i] = -1;
    }
    __syncthreads();
    for (int kb = ((n - 1) / nb) * nb; kb >= 0; kb -= nb) {
      const int jbb = min(nb, n - kb), kn = kb + jbb, rows = n - kn;
      if (rows > 0 && kb < kn) {
        const int cw_max = max(1, min(jbb, cap / rows));
        for (int c0 = kb; c0 < kn; c0 += cw_max) {
          const int cw = min(cw_max, kn - c0);
          for (int idx = threadIdx.x; idx < cw * rows; idx += kBT) {
            const int i = idx % rows, c = idx / rows;
            buf[idx] = W[(kn + i) + (long)(c0 + c) * ld];
          }
          __syncthreads();
          for (int idx = threadIdx.x; idx < cw * rows; idx += kBT) {
            const int i = idx % rows, c = idx / rows;
            const int src = lab[kn + i] - kn;
            if (src != i) W[(kn + i) + (long)(c0 + c) * ld] = buf[src + c * rows];
          }
          __syncthreads();
        }
      }
      // fold panel b's interchanges into lab
      for (int j = threadIdx.x; j < jbb; j += kBT) sh.piv[j] = piv_out[kb + j];
      __syncthreads();
      cta_build_pairs(kb, jbb, sh);
      const int cnt = sh.ival[0];
      for (int e = threadIdx.x; e < cnt; e += kBT) pmap[sh.pairs[e]] = e;
      __syncthreads();
      for (int i = threadIdx.x; i < n; i += kBT) {
        const int x = lab[i];
        const int e = pmap[x];
        if (e >= 0) lab[i] = sh.pairs[128 + e];
      }
      __syncthreads();
      for (int e = threadIdx.x; e < cnt; e += kBT) pmap[sh.pairs[e]] = -1;
      __syncthreads();
    }
  }
  phase(1);
  return info;
}

// In-CTA lower Cholesky of W; returns info (j+1 at the first non-positive pivot).
template <typename T>
__device__ __noinline__ int cta_chol(T* W, int n, int ld, int nb, T* smem, bool lowp) {
  __shared__ int s_bad;
  if (threadIdx.x == 0) s_bad = 0;
  __syncthreads();
  for (int k = 0; k < n; k += nb) {
    const int jb = min(nb, n - k);
    const int mp = n - k;
    T* panel = smem;  // mp x jb
    for (int idx = threadIdx.x; idx < mp * jb; idx += kBT) {
      const int r = idx % mp, c = idx / mp;
      panel[idx] = W[(k + r) + (long)(k + c) * ld];
    }
    __syncthreads();
    for (int j = 0; j < jb; ++j) {
      const T a = panel[j + j * mp];
      if (!(a > T(0))) {
        if (threadIdx.x == 0 && s_bad == 0) s_bad = k + j + 1;
        __syncthreads();
        return s_bad;
      }
      const T d = sqrt(a);
      const T inv = T(1) / d;
      __syncthreads();
      if (threadIdx.x == 0) panel[j + j * mp] = d;
      for (int r = j + 1 + threadIdx.x; r < mp; r += kBT) panel[r + j * mp] *= inv;
      __syncthreads();
      // rank-1 update of the panel's trailing columns (rows >= column)
      for (int r = j + 1 + threadIdx.x; r < mp; r += kBT) {
        const T l = rnd(panel[r + j * mp], lowp);
        for (int c = j + 1; c < jb && c <= r; ++c)
          panel[r + c * mp] = fma(-l, rnd(panel[c + j * mp], lowp), panel[r + c * mp]);
      }
      __syncthreads();
    }
    for (int idx = threadIdx.x; idx < mp * jb; idx += kBT) {
      const int r = idx % mp, c = idx / mp;
      if (r >= c) W[(k + r) + (long)(k + c) * ld] = panel[idx];
    }
    __syncthreads();
    const int n2 = n - k - jb;
    if (n2 > 0) {
      // A22 -= A21 A21^T on the lower triangle; A21 = panel rows jb.., its
      // transpose read from the panel as Q(kk, c) = panel[jb + c + kk*mp]
      T* qs = smem + mp * jb;
      const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
      for (int c0 = 0; c0 < n2; c0 += 64) {
        const int cw = min(64, n2 - c0);
        for (int r0 = c0 - (c0 % 64); r0 < n2; r0 += 64) {
          if (r0 + 63 < c0) continue;
          T acc[4][4];
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) acc[i][jj] = T(0);
          for (int kk = 0; kk < jb; ++kk) {
            T av[4], bv[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              const int r = r0 + tx + 16 * i;
              av[i] = r < n2 ? rnd(panel[jb + r + kk * mp], lowp) : T(0);
            }
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) {
              const int cc = c0 + ty + 16 * jj;
              bv[jj] = cc < n2 ? rnd(panel[jb + cc + kk * mp], lowp) : T(0);
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
              for (int jj = 0; jj < 4; ++jj) acc[i][jj] = fma(av[i], bv[jj], acc[i][jj]);
          }
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int r = r0 + tx + 16 * i;
            if (r >= n2) continue;
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) {
              const int cc = c0 + ty + 16 * jj;
              if (cc >= c0 + cw || cc > r) continue;
              W[(k + jb + r) + (long)(k + jb + cc) * ld] -= acc[i][jj];
            }
          }
        }
      }
      (void)qs;
    }
    __syncthreads();
  }
  return 0;
}

// Explicit permutation of an LU's swap sequence into perm (thread 0, the
// labels staged in shared memory when they fit).
__device__ void cta_perm_from_swaps(const int* piv, int n, int* perm, int* lab_smem, int cap) {
  int* lab = n <= cap ? lab_smem : perm;
  for (int i = threadIdx.x; i < n; i += kBT) lab[i] = i;
  __syncthreads();
  if (threadIdx.x == 0)
    for (int i = 0; i < n; ++i) {
      const int pv = piv[i];
      if (pv != i) {
        const int t = lab[i];
        lab[i] = lab[pv];
        lab[pv] = t;
      }
    }
  __syncthreads();
  if (lab != perm)
    for (int i = threadIdx.x; i < n; i += kBT) perm[i] = lab[i];
  __syncthreads();
}

// x[r, c] -= sum_{jj < jb} W[r, j0 + jj] x[j0 + jj, c] for rows r in
// [r_lo, r_hi): eight rows per thread at a time, so every jj step has eight
// independent coalesced loads of W in flight.
template <int RG, typename S, typename T>
__device__ __forceinline__ void cta_solve_rows_g(const S* W, int ld, T* x, int n, int q, int j0,
                                                 int jb, int r_lo, int r_hi) {
  const int rows = r_hi - r_lo;
  if (rows <= 0) return;
  for (int c = 0; c < q; ++c) {
    T* xc = x + (long)c * n;
    const T* xb = xc + j0;
    for (int b0 = 0; b0 < rows; b0 += RG * kBT) {
      T acc[RG];
      int rr[RG];
#pragma unroll
      for (int g = 0; g < RG; ++g) {
        const int i = b0 + threadIdx.x + g * kBT;
        rr[g] = r_lo + (i < rows ? i : rows - 1);  // clamped: loads stay in bounds
        acc[g] = T(0);
      }
      // U columns' W and x values loaded together, then the fmas in the
      // same order (loads left between the fmas would each wait a round trip)
      constexpr int U = RG >= 4 ? 4 : 16 / RG;
      for (int jj0 = 0; jj0 < jb; jj0 += U) {
        S wv[U][RG];
        T xv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int jc = min(jj0 + u, jb - 1);
          const S* wc = W + (long)(j0 + jc) * ld;
#pragma unroll
          for (int g = 0; g < RG; ++g) wv[u][g] = wc[rr[g]];
          xv[u] = xb[jc];
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
          if (jj0 + u < jb) {
#pragma unroll
            for (int g = 0; g < RG; ++g) acc[g] = fma(-(T)wv[u][g], xv[u], acc[g]);
          }
      }
#pragma unroll
      for (int g = 0; g < RG; ++g) {
        const int i = b0 + threadIdx.x + g * kBT;
        if (i < rows) xc[r_lo + i] += acc[g];
      }
    }
  }
}

// RG matched to the row count: no idle duplicate loads on short columns.
template <typename S, typename T>
__device__ __forceinline__ void cta_solve_rows(const S* W, int ld, T* x, int n, int q, int j0,
                                               int jb, int r_lo, int r_hi) {
  const int rows = r_hi - r_lo;
  if (rows <= kBT)
    cta_solve_rows_g<1>(W, ld, x, n, q, j0, jb, r_lo, r_hi);
  else if (rows <= 2 * kBT)
    cta_solve_rows_g<2>(W, ld, x, n, q, j0, jb, r_lo, r_hi);
  else if (rows <= 4 * kBT)
    cta_solve_rows_g<4>(W, ld, x, n, q, j0, jb, r_lo, r_hi);
  else
    cta_solve_rows_g<8>(W, ld, x, n, q, j0, jb, r_lo, r_hi);
}

// x := U^{-1} L^{-1} x for n x q x (ld n): L lower (unit or not), U upper
// (non-unit) both in W (for Cholesky U = L^T has been written to the upper
// triangle).  Factors stored as S, arithmetic in T (T = double with S =
// float applies FP32 factors exactly, as a fixed FP64 operator).  Each
// 32 x 32 diagonal block is first staged in shared memory by all threads,
// then solved by one warp per column in registers; the rows after (before)
// the block are updated by all threads.
template <typename S, typename T>
__device__ __noinline__ void cta_solve(const S* W, int n, int ld, bool unit_lower, T* x, int q) {
  // the 32 x 32 diagonal block, staged at the start of the dynamic shared
  // memory (the panel region, unused once a factorization is done)
  extern __shared__ __align__(16) unsigned char smem_dyn[];
  T(*sdg)[33] = reinterpret_cast<T(*)[33]>(smem_dyn);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  auto stage = [&](int j0, int jb) {
    __syncthreads();  // the previous block's readers are done
    for (int idx = threadIdx.x; idx < 32 * 32; idx += kBT) {
      const int r = idx & 31, c = idx >> 5;
      sdg[r][c] = (r < jb && c < jb) ? (T)W[(j0 + r) + (long)(j0 + c) * ld] : T(0);
    }
    __syncthreads();
  };
  for (int j0 = 0; j0 < n; j0 += 32) {
    const int jb = min(32, n - j0);
    stage(j0, jb);
    if (warp < q) {
      T* xc = x + (long)warp * n;
      T v = lane < jb ? xc[j0 + lane] : T(0);
      for (int jj = 0; jj < jb; ++jj) {
        if (!unit_lower && lane == jj) v = v / sdg[jj][jj];
        const T xj = __shfl_sync(0xffffffffu, v, jj);
        if (lane > jj && lane < jb) v = fma(-sdg[lane][jj], xj, v);
      }
      if (lane < jb) xc[j0 + lane] = v;
    }
    __syncthreads();
    cta_solve_rows(W, ld, x, n, q, j0, jb, j0 + jb, n);
    __syncthreads();
  }
  for (int j0 = ((n - 1) / 32) * 32; j0 >= 0; j0 -= 32) {
    const int jb = min(32, n - j0);
    stage(j0, jb);
    if (warp < q) {
      T* xc = x + (long)warp * n;
      T v = lane < jb ? xc[j0 + lane] : T(0);
      for (int jj = jb - 1; jj >= 0; --jj) {
        if (lane == jj) v = v / sdg[jj][jj];
        const T xj = __shfl_sync(0xffffffffu, v, jj);
        if (lane < jj) v = fma(-sdg[lane][jj], xj, v);
      }
      if (lane < jb) xc[j0 + lane] = v;
    }
    __syncthreads();
    cta_solve_rows(W, ld, x, n, q, j0, jb, 0, j0);
    __syncthreads();
  }
}

// Cholesky: mirror L into the upper triangle (U = L^T) for the solves.
template <typename T>
__device__ void cta_mirror_lower(T* W, int n, int ld) {
  for (long idx = threadIdx.x; idx < (long)n * n; idx += kBT) {
    const int r = (int)(idx % n), c = (int)(idx / n);
    if (r < c) W[r + (long)c * ld] = W[c + (long)r * ld];
  }
  __syncthreads();
}

// x (FP64 in, the solution out) through the factors of precision T:
// scaled per column into the FP32/FP64 vector xt, permuted, solved, and
// added back (accumulate) or stored.
template <typename T>
__device__ void cta_apply_inverse(const T* W, int n, int kind, const int* perm, const double* rhs,
                                  double* x, T* xt, T* tmp, int q, bool accumulate,
                                  double* scale) {
  __syncthreads();
  {  // per-column max |rhs| (one warp per column)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int c = warp; c < q; c += kBT / 32) {
      double m = 0.0;
      for (int r = lane; r < n; r += 32) m = fmax(m, fabs(rhs[r + (long)c * n]));
      for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
      if (lane == 0) scale[c] = (m > 0 && m < INFINITY) ? m : 1.0;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n * q; i += kBT) {
    const int r = i % n, c = i / n;
    const int src = kind == 0 ? perm[r] : r;
    xt[i] = (T)(rhs[src + (long)c * n] / scale[c]);
  }
  __syncthreads();
  cta_solve<T, T>(W, n, n, kind == 0, xt, q);
  for (int i = threadIdx.x; i < n * q; i += kBT) {
    const double v = (double)xt[i] * scale[i / n];
    x[i] = accumulate ? x[i] + v : v;
  }
  __syncthreads();
  (void)tmp;
}

struct BatchParams {
  const SysDesc* desc;
  const int* order;
  int count, q;
  const double* A;
  const double* B;
  double* X;
  void* wsf;   // per-CTA FP32 workspace (ld = n)
  double* wsd; // per-CTA FP64 workspace
  long ws_elems;     // elements per CTA in each workspace
  int* pivws;        // per CTA, 2 n_max ints (swap destinations, permutation)
  double* vec;       // per CTA: r, x_prev, solve vector (3 x n_max x q doubles)
  int nmax;
  double tol;
  int max_iters;
  unsigned* ticket;
  BatchResult* out;
  int mode;          // 0 solve, 1 features only, 2 features -> selector -> solve
  int fallback;      // FP64 refactorization when refinement does not converge
  float* feat;       // mode 1: count x 16 features
  int method;        // 0 LU-IR then FGMRES-IR on stall, 1 LU-IR only, 2 FGMRES-IR only
  int kry_m;         // FGMRES restart length (<= kKryMax)
  int kry_max;       // FGMRES inner iterations per right-hand side
  double* kry;       // per CTA: (2 kry_m + 2) x n_max doubles (V, Z, scratch)
  const int* prec_dev;  // per-system precision read at run time (or null)
  unsigned long long* phase_ns;  // count x kPhases phase times (or null)
  const float* mlp;  // mode 2: the selector network's parameters
  int tc;            // 1: FP32 / BF16 trailing updates on the tensor cores
  int* err;          // set when a tensor-core wait timed out
};

// Y = B - A X (B != null) or Y = A X (B == null) for the n x q block X (all
// ld n), FP64.  Thread t owns rows t + kBT g (g < RG) of each 8-row-group
// sweep, so every j step has RG independent coalesced loads of A in flight
// (the product is latency-bound otherwise: one SM, 8 warps).
template <int RG, int QM, int U>
__device__ void cta_gemv_rows(const double* __restrict__ A, int n, const double* X, int q,
                              const double* B, double* Y) {
  for (int r0 = 0; r0 < n; r0 += RG * kBT) {
    double acc[RG][QM];
#pragma unroll
    for (int g = 0; g < RG; ++g)
#pragma unroll
      for (int c = 0; c < QM; ++c) acc[g][c] = 0.0;
    int rr[RG];
#pragma unroll
    for (int g = 0; g < RG; ++g) {
      const int r = r0 + threadIdx.x + g * kBT;
      rr[g] = r < n ? r : n - 1;  // clamped: loads stay in bounds, results unused
    }
    // U columns' loads issued together: RG * U independent coalesced loads
    // in flight per thread (one CTA per SM is latency-bound otherwise)
    for (int j0 = 0; j0 < n; j0 += U) {
      // the block's A and x values all loaded before any fma (x loads placed
      // after the fmas would each wait a full round trip)
      double a[U][RG], x[U][QM];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int jj = min(j0 + u, n - 1);
        const long col = (long)jj * n;
#pragma unroll
        for (int g = 0; g < RG; ++g) a[u][g] = A[rr[g] + col];
#pragma unroll
        for (int c = 0; c < QM; ++c) x[u][c] = c < q ? X[jj + (long)c * n] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (j0 + u < n) {
#pragma unroll
          for (int g = 0; g < RG; ++g)
#pragma unroll
            for (int c = 0; c < QM; ++c) acc[g][c] = fma(a[u][g], x[u][c], acc[g][c]);
        }
      }
    }
#pragma unroll
    for (int g = 0; g < RG; ++g) {
      const int r = r0 + threadIdx.x + g * kBT;
      if (r >= n) continue;
#pragma unroll
      for (int c = 0; c < QM; ++c)
        if (c < q) Y[r + (long)c * n] = B ? B[r + (long)c * n] - acc[g][c] : acc[g][c];
    }
  }
}

__device__ __noinline__ void cta_gemv(const double* A, int n, const double* X, int q,
                                      const double* B, double* Y) {
  // row groups matched to n (no clamped duplicate rows), the rest of the
  // loads in flight taken from more columns
  if (q == 1) {
    if (n <= kBT) cta_gemv_rows<1, 1, 16>(A, n, X, q, B, Y);
    else if (n <= 2 * kBT) cta_gemv_rows<2, 1, 8>(A, n, X, q, B, Y);
    else if (n <= 4 * kBT) cta_gemv_rows<4, 1, 8>(A, n, X, q, B, Y);
    else cta_gemv_rows<8, 1, 4>(A, n, X, q, B, Y);
  } else if (q == 2) {
    if (n <= kBT) cta_gemv_rows<1, 2, 16>(A, n, X, q, B, Y);
    else if (n <= 2 * kBT) cta_gemv_rows<2, 2, 8>(A, n, X, q, B, Y);
    else if (n <= 4 * kBT) cta_gemv_rows<4, 2, 4>(A, n, X, q, B, Y);
    else cta_gemv_rows<8, 2, 4>(A, n, X, q, B, Y);
  } else if (q <= 4) {
    if (n <= kBT) cta_gemv_rows<1, 4, 8>(A, n, X, q, B, Y);
    else if (n <= 2 * kBT) cta_gemv_rows<2, 4, 8>(A, n, X, q, B, Y);
    else cta_gemv_rows<4, 4, 4>(A, n, X, q, B, Y);
  } else {
    if (n <= kBT) cta_gemv_rows<1, kBQ, 4>(A, n, X, q, B, Y);
    else if (n <= 2 * kBT) cta_gemv_rows<2, kBQ, 4>(A, n, X, q, B, Y);
    else cta_gemv_rows<4, kBQ, 2>(A, n, X, q, B, Y);
  }
  __syncthreads();
}

__device__ double sys_berr(const double* A, int n, const double* X, const double* B, double* R,
                           int q, Shared& sh, double nA) {
  // R = B - A X (FP64), berr = max_c ||R_c|| / (nA ||X_c|| + ||B_c||)
  cta_gemv(A, n, X, q, B, R);
  double nr[kBQ], nx[kBQ], nb[kBQ];
  __shared__ double s_n[3][kBQ];
  block_colsum(n, q, [&](int r, int c) { const double v = R[r + (long)c * n]; return v * v; }, sh,
               s_n[0]);
  block_colsum(n, q, [&](int r, int c) { const double v = X[r + (long)c * n]; return v * v; }, sh,
               s_n[1]);
  block_colsum(n, q, [&](int r, int c) { const double v = B[r + (long)c * n]; return v * v; }, sh,
               s_n[2]);
  double worst = 0.0;
  for (int c = 0; c < q; ++c) {
    nr[c] = sqrt(s_n[0][c]);
    nx[c] = sqrt(s_n[1][c]);
    nb[c] = sqrt(s_n[2][c]);
    const double den = nA * nx[c] + nb[c];
    const double v = den > 0 ? nr[c] / den : (nr[c] > 0 ? INFINITY : 0.0);
    worst = (v > worst || v != v) ? v : worst;
  }
  __syncthreads();
  return worst;
}

// x := (L U)^{-T} x for one vector: U^T (lower, diag u_jj) forward, then
// L^T (upper; unit diagonal for LU, l_jj for Cholesky) backward, both read
// transposed from W.  Each 32 x 32 diagonal block is staged in shared memory
// (the panel region) before one warp solves it in registers; the other rows
// take the block's update with the block's 32 loads of their column segment
// issued together.
template <typename T>
__device__ void cta_solve_t(const T* W, int n, int ld, bool unit_lower, T* x) {
  extern __shared__ __align__(16) unsigned char smem_dyn[];
  T(*sdg)[33] = reinterpret_cast<T(*)[33]>(smem_dyn);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  auto stage = [&](int j0, int jb) {
    __syncthreads();  // the previous block's readers are done
    for (int idx = threadIdx.x; idx < 32 * 32; idx += kBT) {
      const int r = idx & 31, c = idx >> 5;
      sdg[r][c] = (r < jb && c < jb) ? W[(j0 + r) + (long)(j0 + c) * ld] : T(0);
    }
    __syncthreads();
  };
  // x[r] -= sum_jj W[j0 + jj, r] x[j0 + jj] for r in [r_lo, r_hi)
  auto update = [&](int j0, int jb, int r_lo, int r_hi) {
    for (int r = r_lo + threadIdx.x; r < r_hi; r += kBT) {
      const T* wr = W + j0 + (long)r * ld;
      T acc = x[r];
      if (jb == 32) {
        T w[32];
#pragma unroll
        for (int jj = 0; jj < 32; ++jj) w[jj] = wr[jj];
#pragma unroll
        for (int jj = 0; jj < 32; ++jj) acc = fma(-w[jj], x[j0 + jj], acc);
      } else {
        for (int jj = 0; jj < jb; ++jj) acc = fma(-wr[jj], x[j0 + jj], acc);
      }
      x[r] = acc;
    }
  };
  for (int j0 = 0; j0 < n; j0 += 32) {
    const int jb = min(32, n - j0);
    stage(j0, jb);
    if (warp == 0) {
      T v = lane < jb ? x[j0 + lane] : T(0);
      for (int jj = 0; jj < jb; ++jj) {
        if (lane == jj) v = v / sdg[jj][jj];
        const T xj = __shfl_sync(0xffffffffu, v, jj);
        if (lane > jj && lane < jb) v = fma(-sdg[jj][lane], xj, v);
      }
      if (lane < jb) x[j0 + lane] = v;
    }
    __syncthreads();
    update(j0, jb, j0 + jb, n);
  }
  for (int j0 = ((n - 1) / 32) * 32; j0 >= 0; j0 -= 32) {
    const int jb = min(32, n - j0);
    stage(j0, jb);
    if (warp == 0) {
      T v = lane < jb ? x[j0 + lane] : T(0);
      for (int jj = jb - 1; jj >= 0; --jj) {
        if (!unit_lower && lane == jj) v = v / sdg[jj][jj];
        const T xj = __shfl_sync(0xffffffffu, v, jj);
        if (lane < jj) v = fma(-sdg[jj][lane], xj, v);
      }
      if (lane < jb) x[j0 + lane] = v;
    }
    __syncthreads();
    update(j0, jb, 0, j0);
  }
  __syncthreads();
}

// Block-wide sum and max of f(i), i < n (double).
template <typename F>
__device__ void block_sum_max(int n, F f, Shared& sh, double* out_sum, double* out_max) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double sm = 0.0, mx = 0.0;
  for (int i = threadIdx.x; i < n; i += kBT) {
    const double v = f(i);
    sm += v;
    mx = fmax(mx, v);
  }
  for (int o = 16; o > 0; o >>= 1) {
    sm += __shfl_xor_sync(0xffffffffu, sm, o);
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  if (lane == 0) {
    sh.red[warp][0] = sm;
    sh.red[warp][1] = mx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < kBT / 32; ++w) {
      a += sh.red[w][0];
      b = fmax(b, sh.red[w][1]);
    }
    sh.colv[0] = a;
    sh.colv[1] = b;
  }
  __syncthreads();
  *out_sum = sh.colv[0];
  *out_max = sh.colv[1];
  __syncthreads();
}

// ---- FGMRES-IR ------------------------------------------------------------
// Flexible right-preconditioned restarted GMRES on A x = b in FP64, the
// preconditioner being the low-precision factors (El's FGMRES,
// include/El/lapack_like/solve/FGMRES.hpp:37-290: z_j = M^{-1} v_j kept,
// w = A z_j, Givens-updated least squares, x = x0 + Z y, explicit residual
// at every restart).  The orthogonalization is classical Gram-Schmidt
// applied twice (each pass one warp per basis vector) instead of the
// reference's modified Gram-Schmidt: same subspace, fewer block barriers.
constexpr int kKryMax = 32;

struct KryShared {
  double H[kKryMax + 1][kKryMax];
  double cs[kKryMax], sn[kKryMax], g[kKryMax + 1], y[kKryMax], h[kKryMax + 1];
  int stop;
};

// h[i] = <w, V_i>, i < cnt (one warp per basis vector).
__device__ void cta_multi_dot(const double* Vk, long ldv, int cnt, const double* w, int n,
                              double* h) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = warp; i < cnt; i += kBT / 32) {
    const double* v = Vk + (long)i * ldv;
    double acc = 0.0;
    for (int r = lane; r < n; r += 32) acc = fma(w[r], v[r], acc);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) h[i] = acc;
  }
  __syncthreads();
}

// y = A v (FP64), one thread per row.
__device__ void cta_matvec(const double* A, int n, const double* v, double* y) {
  cta_gemv(A, n, v, 1, nullptr, y);
}

// z = M^{-1} v with the low-precision factors applied in FP64 arithmetic:
// M = L U exactly (a fixed linear operator), the GMRES-IR preconditioner of
// Carson and Higham (the factors' precision limits M's quality, not the
// solve's rounding).  z may alias nothing else; perm maps rows for LU.
template <typename T>
__device__ void cta_precond(const T* W, int n, int kind, const int* perm, const double* v,
                            double* z) {
  for (int r = threadIdx.x; r < n; r += kBT) z[r] = v[kind == 0 ? perm[r] : r];
  __syncthreads();
  cta_solve<T, double>(W, n, n, kind == 0, z, 1);
}

// One right-hand side: improves x in place until its normwise backward
// error ||b - A x|| / (nA ||x|| + ||b||) <= tol or max_inner iterations are
// spent.  Returns the inner iterations used; *berr gets the last explicit
// backward error.
template <typename T>
__device__ __noinline__ int cta_fgmres(const double* A, int n, double nA, const T* W, int kind,
                          const int* perm, const double* b, double* x, double* kry, int m,
                          int max_inner, double tol, T* vt, Shared& sh, KryShared& ks,
                          double* berr) {
  double* Vk = kry;                       // V_0 .. V_m
  double* Zk = kry + (long)(m + 1) * n;   // Z_0 .. Z_{m-1}
  double* tmp = Zk + (long)m * n;
  int total = 0;
  double sum, mx;
  block_sum_max(n, [&](int i) { return b[i] * b[i]; }, sh, &sum, &mx);
  const double nb = sqrt(sum);
  while (true) {
    cta_matvec(A, n, x, tmp);
    for (int r = threadIdx.x; r < n; r += kBT) Vk[r] = b[r] - tmp[r];
    __syncthreads();
    block_sum_max(n, [&](int i) { return Vk[i] * Vk[i]; }, sh, &sum, &mx);
    const double beta = sqrt(sum);
    block_sum_max(n, [&](int i) { return x[i] * x[i]; }, sh, &sum, &mx);
    const double den = nA * sqrt(sum) + nb;
    const double be = den > 0 ? beta / den : (beta > 0 ? INFINITY : 0.0);
    *berr = be;
    if (be <= tol || total >= max_inner || !(be == be) || beta == 0.0) return total;
    for (int r = threadIdx.x; r < n; r += kBT) Vk[r] /= beta;
    if (threadIdx.x == 0) {
      ks.g[0] = beta;
      for (int k = 1; k <= kKryMax; ++k) ks.g[k] = 0.0;
    }
    __syncthreads();
    int jd = 0;
    for (int j = 0; j < m && total < max_inner; ++j) {
      double* zj = Zk + (long)j * n;
      double* w = Vk + (long)(j + 1) * n;
      cta_precond<T>(W, n, kind, perm, Vk + (long)j * n, zj);
      cta_matvec(A, n, zj, w);
      for (int pass = 0; pass < 2; ++pass) {
        cta_multi_dot(Vk, n, j + 1, w, n, ks.h);
        for (int r = threadIdx.x; r < n; r += kBT) {
          double acc = w[r];
          for (int i = 0; i <= j; ++i) acc = fma(-ks.h[i], Vk[(long)i * n + r], acc);
          w[r] = acc;
        }
        if (threadIdx.x == 0)
          for (int i = 0; i <= j; ++i) ks.H[i][j] = (pass ? ks.H[i][j] : 0.0) + ks.h[i];
        __syncthreads();
      }
      block_sum_max(n, [&](int i) { return w[i] * w[i]; }, sh, &sum, &mx);
      const double hn = sqrt(sum);
      for (int r = threadIdx.x; r < n; r += kBT) w[r] = hn > 0 ? w[r] / hn : 0.0;
      if (threadIdx.x == 0) {
        for (int i = 0; i < j; ++i) {  // previous rotations
          const double t = ks.cs[i] * ks.H[i][j] + ks.sn[i] * ks.H[i + 1][j];
          ks.H[i + 1][j] = -ks.sn[i] * ks.H[i][j] + ks.cs[i] * ks.H[i + 1][j];
          ks.H[i][j] = t;
        }
        const double a = ks.H[j][j];
        const double rr = hypot(a, hn);
        const double c = rr > 0 ? a / rr : 1.0, sv = rr > 0 ? hn / rr : 0.0;
        ks.cs[j] = c;
        ks.sn[j] = sv;
        ks.H[j][j] = rr;
        ks.g[j + 1] = -sv * ks.g[j];
        ks.g[j] = c * ks.g[j];
        // the least-squares residual estimate is |g_{j+1}|
        ks.stop = (fabs(ks.g[j + 1]) <= 0.25 * tol * den || hn == 0.0) ? 1 : 0;
      }
      __syncthreads();
      ++total;
      jd = j + 1;
      if (ks.stop) break;
    }
    if (threadIdx.x == 0) {
      for (int i = jd - 1; i >= 0; --i) {
        double acc = ks.g[i];
        for (int k = i + 1; k < jd; ++k) acc -= ks.H[i][k] * ks.y[k];
        ks.y[i] = ks.H[i][i] != 0.0 ? acc / ks.H[i][i] : 0.0;
      }
    }
    __syncthreads();
    for (int r = threadIdx.x; r < n; r += kBT) {
      double acc = x[r];
      for (int i = 0; i < jd; ++i) acc = fma(ks.y[i], Zk[(long)i * n + r], acc);
      x[r] = acc;
    }
    __syncthreads();
  }
}

template <typename T>
__device__ int factor_sys(T* W, int n, int kind, int nb, int ib, int* piv, Shared& sh, T* smem,
                          unsigned char* tc_tiles,
                          int smem_elems, bool lowp) {
  return kind == 0 ? cta_lu<T>(W, n, n, nb, ib, piv, sh, smem, smem_elems, lowp, tc_tiles)
                   : cta_chol<T>(W, n, n, ib, smem, lowp);
}

// W = (T) A over nn elements, 8 loads in flight per thread.
template <typename T>
__device__ __forceinline__ void cta_copy_cast(const double* A, T* W, long nn) {
  long i = threadIdx.x;
  for (; i + 7L * kBT < nn; i += 8L * kBT) {
    double v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = A[i + (long)u * kBT];
#pragma unroll
    for (int u = 0; u < 8; ++u) W[i + (long)u * kBT] = (T)v[u];
  }
  for (; i < nn; i += kBT) W[i] = (T)A[i];
}

// One pass over the FP64 matrix (column-major n x n) for the selector's
// norm features: the sum of squares (||A||_F^2), the largest column sum
// (||A||_1), max |a_ij|, sum |a_ii|, the row sums of |A| accumulated in
// shared memory (rowacc, n doubles; ||A||_inf), and the FP32 copy Wf that
// the feature LU factors.  One warp per column with 16 loads in flight per
// lane, so A is read once instead of once per quantity.
struct MatScan {
  double fro2, col1, amax, rowinf, dsum;
};

__device__ __noinline__ void cta_scan_matrix(const double* A, int n, float* Wf, double* rowacc,
                                             Shared& sh, MatScan* out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < n; i += kBT) rowacc[i] = 0.0;
  __syncthreads();
  constexpr int V = 16;
  double fro = 0.0, cmax = 0.0, am = 0.0, ds = 0.0;
  for (int j = warp; j < n; j += kBT / 32) {
    const double* col = A + (long)j * n;
    float* wcol = Wf + (long)j * n;
    double c = 0.0, m = 0.0;
    for (int i0 = 0; i0 < n; i0 += 32 * V) {
      double v[V];
#pragma unroll
      for (int u = 0; u < V; ++u) {
        const int i = i0 + lane + 32 * u;
        v[u] = i < n ? col[i] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < V; ++u) {
        const int i = i0 + lane + 32 * u;
        if (i < n) {
          const double a = fabs(v[u]);
          c += a;
          m = fmax(m, a);
          fro = fma(v[u], v[u], fro);
          atomicAdd(&rowacc[i], a);
          wcol[i] = (float)v[u];
          if (i == j) ds += a;
        }
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      c += __shfl_xor_sync(0xffffffffu, c, o);
      m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    }
    cmax = fmax(cmax, c);
    am = fmax(am, m);
  }
  for (int o = 16; o > 0; o >>= 1) {
    fro += __shfl_xor_sync(0xffffffffu, fro, o);
    ds += __shfl_xor_sync(0xffffffffu, ds, o);
  }
  __syncthreads();  // row sums complete
  double rmax = 0.0;
  for (int i = threadIdx.x; i < n; i += kBT) rmax = fmax(rmax, rowacc[i]);
  for (int o = 16; o > 0; o >>= 1) rmax = fmax(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
  if (lane == 0) {
    sh.red[warp][0] = fro;
    sh.red[warp][1] = cmax;
    sh.red[warp][2] = am;
    sh.red[warp][3] = ds;
    sh.red[warp][4] = rmax;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    MatScan r{0.0, 0.0, 0.0, 0.0, 0.0};
    for (int w = 0; w < kBT / 32; ++w) {
      r.fro2 += sh.red[w][0];
      r.col1 = fmax(r.col1, sh.red[w][1]);
      r.amax = fmax(r.amax, sh.red[w][2]);
      r.dsum += sh.red[w][3];
      r.rowinf = fmax(r.rowinf, sh.red[w][4]);
    }
    sh.colv[0] = r.fro2;
    sh.colv[1] = r.col1;
    sh.colv[2] = r.amax;
    sh.colv[3] = r.dsum;
    sh.colv[4] = r.rowinf;
  }
  __syncthreads();
  *out = MatScan{sh.colv[0], sh.colv[1], sh.colv[2], sh.colv[4], sh.colv[3]};
  __syncthreads();
}

// The selector's 16 features of one system (written to p.feat[s * 16 ..]):
// norm ratios of A, an FP32 LU's growth and pivot spread, and a Hager /
// Higham 1-norm estimate of ||A^{-1}||_1 (LAPACK xLACON's iteration plus
// Higham's alternating vector) computed with that FP32 LU.
__device__ __noinline__ int compute_features(const BatchParams& p, const SysDesc& d, int s, const double* A,
                                 int n, double* na_out, float* Wf, int* piv, int* perm, float* v,
                                 Shared& sh, float* smf, unsigned char* tc_tiles) {
  __shared__ float s_fv[16];
  double sum;
  // one pass over A: norms, row sums (in the panel's shared memory), FP32 copy
  MatScan ms;
  // (row sums in the vector workspace -- n doubles -- past the panel's size)
  cta_scan_matrix(A, n, Wf,
                  (long)n * 8 <= kSmemPanel ? reinterpret_cast<double*>(smf)
                                            : reinterpret_cast<double*>(v),
                  sh, &ms);
  const double colmax = ms.col1, rowmax = ms.rowinf, amax = ms.amax, dsum = ms.dsum;
  const double nA = sqrt(ms.fro2);
  if (threadIdx.x == 0) *na_out = nA;
  // FP32 factorization (Wf holds the FP32 copy)
  const int info = factor_sys<float>(Wf, n, d.kind, d.nb, d.ib, piv, sh, smf, p.tc ? tc_tiles : nullptr,
                                     kSmemPanel / (int)sizeof(float), false);
  double umax = 0.0, dmin = 0.0, dmax = 0.0;
  block_sum_max(n, [&](int j) {
    double m = 0.0;
    const int top = d.kind == 0 ? j : n - 1;  // U (LU) or L (Cholesky) column j
    const int i0 = d.kind == 0 ? 0 : j;
    for (int i = i0; i <= top; ++i) m = fmax(m, fabs((double)Wf[i + (long)j * n]));
    return m;
  }, sh, &sum, &umax);
  block_sum_max(n, [&](int j) { return fabs((double)Wf[j + (long)j * n]); }, sh, &sum, &dmax);
  block_sum_max(n, [&](int j) { return 1.0 / fmax(fabs((double)Wf[j + (long)j * n]), 1e-300); },
                sh, &sum, &dmin);
  dmin = 1.0 / dmin;
  double est = 0.0, est2 = 0.0;
  int iters = 0;
  if (info == 0) {
    if (d.kind == 0)
      cta_perm_from_swaps(piv, n, perm, reinterpret_cast<int*>(smf), kSmemPanel / (int)sizeof(int));
    else
      cta_mirror_lower(Wf, n, n);
    float* y = v;
    float* z = v + n;
    // Hager: x = 1/n
    int jlast = -1;
    for (int it = 0; it < 5; ++it) {
      ++iters;
      for (int i = threadIdx.x; i < n; i += kBT) {
        const float xi = it == 0 ? 1.f / n : (i == jlast ? 1.f : 0.f);
        z[i] = xi;
      }
      __syncthreads();
      for (int i = threadIdx.x; i < n; i += kBT) y[i] = z[d.kind == 0 ? perm[i] : i];
      __syncthreads();
      cta_solve<float, float>(Wf, n, n, d.kind == 0, y, 1);  // y = A^{-1} x
      double ny, dum;
      block_sum_max(n, [&](int i) { return fabs((double)y[i]); }, sh, &ny, &dum);
      if (it > 0 && ny <= est) break;
      est = ny;
      // z = A^{-T} sign(y)
      for (int i = threadIdx.x; i < n; i += kBT) z[i] = y[i] >= 0.f ? 1.f : -1.f;
      __syncthreads();
      cta_solve_t<float>(Wf, n, n, d.kind == 0, z);
      if (d.kind == 0) {  // inverse permutation: P^T z
        for (int i = threadIdx.x; i < n; i += kBT) y[perm[i]] = z[i];
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += kBT) z[i] = y[i];
        __syncthreads();
      }
      // j = argmax |z|, and z^T x
      __shared__ float s_zx;
      __shared__ int s_j;
      if (threadIdx.x == 0) {
        int jb = 0;
        float zb = -1.f, zx = 0.f;
        for (int i = 0; i < n; ++i) {
          const float a = fabsf(z[i]);
          if (a > zb) {
            zb = a;
            jb = i;
          }
          zx += z[i] * (it == 0 ? 1.f / n : (i == jlast ? 1.f : 0.f));
        }
        s_j = jb;
        s_zx = (fabsf(z[jb]) <= zx) ? 1.f : 0.f;
      }
      __syncthreads();
      if (it > 0 && s_zx > 0.f) break;
      if (s_j == jlast) break;
      jlast = s_j;
    }
    // Higham's alternating vector: x_i = (-1)^i (1 + i / (n - 1))
    for (int i = threadIdx.x; i < n; i += kBT) {
      const int src = d.kind == 0 ? perm[i] : i;
      y[i] = (src & 1 ? -1.f : 1.f) * (1.f + (n > 1 ? (float)src / (n - 1) : 0.f));
    }
    __syncthreads();
    cta_solve<float, float>(Wf, n, n, d.kind == 0, y, 1);
    double ny, dum;
    block_sum_max(n, [&](int i) { return fabs((double)y[i]); }, sh, &ny, &dum);
    est2 = 2.0 * ny / (3.0 * n);
  }
  if (threadIdx.x == 0) {
    const double tiny = 1e-300;
    const double e = fmax(est, est2);
    const double fro = fmax(nA, tiny);
    s_fv[0] = (float)log2((double)n);
    s_fv[1] = (float)log10(fmax(colmax * e, 1.0));
    s_fv[2] = (float)log10(fmax(colmax, tiny) / fro);
    s_fv[3] = (float)log10(fmax(rowmax, tiny) / fro);
    s_fv[4] = (float)log10(fmax(amax, tiny) / fro);
    s_fv[5] = (float)log10(fmax(umax, tiny) / fmax(amax, tiny));
    s_fv[6] = (float)log10(fmax(dmin, tiny) / fmax(dmax, tiny));
    s_fv[7] = (float)log10(fmax(dsum / (n * fmax(amax, tiny)), 1e-30));
    s_fv[8] = (float)d.kind;
    s_fv[9] = (float)log10(fro);
    s_fv[10] = (float)log10(fmax(e, tiny));
    s_fv[11] = (float)log10(fmax(dmin, tiny));
    s_fv[12] = (float)log10(fmax(dmax, tiny));
    s_fv[13] = (float)iters;
    s_fv[14] = info != 0 ? 1.f : 0.f;
    s_fv[15] = (float)log10(fmax(est2, tiny) / fmax(est, tiny));
    for (int k = 0; k < 16; ++k) {
      float f = s_fv[k];
      if (!(f == f) || f > 1e30f || f < -1e30f) f = 0.f;  // keep features finite
      sh.feat[k] = f;
      if (p.feat) p.feat[(long)s * 16 + k] = f;
    }
    BatchResult r{};
    r.info = info;
    r.berr = colmax * fmax(est, est2);  // the kappa_1 estimate
    p.out[s] = r;
  }
  __syncthreads();
  return info;
}

__global__ void __launch_bounds__(kBT, 1)
batched_solve_kernel(BatchParams p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ Shared sh;
  __shared__ int s_sys;
  __shared__ double s_na;
  __shared__ double s_sc[kBQ];
  const long cta = blockIdx.x;
  float* Wf = static_cast<float*>(p.wsf) + cta * p.ws_elems;
  double* Wd = p.wsd + cta * p.ws_elems;
  int* piv = p.pivws + cta * 2 * p.nmax;
  int* perm = piv + p.nmax;
  double* R = p.vec + cta * (long)p.nmax * p.q * 3;
  double* Xprev = R + (long)p.nmax * p.q;
  double* V = Xprev + (long)p.nmax * p.q;  // solve vector, as float or double
  double* kry = p.kry + cta * (long)(2 * p.kry_m + 2) * p.nmax;
  __shared__ KryShared ks;
  const int q = p.q;
  // tensor-core update state: operand tiles after the panel budget (1024-
  // byte aligned), the commit barrier, two 128-column TMEM accumulators
  unsigned char* tc_tiles = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + kSmemPanel + 1023) & ~uintptr_t(1023));
  if (threadIdx.x == 0) {
    tc::mbar_init(reinterpret_cast<uint64_t*>(&sh.mma_bar), 1);
    tc::fence_mbar_init();
    sh.mma_phase = 0;
    sh.tc_err = 0;
  }
  if (threadIdx.x < 32) tc::tmem_alloc(&sh.tmem, kTcCols);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  while (true) {
    __syncthreads();
    if (threadIdx.x == 0) s_sys = (int)atomicAdd(p.ticket, 1u);
    __syncthreads();
    const int t = s_sys;
    if (t >= p.count) break;
    const int s = p.order[t];
    const SysDesc d = p.desc[s];
    const int n = d.n;
    const double* A = p.A + d.a_off;
    const double* B = p.B + d.b_off;
    double* X = p.X + d.b_off;
    BatchResult res{};
    const unsigned long long t_begin = globaltimer_ns();
    if (threadIdx.x < kPhases) sh.ph[threadIdx.x] = 0ull;
    auto mark = [&](int i, unsigned long long since) {  // thread 0, after a barrier
      if (threadIdx.x == 0) sh.ph[i] += globaltimer_ns() - since;
    };
    bool done = false;
    if (p.mode == 1) {
      compute_features(p, d, s, A, n, &s_na, Wf, piv, perm, reinterpret_cast<float*>(V), sh,
                       reinterpret_cast<float*>(smem_raw), tc_tiles);
      __syncthreads();
      mark(7, t_begin);
      if (p.phase_ns && threadIdx.x < kPhases)
        p.phase_ns[(long)s * kPhases + threadIdx.x] = sh.ph[threadIdx.x];
      continue;
    }
    if (p.mode == 0) {  // ||A||_F (the feature pass computes it in mode 2)
      const long nn = (long)n * n;
      double acc[4] = {0.0, 0.0, 0.0, 0.0};
      long i = threadIdx.x;
      for (; i + 7L * kBT < nn; i += 8L * kBT) {  // 8 loads in flight
        double v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = A[i + (long)u * kBT];
#pragma unroll
        for (int u = 0; u < 8; ++u) acc[u & 3] = fma(v[u], v[u], acc[u & 3]);
      }
      for (; i < nn; i += kBT) acc[0] = fma(A[i], A[i], acc[0]);
      double a = (acc[0] + acc[1]) + (acc[2] + acc[3]);
      for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
      if ((threadIdx.x & 31) == 0) sh.red[threadIdx.x >> 5][0] = a;
      __syncthreads();
      if (threadIdx.x == 0) {
        double v = 0.0;
        for (int w = 0; w < kBT / 32; ++w) v += sh.red[w][0];
        s_na = sqrt(v);
      }
      __syncthreads();
    }
    // precision chosen at run time (the selector's output) or at plan time
    int prec = d.prec;
    if (p.prec_dev) prec = min(max(p.prec_dev[s], 0), 2);
    bool have32 = false;  // FP32 factors of this system already in Wf
    if (p.mode == 2) {
      // fused selection: features from an FP32 LU (kept), the network's
      // choice, then the solve -- a low-precision choice refines with the
      // FP32 factors just computed (they are at least as good as BF16's)
      const int finfo = compute_features(p, d, s, A, n, &s_na, Wf, piv, perm,
                                         reinterpret_cast<float*>(V), sh,
                                         reinterpret_cast<float*>(smem_raw), tc_tiles);
      __syncthreads();
      mark(7, t_begin);
      prec = mlpd::block_argmax(p.mlp, sh.feat, sh.h1, sh.h2, sh.lg);
      res.choice = prec;
      have32 = finfo == 0;
    }
    const double nA = s_na;
    res.prec = prec;  // becomes the precision the result came from
    // low-precision attempts: BF16 (if chosen), then FP32 when falling back
    for (int pr = prec; pr >= 1 && !done; --pr) {
      if (pr != prec && !p.fallback) break;
      if (have32 && pr != prec) break;  // the kept FP32 factors were the attempt
      // FP32 factors (BF16 operand products for pr 2) + FP64 refinement
      float* smf = reinterpret_cast<float*>(smem_raw);
      int info = 0;
      if (!have32) {
        cta_copy_cast(A, Wf, (long)n * n);
        __syncthreads();
        info = factor_sys<float>(Wf, n, d.kind, d.nb, d.ib, piv, sh, smf, p.tc ? tc_tiles : nullptr,
                                 kSmemPanel / (int)sizeof(float), pr == 2);
        if (info == 0) {
          if (d.kind == 0)
            cta_perm_from_swaps(piv, n, perm, reinterpret_cast<int*>(smem_raw),
                                kSmemPanel / (int)sizeof(int));
          else
            cta_mirror_lower(Wf, n, n);
        }
      }
      res.info = info;
      if (info == 0) {
        float* vf = reinterpret_cast<float*>(V);
        const unsigned long long t_ir = globaltimer_ns();
        unsigned long long t_sub = t_ir;
        cta_apply_inverse<float>(Wf, n, d.kind, perm, B, X, vf, nullptr, q, false, s_sc);
        mark(9, t_sub);
        const int lu_its = p.method == 2 ? 0 : p.max_iters;
        double prev = INFINITY;
        for (int it = 0;; ++it) {
          t_sub = globaltimer_ns();
          const double be = sys_berr(A, n, X, B, R, q, sh, nA);
          mark(8, t_sub);
          if (it > 0 && !(be < prev)) {
            // Refined.hpp keeps an update only if it lowers the residual
            for (int i = threadIdx.x; i < n * q; i += kBT) X[i] = Xprev[i];
            __syncthreads();
            res.berr = prev;
            break;
          }
          res.berr = be;
          res.iters = it;
          if (be <= p.tol) {
            done = true;
            res.prec = pr;
            break;
          }
          if (it >= lu_its) break;
          prev = be;
          for (int i = threadIdx.x; i < n * q; i += kBT) Xprev[i] = X[i];
          t_sub = globaltimer_ns();
          cta_apply_inverse<float>(Wf, n, d.kind, perm, R, X, vf, nullptr, q, true, s_sc);
          mark(9, t_sub);
        }
        __syncthreads();
        mark(4, t_ir);
        const int kry_budget = p.kry_max > 0 ? p.kry_max : max(16, n / -p.kry_max);
        if (!done && p.method != 1) {
          const unsigned long long t_kr = globaltimer_ns();
          // LU-IR stalled (or was skipped): FGMRES-IR per right-hand side
          // from the best iterate, kept only if it lowers the backward error
          for (int i = threadIdx.x; i < n * q; i += kBT) Xprev[i] = X[i];
          __syncthreads();
          int used = 0;
          for (int c = 0; c < q; ++c) {
            double bc;
            used += cta_fgmres<float>(A, n, nA, Wf, d.kind, perm, B + (long)c * n,
                                      X + (long)c * n, kry, p.kry_m, kry_budget, p.tol, vf, sh,
                                      ks, &bc);
          }
          res.gmres_iters = used;
          const double be = sys_berr(A, n, X, B, R, q, sh, nA);
          if (be < res.berr) {
            res.berr = be;
            done = be <= p.tol;
            if (done) res.prec = pr;
          } else {
            for (int i = threadIdx.x; i < n * q; i += kBT) X[i] = Xprev[i];
            __syncthreads();
          }
          __syncthreads();
          mark(5, t_kr);
        }
      }
    }
    if (!done && (p.fallback || prec == 0)) {
      // FP64 factors: the plain path, or the fallback
      res.prec = 0;
      const unsigned long long t_64 = globaltimer_ns();
      unsigned long long keep[4];
      for (int i = 0; i < 4; ++i) keep[i] = sh.ph[i];  // the FP64 LU's phases go to 6
      double* smd = reinterpret_cast<double*>(smem_raw);
      cta_copy_cast(A, Wd, (long)n * n);
      __syncthreads();
      int nb64 = max(1, min(d.nb, (kSmemPanel / 8 - 64 * 64) / max(n, 1)));
      if (nb64 > 8) nb64 = nb64 / 8 * 8;
      const int info = factor_sys<double>(Wd, n, d.kind, nb64, nb64, piv, sh, smd, nullptr,
                                          kSmemPanel / (int)sizeof(double), false);
      res.info = info;
      if (info == 0) {
        if (d.kind == 0)
          cta_perm_from_swaps(piv, n, perm, reinterpret_cast<int*>(smem_raw),
                              kSmemPanel / (int)sizeof(int));
        else
          cta_mirror_lower(Wd, n, n);
        cta_apply_inverse<double>(Wd, n, d.kind, perm, B, X, V, nullptr, q, false, s_sc);
      }
      res.berr = sys_berr(A, n, X, B, R, q, sh, nA);
      done = res.berr <= p.tol;
      __syncthreads();
      if (threadIdx.x == 0)
        for (int i = 0; i < 4; ++i) sh.ph[i] = keep[i];
      mark(6, t_64);
    }
    res.converged = done ? 1 : 0;
    res.fell_back = (res.prec != prec) ? 1 : 0;
    res.ns = (long long)(globaltimer_ns() - t_begin);
    if (sh.tc_err) res.info = -1;  // a tensor-core wait timed out: result invalid
    if (threadIdx.x == 0) p.out[s] = res;
    __syncthreads();
    if (p.phase_ns && threadIdx.x < kPhases)
        p.phase_ns[(long)s * kPhases + threadIdx.x] = sh.ph[threadIdx.x];
  }
  __syncthreads();
  if (sh.tc_err) {
    if (threadIdx.x == 0) atomicExch(p.err, 1);
    // let an MMA that outlived the wait finish before the TMEM goes (bounded)
    const unsigned long long t0 = globaltimer_ns();
    while (!tc::mbar_try_wait(reinterpret_cast<uint64_t*>(&sh.mma_bar), sh.mma_phase) &&
           globaltimer_ns() - t0 < kSpinLimitNs) {
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (threadIdx.x < 32) {
    tc::tc_fence_after();
    tc::tmem_dealloc(sh.tmem, kTcCols);
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// host side: plan (descriptors, order, workspaces, CUDA graph) and execute
// ---------------------------------------------------------------------------
struct BatchPlan {
  Context* ctx = nullptr;
  int count = 0, q = 0, nmax = 0;
  SysDesc* d_desc = nullptr;
  int* d_order = nullptr;
  void* d_wsf = nullptr;
  double* d_wsd = nullptr;
  int* d_piv = nullptr;
  double* d_vec = nullptr;
  double* d_kry = nullptr;
  unsigned* d_ticket = nullptr;
  int* d_err = nullptr;
  BatchResult* d_out = nullptr;
  int grid = 0;
  long ws_elems = 0;
  BatchParams prm{};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  double flops = 0;
};

// Block width nb (from the tuned table, <= 64) and the shared-memory panel
// width ib <= nb: the panel (n x ib) plus a 64-column staging tile fit the
// budget.  Multiples of 8 (the register-resident U12 solves take 8 / 16 / 32).
static void pick_nb(int n, int prec, const int* nb_table, int* nb_out, int* ib_out) {
  // size buckets: <=32, <=64, <=128, <=256, <=512, <=1024, <=2048, larger
  int b = 0;
  for (int lim = 32; b < 7 && n > lim; lim *= 2) ++b;
  int nb = nb_table ? nb_table[b] : 32;
  if (nb <= 0) nb = 32;
  nb = std::max(1, std::min(nb, 64));
  if (nb > 8) nb = nb / 8 * 8;
  const int es = prec == 0 ? 8 : 4;  // the FP64 path re-caps for itself
  const int cap = (kSmemPanel / es - 64 * 64) / std::max(n, 1);
  int ib = std::min(nb, std::max(cap, 1));
  if (ib > 8) ib = ib / 8 * 8;
  *nb_out = nb;
  *ib_out = ib;
}

cudaError_t batched_plan(Context* ctx, int count, const int* h_n, const int* h_kind,
                         const int* h_prec, int q, const double* A, const double* B, double* X,
                         const int* nb_table, int ctas_per_sm, double tol, int max_iters,
                         int fallback, int mode, float* feat, int method, int kry_m,
                         int kry_max, const int* prec_dev, unsigned long long* phase_ns,
                         const float* mlp, int tc, BatchPlan** out) {
  *out = nullptr;
  if (q < 1 || q > kBQ) return cudaErrorInvalidValue;
  kry_m = kry_m > 0 ? std::min(kry_m, kKryMax) : 30;
  // <= 0: per-system budget max(16, n / 24) inner iterations: an iteration
  // (FP64 matrix-vector product + FP64-arithmetic triangular solves, both
  // bandwidth-bound in one CTA) costs ~12 / n of an FP64 LU, so FGMRES stays
  // under ~half of the factorization it would save
  kry_max = kry_max > 0 ? kry_max : (kry_max < 0 ? kry_max : -24);
  if (method == 1) kry_m = 1;  // no Krylov workspace beyond a token
  auto* P = new BatchPlan();
  P->ctx = ctx;
  P->count = count;
  P->q = q;
  std::vector<SysDesc> desc(count);
  long aoff = 0, boff = 0;
  int nmax = 1;
  for (int i = 0; i < count; ++i) {
    SysDesc& s = desc[i];
    s.n = h_n[i];
    s.kind = h_kind ? h_kind[i] : 0;
    s.prec = h_prec ? h_prec[i] : 1;
    pick_nb(s.n, s.prec, nb_table, &s.nb, &s.ib);
    s.a_off = aoff;
    s.b_off = boff;
    aoff += (long)s.n * s.n;
    boff += (long)s.n * q;
    nmax = std::max(nmax, s.n);
    P->flops += (s.kind == 0 ? 2.0 / 3.0 : 1.0 / 3.0) * (double)s.n * s.n * s.n +
                2.0 * (double)s.n * s.n * q;
  }
  P->nmax = nmax;
  std::vector<int> order(count);
  std::iota(order.begin(), order.end(), 0);
  // largest expected cost first; FP64 arithmetic runs at ~1/60 of the FP32
  // rate on this GPU (a run-time precision is not known here: n^3 alone)
  auto cost = [&](const SysDesc& x) {
    return (double)x.n * x.n * x.n * ((!prec_dev && x.prec == 0) ? 48.0 : 1.0);
  };
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return cost(desc[a]) > cost(desc[b]); });
  P->grid = std::max(1, std::min(count, ctx->num_sms * std::max(1, ctas_per_sm)));
  P->ws_elems = (long)nmax * nmax;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e == cudaSuccess) e = cudaMalloc(&P->d_desc, sizeof(SysDesc) * count);
  if (e == cudaSuccess) e = cudaMalloc(&P->d_order, sizeof(int) * count);
  if (e == cudaSuccess) e = cudaMalloc(&P->d_wsf, sizeof(float) * P->ws_elems * P->grid);
  if (e == cudaSuccess) e = cudaMalloc(&P->d_wsd, sizeof(double) * P->ws_elems * P->grid);
  if (e == cudaSuccess) e = cudaMalloc(&P->d_piv, sizeof(int) * 2 * (long)nmax * P->grid);
  if (e == cudaSuccess) e = cudaMalloc(&P->d_vec, sizeof(double) * 3 * (long)nmax * q * P->grid);
  if (e == cudaSuccess)
    e = cudaMalloc(&P->d_kry, sizeof(double) * (2 * (long)kry_m + 2) * nmax * P->grid);
  if (e == cudaSuccess) e = cudaMalloc(&P->d_ticket, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMalloc(&P->d_err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(P->d_err, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&P->d_out, sizeof(BatchResult) * count);
  if (e == cudaSuccess)
    e = cudaMemcpy(P->d_desc, desc.data(), sizeof(SysDesc) * count, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(P->d_order, order.data(), sizeof(int) * count, cudaMemcpyHostToDevice);
  // the memset and the pageable copies above ran on the legacy stream, which
  // the stream the plan later launches on need not wait for: drain it now
  if (e == cudaSuccess) e = cudaStreamSynchronize(cudaStreamLegacy);
  if (e != cudaSuccess) {
    batched_destroy(P);
    return e;
  }
  BatchParams& prm = P->prm;
  prm.desc = P->d_desc;
  prm.order = P->d_order;
  prm.count = count;
  prm.q = q;
  prm.A = A;
  prm.B = B;
  prm.X = X;
  prm.wsf = P->d_wsf;
  prm.wsd = P->d_wsd;
  prm.ws_elems = P->ws_elems;
  prm.pivws = P->d_piv;
  prm.vec = P->d_vec;
  prm.nmax = nmax;
  prm.tol = tol > 0 ? tol : 1e-13;
  prm.max_iters = max_iters > 0 ? max_iters : 10;
  prm.ticket = P->d_ticket;
  prm.out = P->d_out;
  prm.mode = (mode == 0 && mlp) ? 2 : mode;
  prm.mlp = mlp;
  prm.tc = tc ? 1 : 0;
  prm.err = P->d_err;
  prm.fallback = fallback;
  prm.feat = feat;
  prm.method = method;
  prm.kry_m = kry_m;
  prm.kry_max = kry_max;
  prm.kry = P->d_kry;
  prm.prec_dev = prec_dev;
  prm.phase_ns = phase_ns;
  e = cudaFuncSetAttribute(batched_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           kDynSmem);
  if (e != cudaSuccess) {
    batched_destroy(P);
    return e;
  }
  // capture the launch (ticket reset + persistent kernel) into a CUDA graph
  cudaStream_t cs;
  e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaMemsetAsync(P->d_ticket, 0, sizeof(unsigned), cs);
    batched_solve_kernel<<<P->grid, kBT, kDynSmem, cs>>>(prm);
    e = cudaStreamEndCapture(cs, &P->graph);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&P->exec, P->graph, 0);
  cudaStreamDestroy(cs);
  if (e != cudaSuccess) {
    batched_destroy(P);
    return e;
  }
  *out = P;
  return cudaSuccess;
}

cudaError_t batched_execute(BatchPlan* P) {
  cudaError_t e = cudaSetDevice(P->ctx->device);
  if (e != cudaSuccess) return e;
  e = cudaGraphLaunch(P->exec, P->ctx->stream);
  P->ctx->launches += 1;
  return e;
}

cudaError_t batched_results(BatchPlan* P, BatchResult* h_out) {
  cudaError_t e = cudaMemcpyAsync(h_out, P->d_out, sizeof(BatchResult) * P->count,
                                  cudaMemcpyDeviceToHost, P->ctx->stream);
  int err = 0;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&err, P->d_err, sizeof(int), cudaMemcpyDeviceToHost, P->ctx->stream);
  if (e != cudaSuccess) return e;
  e = cudaStreamSynchronize(P->ctx->stream);
  if (e == cudaSuccess && err) return cudaErrorLaunchTimeout;  // a bounded wait expired
  return e;
}

void batched_destroy(BatchPlan* P) {
  if (!P) return;
  if (P->exec) cudaGraphExecDestroy(P->exec);
  if (P->graph) cudaGraphDestroy(P->graph);
  cudaFree(P->d_desc);
  cudaFree(P->d_order);
  cudaFree(P->d_wsf);
  cudaFree(P->d_wsd);
  cudaFree(P->d_piv);
  cudaFree(P->d_vec);
  cudaFree(P->d_kry);
  cudaFree(P->d_ticket);
  cudaFree(P->d_err);
  cudaFree(P->d_out);
  delete P;
}

double batched_flops(const BatchPlan* P) { return P->flops; }

}  // namespace elgb

// ===========================================================================
// C ABI (include/elgb300.h)
// ===========================================================================
struct ElGBBatchPlanImpl {
  elgb::BatchPlan* p;
};

extern "C" {

int ElGBBatchedPlanCreate(ElGBContext ctx, int count, const int* n, int nrhs, const double* A,
                          const double* B, double* X, const ElGBBatchOptions* opt,
                          ElGBBatchPlan* plan) {
  ElGBBatchOptions o{};
  if (opt) o = *opt;
  if (!ctx || !plan || count <= 0 || !n || nrhs < 1 || nrhs > 8 || !A ||
      (!o.features_only && (!B || !X)) || (o.features_only && !o.features))
    return elgb::kElArgError;
  for (int i = 0; i < count; ++i)
    if (n[i] < 1 || (o.kind && (o.kind[i] < 0 || o.kind[i] > 1)) ||
        (o.precision && (o.precision[i] < 0 || o.precision[i] > 2)))
      return elgb::kElArgError;
  if (o.method < 0 || o.method > 2 || o.gmres_restart < 0 || o.gmres_restart > 32 ||
      o.gmres_max_iters < -4096)
    return elgb::kElArgError;
  *plan = nullptr;
  elgb::BatchPlan* p = nullptr;
  cudaError_t e = elgb::batched_plan(static_cast<elgb::Context*>(ctx), count, n, o.kind,
                                     o.precision, nrhs, A, B, X, o.nb_table, o.ctas_per_sm, o.tol,
                                     o.max_iters, o.no_fallback ? 0 : 1,
                                     o.features_only ? 1 : 0, o.features, o.method,
                                     o.gmres_restart, o.gmres_max_iters, o.precision_device,
                                     reinterpret_cast<unsigned long long*>(o.phase_ns),
                                     o.selector_params, o.simt_update ? 0 : 1, &p);
  if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? elgb::kElAllocError
                                                               : elgb::kElRuntimeError;
  *plan = new ElGBBatchPlanImpl{p};
  return 0;
}

int ElGBBatchedExecute(ElGBBatchPlan plan) {
  if (!plan) return elgb::kElArgError;
  return elgb::to_el_error(elgb::batched_execute(plan->p));
}

int ElGBBatchedResults(ElGBBatchPlan plan, ElGBBatchResult* out) {
  if (!plan || !out) return elgb::kElArgError;
  static_assert(sizeof(ElGBBatchResult) == sizeof(elgb::BatchResult), "layout");
  return elgb::to_el_error(
      elgb::batched_results(plan->p, reinterpret_cast<elgb::BatchResult*>(out)));
}

double ElGBBatchedFlops(ElGBBatchPlan plan) { return plan ? elgb::batched_flops(plan->p) : 0.0; }

int ElGBBatchedPlanDestroy(ElGBBatchPlan plan) {
  if (!plan) return elgb::kElArgError;
  elgb::batched_destroy(plan->p);
  delete plan;
  return 0;
}

}  // extern "C"
