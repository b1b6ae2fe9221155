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

namespace elgb {

namespace {

constexpr int kBT = 256;               // threads per CTA
constexpr int kBQ = 8;                 // max right-hand sides
constexpr int kSmemPanel = 160 * 1024; // panel staging budget (bytes)

struct SysDesc {
  int n, kind, nb, prec;  // kind 0 LU, 1 Cholesky; prec 0 FP64, 1 FP32 + IR
  long a_off, b_off;      // into A (FP64, ld n) and B / X (FP64, ld n)
};

struct Shared {
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
// Row interchanges of the panel's swaps (rows k+i <-> piv[i], i < jb) on the
// columns outside [k, k+jb), via the (dst, src) list of changed rows, staged
// through shared memory in column chunks.
template <typename T>
__device__ void cta_apply_swaps(T* W, int n, int ld, int k, int jb, Shared& sh, T* stage,
                                int stage_elems) {
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
  const int cnt = sh.ival[0];
  if (cnt == 0) return;
  const int ncols_out = n - jb;
  const int chunk = max(1, stage_elems / cnt);
  for (int c0 = 0; c0 < ncols_out; c0 += chunk) {
    const int cw = min(chunk, ncols_out - c0);
    for (int idx = threadIdx.x; idx < cw * cnt; idx += kBT) {
      const int e = idx % cnt, cc = c0 + idx / cnt;
      const int col = cc < k ? cc : cc + jb;
      stage[idx] = W[sh.pairs[128 + e] + (long)col * ld];
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < cw * cnt; idx += kBT) {
      const int e = idx % cnt, cc = c0 + idx / cnt;
      const int col = cc < k ? cc : cc + jb;
      W[sh.pairs[e] + (long)col * ld] = stage[idx];
    }
    __syncthreads();
  }
}

// C[m x nc] -= P[m x jb] * Q[jb x nc]: P in shared memory (ld = ldp), Q in
// global (ld = ldq, staged in 64-column chunks into `qs`), C in global.
// 64 x 64 tiles, each thread a 4 x 4 block (rows tx + 16 i, cols ty + 16 j).
template <typename T>
__device__ void cta_gemm_update(const T* P, int ldp, const T* Q, int ldq, T* C, int ldc, int m,
                                int nc, int jb, T* qs, bool lower_only, int row_base,
                                int col_base, bool lowp) {
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  for (int c0 = 0; c0 < nc; c0 += 64) {
    const int cw = min(64, nc - c0);
    __syncthreads();
    for (int idx = threadIdx.x; idx < jb * 64; idx += kBT) {
      const int kk = idx % jb, cc = idx / jb;
      qs[kk + cc * jb] = cc < cw ? rnd(Q[kk + (long)(c0 + cc) * ldq], lowp) : T(0);
    }
    __syncthreads();
    for (int r0 = 0; r0 < m; r0 += 64) {
      if (lower_only && row_base + r0 + 63 < col_base + c0) continue;
      T acc[4][4];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
      for (int kk = 0; kk < jb; ++kk) {
        T a[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int r = r0 + tx + 16 * i;
          a[i] = r < m ? rnd(P[r + kk * ldp], lowp) : T(0);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) b[j] = qs[kk + (ty + 16 * j) * jb];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int r = r0 + tx + 16 * i;
        if (r >= m) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int cc = ty + 16 * j;
          if (cc >= cw) continue;
          if (lower_only && row_base + r < col_base + c0 + cc) continue;
          T* cp = C + r + (long)(c0 + cc) * ldc;
          *cp -= acc[i][j];
        }
      }
    }
  }
  __syncthreads();
}

// In-CTA LU with partial pivoting of the n x n matrix W (ld), blocked by nb.
// piv_out[0..n) receives the swap destinations; returns info (0 ok, j+1 at
// the first zero pivot).
template <typename T>
__device__ int cta_lu(T* W, int n, int ld, int nb, int* piv_out, Shared& sh, T* smem,
                      int smem_elems, bool lowp) {
  __shared__ T fv[9];
  __shared__ int fr[9];
  int info = 0;
  for (int k = 0; k < n; k += nb) {
    const int jb = min(nb, n - k);
    const int mp = n - k;
    T* panel = smem;  // mp x jb, ld mp
    for (int idx = threadIdx.x; idx < mp * jb; idx += kBT) {
      const int r = idx % mp, c = idx / mp;
      panel[idx] = W[(k + r) + (long)(k + c) * ld];
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
      if (threadIdx.x == 0) sh.piv[j] = k + p;
      if (p != j)
        for (int c = threadIdx.x; c < jb; c += kBT) {
          const T t = panel[j + c * mp];
          panel[j + c * mp] = panel[p + c * mp];
          panel[p + c * mp] = t;
        }
      __syncthreads();
      const T alpha = panel[j + j * mp];
      if (alpha == T(0)) {
        if (info == 0) info = k + j + 1;
      } else {
        const T inv = T(1) / alpha;
        for (int r = j + 1 + threadIdx.x; r < mp; r += kBT) {
          const T l = panel[r + j * mp] * inv;
          panel[r + j * mp] = l;
          const T lr = rnd(l, lowp);
          for (int c = j + 1; c < jb; ++c)
            panel[r + c * mp] = fma(-lr, rnd(panel[j + c * mp], lowp), panel[r + c * mp]);
        }
      }
      __syncthreads();
    }
    for (int idx = threadIdx.x; idx < mp * jb; idx += kBT) {
      const int r = idx % mp, c = idx / mp;
      W[(k + r) + (long)(k + c) * ld] = panel[idx];
    }
    for (int j = threadIdx.x; j < jb; j += kBT) piv_out[k + j] = sh.piv[j];
    __syncthreads();
    // swaps on the other columns (staging space after the panel)
    cta_apply_swaps(W, n, ld, k, jb, sh, smem + mp * jb, smem_elems - mp * jb);
    const int n2 = n - k - jb;
    if (n2 > 0) {
      // U12 = L11^{-1} A12 (one thread per column, L11 from the panel)
      for (int c = threadIdx.x; c < n2; c += kBT) {
        T* col = W + k + (long)(k + jb + c) * ld;
        for (int i = 1; i < jb; ++i) {
          T s = col[i];
          for (int l = 0; l < i; ++l) s = fma(-rnd(panel[i + l * mp], lowp), rnd(col[l], lowp), s);
          col[i] = s;
        }
      }
      __syncthreads();
      // A22 -= A21 U12, A21 = panel rows jb.. (still in shared memory)
      cta_gemm_update<T>(panel + jb, mp, W + k + (long)(k + jb) * ld, ld,
                         W + (k + jb) + (long)(k + jb) * ld, ld, n2, n2, jb,
                         smem + mp * jb, false, 0, 0, lowp);
    }
    __syncthreads();
  }
  return info;
}

// In-CTA lower Cholesky of W; returns info (j+1 at the first non-positive pivot).
template <typename T>
__device__ int cta_chol(T* W, int n, int ld, int nb, T* smem, bool lowp) {
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

// x := U^{-1} L^{-1} x for n x q x (ld n): L lower (unit or not), U upper
// (non-unit) both in W (for Cholesky U = L^T has been written to the upper
// triangle).  32-row diagonal blocks are solved by one warp per column in
// registers; the rows after (before) a block are updated by all threads.
template <typename T>
__device__ void cta_solve(const T* W, int n, int ld, bool unit_lower, T* x, int q) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int j0 = 0; j0 < n; j0 += 32) {
    const int jb = min(32, n - j0);
    if (warp < q) {
      T* xc = x + (long)warp * n;
      T v = lane < jb ? xc[j0 + lane] : T(0);
      for (int jj = 0; jj < jb; ++jj) {
        if (!unit_lower && lane == jj) v = v / W[(j0 + jj) + (long)(j0 + jj) * ld];
        const T xj = __shfl_sync(0xffffffffu, v, jj);
        if (lane > jj && lane < jb) v = fma(-W[(j0 + lane) + (long)(j0 + jj) * ld], xj, v);
      }
      if (lane < jb) xc[j0 + lane] = v;
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < (n - j0 - jb) * q; idx += kBT) {
      const int r = j0 + jb + idx % (n - j0 - jb), c = idx / (n - j0 - jb);
      T s = x[r + (long)c * n];
      for (int jj = 0; jj < jb; ++jj) s = fma(-W[r + (long)(j0 + jj) * ld], x[j0 + jj + (long)c * n], s);
      x[r + (long)c * n] = s;
    }
    __syncthreads();
  }
  for (int j0 = ((n - 1) / 32) * 32; j0 >= 0; j0 -= 32) {
    const int jb = min(32, n - j0);
    if (warp < q) {
      T* xc = x + (long)warp * n;
      T v = lane < jb ? xc[j0 + lane] : T(0);
      for (int jj = jb - 1; jj >= 0; --jj) {
        if (lane == jj) v = v / W[(j0 + jj) + (long)(j0 + jj) * ld];
        const T xj = __shfl_sync(0xffffffffu, v, jj);
        if (lane < jj) v = fma(-W[(j0 + lane) + (long)(j0 + jj) * ld], xj, v);
      }
      if (lane < jb) xc[j0 + lane] = v;
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < j0 * q; idx += kBT) {
      const int r = idx % j0, c = idx / j0;
      T s = x[r + (long)c * n];
      for (int jj = 0; jj < jb; ++jj) s = fma(-W[r + (long)(j0 + jj) * ld], x[j0 + jj + (long)c * n], s);
      x[r + (long)c * n] = s;
    }
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
  if (threadIdx.x < q) {
    double m = 0.0;
    for (int r = 0; r < n; ++r) m = fmax(m, fabs(rhs[r + (long)threadIdx.x * n]));
    scale[threadIdx.x] = (m > 0 && m < INFINITY) ? m : 1.0;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n * q; i += kBT) {
    const int r = i % n, c = i / n;
    const int src = kind == 0 ? perm[r] : r;
    xt[i] = (T)(rhs[src + (long)c * n] / scale[c]);
  }
  __syncthreads();
  cta_solve<T>(W, n, n, kind == 0, xt, q);
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
  int mode;          // 0 solve, 1 features only
  int fallback;      // FP64 refactorization when refinement does not converge
  float* feat;       // mode 1: count x 16 features
};

__device__ double sys_berr(const double* A, int n, const double* X, const double* B, double* R,
                           int q, Shared& sh, double nA) {
  // R = B - A X (FP64), berr = max_c ||R_c|| / (nA ||X_c|| + ||B_c||)
  for (int r = threadIdx.x; r < n; r += kBT) {
    double acc[kBQ];
#pragma unroll
    for (int c = 0; c < kBQ; ++c) acc[c] = 0.0;
    for (int j = 0; j < n; ++j) {
      const double a = A[r + (long)j * n];
#pragma unroll
      for (int c = 0; c < kBQ; ++c)
        if (c < q) acc[c] = fma(a, X[j + (long)c * n], acc[c]);
    }
#pragma unroll
    for (int c = 0; c < kBQ; ++c)
      if (c < q) R[r + (long)c * n] = B[r + (long)c * n] - acc[c];
  }
  __syncthreads();
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
// transposed from W.
template <typename T>
__device__ void cta_solve_t(const T* W, int n, int ld, bool unit_lower, T* x) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int j0 = 0; j0 < n; j0 += 32) {
    const int jb = min(32, n - j0);
    if (warp == 0) {
      T v = lane < jb ? x[j0 + lane] : T(0);
      for (int jj = 0; jj < jb; ++jj) {
        if (lane == jj) v = v / W[(j0 + jj) + (long)(j0 + jj) * ld];
        const T xj = __shfl_sync(0xffffffffu, v, jj);
        if (lane > jj && lane < jb) v = fma(-W[(j0 + jj) + (long)(j0 + lane) * ld], xj, v);
      }
      if (lane < jb) x[j0 + lane] = v;
    }
    __syncthreads();
    for (int r = j0 + jb + threadIdx.x; r < n; r += kBT) {
      T acc = x[r];
      for (int jj = 0; jj < jb; ++jj) acc = fma(-W[(j0 + jj) + (long)r * ld], x[j0 + jj], acc);
      x[r] = acc;
    }
    __syncthreads();
  }
  for (int j0 = ((n - 1) / 32) * 32; j0 >= 0; j0 -= 32) {
    const int jb = min(32, n - j0);
    if (warp == 0) {
      T v = lane < jb ? x[j0 + lane] : T(0);
      for (int jj = jb - 1; jj >= 0; --jj) {
        if (!unit_lower && lane == jj) v = v / W[(j0 + jj) + (long)(j0 + jj) * ld];
        const T xj = __shfl_sync(0xffffffffu, v, jj);
        if (lane < jj) v = fma(-W[(j0 + jj) + (long)(j0 + lane) * ld], xj, v);
      }
      if (lane < jb) x[j0 + lane] = v;
    }
    __syncthreads();
    for (int r = threadIdx.x; r < j0; r += kBT) {
      T acc = x[r];
      for (int jj = 0; jj < jb; ++jj) acc = fma(-W[(j0 + jj) + (long)r * ld], x[j0 + jj], acc);
      x[r] = acc;
    }
    __syncthreads();
  }
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

template <typename T>
__device__ int factor_sys(T* W, int n, int kind, int nb, int* piv, Shared& sh, T* smem,
                          int smem_elems, bool lowp) {
  return kind == 0 ? cta_lu<T>(W, n, n, nb, piv, sh, smem, smem_elems, lowp)
                   : cta_chol<T>(W, n, n, nb, smem, lowp);
}

// The selector's 16 features of one system (written to p.feat[s * 16 ..]):
// norm ratios of A, an FP32 LU's growth and pivot spread, and a Hager /
// Higham 1-norm estimate of ||A^{-1}||_1 (LAPACK xLACON's iteration plus
// Higham's alternating vector) computed with that FP32 LU.
__device__ void compute_features(const BatchParams& p, const SysDesc& d, int s, const double* A,
                                 int n, double nA, float* Wf, int* piv, int* perm, float* v,
                                 Shared& sh, float* smf) {
  __shared__ float s_fv[16];
  double sum, mx, colmax = 0.0, rowmax = 0.0, amax = 0.0, dsum = 0.0;
  // column sums (||A||_1), row sums (||A||_inf), max |a|, diagonal weight
  block_sum_max(n, [&](int j) {
    double c = 0.0;
    for (int i = 0; i < n; ++i) c += fabs(A[i + (long)j * n]);
    return c;
  }, sh, &sum, &colmax);
  block_sum_max(n, [&](int i) {
    double r = 0.0;
    for (int j = 0; j < n; ++j) r += fabs(A[i + (long)j * n]);
    return r;
  }, sh, &sum, &rowmax);
  block_sum_max(n, [&](int j) {
    double m = 0.0;
    for (int i = 0; i < n; ++i) m = fmax(m, fabs(A[i + (long)j * n]));
    return m;
  }, sh, &sum, &amax);
  block_sum_max(n, [&](int i) { return fabs(A[i + (long)i * n]); }, sh, &dsum, &mx);
  // FP32 factorization
  for (long i = threadIdx.x; i < (long)n * n; i += kBT) Wf[i] = (float)A[i];
  __syncthreads();
  const int info = factor_sys<float>(Wf, n, d.kind, d.nb, piv, sh, smf,
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
      cta_solve<float>(Wf, n, n, d.kind == 0, y, 1);  // y = A^{-1} x
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
    cta_solve<float>(Wf, n, n, d.kind == 0, y, 1);
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
      p.feat[(long)s * 16 + k] = f;
    }
    BatchResult r{};
    r.info = info;
    r.berr = colmax * fmax(est, est2);  // the kappa_1 estimate
    p.out[s] = r;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kBT)
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
  const int q = p.q;
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
    {  // ||A||_F
      double acc = 0.0;
      for (long i = threadIdx.x; i < (long)n * n; i += kBT) acc = fma(A[i], A[i], acc);
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if ((threadIdx.x & 31) == 0) sh.red[threadIdx.x >> 5][0] = acc;
      __syncthreads();
      if (threadIdx.x == 0) {
        double v = 0.0;
        for (int w = 0; w < kBT / 32; ++w) v += sh.red[w][0];
        s_na = sqrt(v);
      }
      __syncthreads();
    }
    const double nA = s_na;
    bool done = false;
    if (p.mode == 1) {
      compute_features(p, d, s, A, n, nA, Wf, piv, perm, reinterpret_cast<float*>(V), sh,
                       reinterpret_cast<float*>(smem_raw));
      continue;
    }
    if (d.prec >= 1) {
      // FP32 factors (BF16 operand products for prec 2) + FP64 refinement
      float* smf = reinterpret_cast<float*>(smem_raw);
      for (long i = threadIdx.x; i < (long)n * n; i += kBT) Wf[i] = (float)A[i];
      __syncthreads();
      const int info = factor_sys<float>(Wf, n, d.kind, d.nb, piv, sh, smf,
                                         kSmemPanel / (int)sizeof(float), d.prec == 2);
      res.info = info;
      if (info == 0) {
        if (d.kind == 0)
          cta_perm_from_swaps(piv, n, perm, reinterpret_cast<int*>(smem_raw),
                              kSmemPanel / (int)sizeof(int));
        else
          cta_mirror_lower(Wf, n, n);
        float* vf = reinterpret_cast<float*>(V);
        cta_apply_inverse<float>(Wf, n, d.kind, perm, B, X, vf, nullptr, q, false, s_sc);
        double prev = INFINITY;
        for (int it = 0;; ++it) {
          const double be = sys_berr(A, n, X, B, R, q, sh, nA);
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
            break;
          }
          if (it >= p.max_iters) break;
          prev = be;
          for (int i = threadIdx.x; i < n * q; i += kBT) Xprev[i] = X[i];
          cta_apply_inverse<float>(Wf, n, d.kind, perm, R, X, vf, nullptr, q, true, s_sc);
        }
      }
    }
    if (!done && (p.fallback || d.prec == 0)) {
      // FP64 factors: the plain path, or the fallback
      res.fell_back = d.prec >= 1 ? 1 : 0;
      double* smd = reinterpret_cast<double*>(smem_raw);
      for (long i = threadIdx.x; i < (long)n * n; i += kBT) Wd[i] = A[i];
      __syncthreads();
      const int nb64 = max(1, min(d.nb, (kSmemPanel / 8 - 64 * 64) / max(n, 1)));
      const int info = factor_sys<double>(Wd, n, d.kind, nb64, piv, sh, smd,
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
    }
    res.converged = done ? 1 : 0;
    if (threadIdx.x == 0) p.out[s] = res;
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
  unsigned* d_ticket = nullptr;
  BatchResult* d_out = nullptr;
  int grid = 0;
  long ws_elems = 0;
  BatchParams prm{};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  double flops = 0;
};

static int pick_nb(int n, int prec, const int* nb_table) {
  // size buckets: <=32, <=64, <=128, <=256, <=512, <=1024, <=2048, larger
  int b = 0;
  for (int lim = 32; b < 7 && n > lim; lim *= 2) ++b;
  int nb = nb_table ? nb_table[b] : 32;
  if (nb <= 0) nb = 32;
  const int es = prec == 1 ? 4 : 8;
  // panel (n x nb) plus a 64-column staging tile within the budget
  const int cap = (kSmemPanel / es - 64 * 64) / std::max(n, 1);
  nb = std::min(nb, std::max(cap, 1));
  nb = std::max(1, std::min(nb, 64));
  return nb;
}

cudaError_t batched_plan(Context* ctx, int count, const int* h_n, const int* h_kind,
                         const int* h_prec, int q, const double* A, const double* B, double* X,
                         const int* nb_table, int ctas_per_sm, double tol, int max_iters,
                         int fallback, int mode, float* feat, BatchPlan** out) {
  *out = nullptr;
  if (q < 1 || q > kBQ) return cudaErrorInvalidValue;
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
    s.nb = pick_nb(s.n, s.prec, nb_table);
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
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    const double ca = (double)desc[a].n * desc[a].n * desc[a].n * (desc[a].prec == 0 ? 16 : 1);
    const double cb = (double)desc[b].n * desc[b].n * desc[b].n * (desc[b].prec == 0 ? 16 : 1);
    return ca > cb;
  });
  P->grid = std::max(1, std::min(count, ctx->num_sms * std::max(1, ctas_per_sm)));
  P->ws_elems = (long)nmax * nmax;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e == cudaSuccess) e = cudaMalloc(&P->d_desc, sizeof(SysDesc) * count);
  if (e == cudaSuccess) e = cudaMalloc(&P->d_order, sizeof(int) * count);
  if (e == cudaSuccess) e = cudaMalloc(&P->d_wsf, sizeof(float) * P->ws_elems * P->grid);
  if (e == cudaSuccess) e = cudaMalloc(&P->d_wsd, sizeof(double) * P->ws_elems * P->grid);
  if (e == cudaSuccess) e = cudaMalloc(&P->d_piv, sizeof(int) * 2 * (long)nmax * P->grid);
  if (e == cudaSuccess) e = cudaMalloc(&P->d_vec, sizeof(double) * 3 * (long)nmax * q * P->grid);
  if (e == cudaSuccess) e = cudaMalloc(&P->d_ticket, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMalloc(&P->d_out, sizeof(BatchResult) * count);
  if (e == cudaSuccess)
    e = cudaMemcpy(P->d_desc, desc.data(), sizeof(SysDesc) * count, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(P->d_order, order.data(), sizeof(int) * count, cudaMemcpyHostToDevice);
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
  prm.mode = mode;
  prm.fallback = fallback;
  prm.feat = feat;
  e = cudaFuncSetAttribute(batched_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           kSmemPanel);
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
    batched_solve_kernel<<<P->grid, kBT, kSmemPanel, cs>>>(prm);
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
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(P->ctx->stream);
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
  cudaFree(P->d_ticket);
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
  *plan = nullptr;
  elgb::BatchPlan* p = nullptr;
  cudaError_t e = elgb::batched_plan(static_cast<elgb::Context*>(ctx), count, n, o.kind,
                                     o.precision, nrhs, A, B, X, o.nb_table, o.ctas_per_sm, o.tol,
                                     o.max_iters, o.no_fallback ? 0 : 1,
                                     o.features_only ? 1 : 0, o.features, &p);
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
