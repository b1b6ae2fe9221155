// The refinement's residual R = B - A X (and its GMRES product W = A Z) to
// FP64 accuracy on the FP32 pipe.  GB300 issues FP32 FMAs at ~64x its FP64
// rate, and the FP64 residual of the mixed-precision solve (2 n^2 q FMAs,
// q <= 16) is bound by the FP64 pipe, not by reading A.
//
// Arithmetic ("double-float", two FP32 words per value; the error-free
// transformations of Dekker's product and Knuth's TwoSum):
//   * A is split once per solve into FP32 words a = ah + al + O(2^-48 |a|)
//     (split_a_kernel, in the same pass that makes the FP32 copy the
//     factorization overwrites and the norms of A);
//   * x, per call, scaled by a power of two per column so that the largest
//     product |a x| is O(1) (no FP32 overflow, no underflow of the terms
//     that matter), then split the same way;
//   * per product: p = ah xh rounded, its exact error e = fma(ah, xh, -p),
//     the cross terms ah xl + al xh (al xl ~ 2^-48 is dropped);
//   * the running sum S takes p with TwoSum, whose exact error goes to the
//     low word L with e and the cross terms; (S, L) is renormalised by
//     TwoSum every 4 columns, which leaves |L| <= ulp(S) / 2, and S alone
//     is flushed into an FP64 accumulator every 32 columns (one conversion
//     and one FP64 add per right-hand side; L carries on and is added at
//     the end of the chunk).  L's own FP32 rounding is the leading error,
//     about 2^-48 sqrt(32 * 4 / n) of sum_j |a_ij x_j| per row.
// Every multiply and add of the transformations is an explicit _rn
// intrinsic, so no contraction into an FMA can break them.  A bit-faithful
// CPU emulation against correctly rounded residuals (N(0,1) A, x near the
// solution): at most 6 ulps of sum_j |a_ij x_j| + |b_i| per row at
// n = 1024 .. 4096 and fewer beyond (18 at n = 100).
//
// The sum over columns is split into chunks (one CTA per 128 rows x chunk);
// the chunks' FP64 partial sums are added in a fixed order by the finish
// kernel, so results are reproducible run to run.
#include <algorithm>

#include "kernels.h"

namespace elgb {

namespace {

constexpr int kDfRows = 128;  // rows (threads) per CTA
constexpr int kDfStage = 64;  // columns of X staged in shared memory at once
constexpr int kDfRenorm = 4;   // columns between renormalisations of (S, L)
constexpr int kDfFlush = 32;   // columns between flushes into FP64

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bp = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
}

// One product a x into (S, L), a = ah + al, x = xh + xl.
__device__ __forceinline__ void df_madd(float ah, float al, float xh, float xl, float& S,
                                        float& L) {
  const float p = __fmul_rn(ah, xh);
  const float e = __fmaf_rn(ah, xh, -p);
  float t, err;
  two_sum(S, p, t, err);
  S = t;
  L = __fmaf_rn(ah, xl, L);
  L = __fmaf_rn(al, xh, L);
  L = __fadd_rn(L, e);
  L = __fadd_rn(L, err);
}

// Power-of-two exponent k with 2^k <= |v| < 2^(k+1); 0 for 0, inf or NaN.
__device__ __forceinline__ int exp2_of(double v) {
  return (v == 0.0 || !isfinite(v)) ? 0 : ilogb(v);
}

// (fl32(v), fl32(v - fl32(v))) for |v| in [2^-74, 2^127) by integer operations
// on v's two 32-bit halves, bit-identical to the two cvt.rn.f32.f64
// conversions.  GB300 runs FP64 conversions -- and 64-bit integer shifts --
// on its FP64 pipe, which bound the split at a third of HBM speed; on
// 32-bit halves it streams at HBM speed.  With v = (-1)^s m 2^(E-1075), m the
// 53-bit significand: the high word keeps m's top 24 bits rounded to
// nearest even (a carry out of them moves into the exponent), and
// v - fl32(v) = (-1)^s d 2^(E-1075) exactly, with d the signed remainder
// (|d| <= 2^28), so its FP32 rounding is that of the integer d times a power
// of two.  Returns false outside the range (zero, subnormal, huge, inf, NaN):
// the caller converts in FP64 there.
__device__ __forceinline__ bool split_bits(double v, float& hi, float& lo) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const unsigned bh = (unsigned)(b >> 32), bl = (unsigned)b;
  const int E = (int)((bh >> 20) & 0x7ffu);
  if (E < 949 || E > 1149) return false;
  const unsigned q = (((bh & 0xFFFFFu) | 0x100000u) << 3) | (bl >> 29);  // top 24 bits of m
  const unsigned rem = bl & 0x1FFFFFFFu;
  const unsigned inc = (rem > 0x10000000u || (rem == 0x10000000u && (q & 1u))) ? 1u : 0u;
  const unsigned sgn = bh >> 31;
  hi = __uint_as_float((sgn << 31) | (((unsigned)(E - 896) << 23) + (q + inc - 0x800000u)));
  const int d = (int)rem - (int)(inc << 29);
  lo = __fmul_rn(__int2float_rn(sgn ? -d : d), __uint_as_float((unsigned)(E - 948) << 23));
  return true;
}

}  // namespace

// a -> Af = fl32(a) (the copy the factorization overwrites; skipped when Af
// is null), ah = fl32(a), al = fl32(a - ah); per CTA the sum of squares and
// max |a| of the entries it visited (fixed-order reductions).  The work is
// cut into chunks of 1024 rows of one column, taken in column-major order
// by a grid-stride loop, so the CTAs running at once stream one contiguous
// stretch of A and of the outputs.  Four rows per thread are in flight at
// once; the only FP64-pipe work per entry is the sum of squares.
__global__ void __launch_bounds__(256)
split_a_kernel(const double* __restrict__ A, long lda, int n, float* __restrict__ Af,
               float* __restrict__ Ahi, float* __restrict__ Alo, double* __restrict__ part) {
  __shared__ double s_sq[256], s_mx[256];
  double sq = 0.0;
  unsigned long long mxb = 0ull;  // bits of max |a| (non-negative doubles order as integers)
  const int rch = ceil_div(n, 1024);
  const long nchunks = (long)rch * n;
  for (long c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const int j = (int)(c / rch);
    const int i0 = (int)(c - (long)j * rch) * 1024;
    const double* a = A + (long)j * lda + i0;
    const long o = (long)j * n + i0;
    const int nr = min(1024, n - i0);
    double v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int r = threadIdx.x + 256 * u;
      v[u] = r < nr ? __ldcs(a + r) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int r = threadIdx.x + 256 * u;
      if (r < nr) {
        float h, l;
        if (!split_bits(v[u], h, l)) {
          h = (float)v[u];
          l = (float)(v[u] - (double)h);
        }
        if (Af) Af[o + r] = h;
        Ahi[o + r] = h;
        Alo[o + r] = l;
        sq = fma(v[u], v[u], sq);
        const unsigned long long ab =
            (unsigned long long)__double_as_longlong(v[u]) & 0x7FFFFFFFFFFFFFFFull;
        if (ab <= 0x7FF0000000000000ull && ab > mxb) mxb = ab;  // NaN never counts
      }
    }
  }
  s_sq[threadIdx.x] = sq;
  s_mx[threadIdx.x] = __longlong_as_double((long long)mxb);
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      s_sq[threadIdx.x] += s_sq[threadIdx.x + s];
      s_mx[threadIdx.x] = fmax(s_mx[threadIdx.x], s_mx[threadIdx.x + s]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s_sq[0];
    part[2 * blockIdx.x + 1] = s_mx[0];
  }
}

// out[0] = ||A||_F^2, out[1] = max |a|: thread t adds the partials t, t + 256,
// ... in order, then a fixed tree (reproducible run to run).
__global__ void __launch_bounds__(256)
split_a_finish_kernel(const double* __restrict__ part, int nblk, double* __restrict__ out) {
  __shared__ double s_sq[256], s_mx[256];
  double sq = 0.0, mx = 0.0;
  for (int b = threadIdx.x; b < nblk; b += 256) {
    sq += part[2 * b];
    mx = fmax(mx, part[2 * b + 1]);
  }
  s_sq[threadIdx.x] = sq;
  s_mx[threadIdx.x] = mx;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      s_sq[threadIdx.x] += s_sq[threadIdx.x + s];
      s_mx[threadIdx.x] = fmax(s_mx[threadIdx.x], s_mx[threadIdx.x + s]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = s_sq[0];
    out[1] = s_mx[0];
  }
}

// Column c of X (c < q; zero columns up to Q): scale s_c = 2^-(k_A + k_x)
// with 2^k_A <= max|a| and 2^k_x <= max|x_c|, then Xs[j Q + c] = (xh, xl)
// of s_c x_jc; inv[c] = 1 / s_c (exact).  One CTA per column.
__global__ void __launch_bounds__(256)
split_x_kernel(const double* __restrict__ X, long ldx, int n, int q, int Q,
               const double* __restrict__ amaxA, float2* __restrict__ Xs,
               double* __restrict__ inv) {
  __shared__ double s_mx[256];
  const int c = blockIdx.x;
  double mx = 0.0;
  if (c < q)
    for (int i = threadIdx.x; i < n; i += blockDim.x) mx = fmax(mx, fabs(X[i + (long)c * ldx]));
  s_mx[threadIdx.x] = mx;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) s_mx[threadIdx.x] = fmax(s_mx[threadIdx.x], s_mx[threadIdx.x + s]);
    __syncthreads();
  }
  const int k = exp2_of(*amaxA) + exp2_of(s_mx[0]);
  const double sc = ldexp(1.0, -k);
  if (threadIdx.x == 0) inv[c] = ldexp(1.0, k);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double v = c < q ? X[i + (long)c * ldx] * sc : 0.0;
    const float h = (float)v;
    Xs[(long)i * Q + c] = make_float2(h, (float)(v - (double)h));
  }
}

// partial[(chunk Q + c) n + i] = sum over this chunk's columns j of
// a_ij (s_c x_jc), in double-float words whose high word is flushed to FP64
// every 32 columns.
template <int Q>
__global__ void __launch_bounds__(kDfRows)
df_residual_partial_kernel(int n, const float* __restrict__ Ahi, const float* __restrict__ Alo,
                           const float2* __restrict__ Xs, int kc,
                           double* __restrict__ partial) {
  __shared__ __align__(16) float2 sx[2][kDfStage * Q];
  const int i = blockIdx.x * kDfRows + threadIdx.x;
  const int chunk = blockIdx.y;
  const int j0 = chunk * kc, j1 = min(j0 + kc, n);
  const bool row = i < n;
  const long ia = row ? i : 0;

  // stage s holds columns [js, js + kDfStage) of Xs (float2 per (j, c))
  auto stage_copy = [&](int buf, int js) {
    const int nj = min(kDfStage, j1 - js);
    // 16-byte vectors (two float2); an odd count (Q = 1) copies one float2
    // past the stage, which Xs holds (it is sized for 64-column stages + 1)
    const int nvec = (nj * Q + 1) / 2;
    const float4* src = reinterpret_cast<const float4*>(Xs + (long)js * Q);
    float4* dst = reinterpret_cast<float4*>(sx[buf]);
    for (int v = threadIdx.x; v < nvec; v += kDfRows)
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                       (unsigned)__cvta_generic_to_shared(dst + v)),
                   "l"(src + v)
                   : "memory");
    asm volatile("cp.async.commit_group;" ::: "memory");
  };

  double acc[Q];
  float L[Q];
#pragma unroll
  for (int c = 0; c < Q; ++c) {
    acc[c] = 0.0;
    L[c] = 0.f;
  }
  if (j0 < j1) stage_copy(0, j0);
  int buf = 0;
  for (int js = j0; js < j1; js += kDfStage, buf ^= 1) {
    const int nj = min(kDfStage, j1 - js);
    if (js + kDfStage < j1) {
      stage_copy(buf ^ 1, js + kDfStage);
      asm volatile("cp.async.wait_group 1;" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    }
    __syncthreads();
    float S[Q];
#pragma unroll
    for (int c = 0; c < Q; ++c) S[c] = 0.f;
    const float* ph = Ahi + ia + (long)js * n;
    const float* pl = Alo + ia + (long)js * n;
    const float2* xs = sx[buf];
    int jj = 0;
    for (; jj + 4 <= nj; jj += 4) {
      float ah[4], al[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        ah[u] = row ? __ldcs(ph + (long)(jj + u) * n) : 0.f;
        al[u] = row ? __ldcs(pl + (long)(jj + u) * n) : 0.f;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
#pragma unroll
        for (int c = 0; c < Q; ++c) {
          const float2 x = xs[(jj + u) * Q + c];
          df_madd(ah[u], al[u], x.x, x.y, S[c], L[c]);
        }
      }
      static_assert(kDfRenorm == 4, "one renormalisation per unrolled group of 4 columns");
#pragma unroll
      for (int c = 0; c < Q; ++c) two_sum(S[c], L[c], S[c], L[c]);
      if (((jj + 4) % kDfFlush) == 0) {
#pragma unroll
        for (int c = 0; c < Q; ++c) {
          acc[c] += (double)S[c];
          S[c] = 0.f;
        }
      }
    }
    for (; jj < nj; ++jj) {
      const float ah = row ? ph[(long)jj * n] : 0.f;
      const float al = row ? pl[(long)jj * n] : 0.f;
#pragma unroll
      for (int c = 0; c < Q; ++c) {
        const float2 x = xs[jj * Q + c];
        df_madd(ah, al, x.x, x.y, S[c], L[c]);
      }
    }
#pragma unroll
    for (int c = 0; c < Q; ++c) acc[c] += (double)S[c];
    __syncthreads();  // every thread is done with sx[buf] before it is refilled
  }
#pragma unroll
  for (int c = 0; c < Q; ++c) acc[c] += (double)L[c];
  if (row)
#pragma unroll
    for (int c = 0; c < Q; ++c) partial[((long)chunk * Q + c) * n + i] = acc[c];
}

// R(:, c) = B(:, c) - inv[c] * sum of the chunks' partials (B == nullptr:
// R = A X), c < q; inv[c] is a power of two, so the unscaling is exact.
__global__ void df_residual_finish_kernel(int n, int q, int Q, int nchunks,
                                          const double* __restrict__ partial,
                                          const double* __restrict__ inv,
                                          const double* __restrict__ B, long ldb,
                                          double* __restrict__ R, long ldr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (i >= n || c >= q) return;
  double s = 0.0;
  for (int ch = 0; ch < nchunks; ++ch) s += partial[((long)ch * Q + c) * n + i];
  s *= inv[c];
  R[i + (long)c * ldr] = B ? B[i + (long)c * ldb] - s : s;
}

size_t df_split_parts(int n) { return (size_t)std::max(1, std::min(n, 4096)); }

cudaError_t launch_split_a(const double* A, long lda, int n, float* Af, float* Ahi, float* Alo,
                           double* part, double* out, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  const int nblk = (int)df_split_parts(n);
  split_a_kernel<<<nblk, 256, 0, stream>>>(A, lda, n, Af, Ahi, Alo, part);
  split_a_finish_kernel<<<1, 256, 0, stream>>>(part, nblk, out);
  return cudaGetLastError();
}

int df_q(int q) { return q <= 1 ? 1 : q <= 2 ? 2 : q <= 4 ? 4 : q <= 8 ? 8 : 16; }

int df_chunks(int n) {
  // ~16 column chunks: 16 x n / 128 CTAs (4096 at n = 32768), chunk widths
  // a multiple of the staging width
  const int kc = std::max(kDfStage, ceil_div(ceil_div(n, 16), kDfStage) * kDfStage);
  return ceil_div(n, kc);
}

size_t df_residual_partial_doubles(int n) { return (size_t)df_chunks(n) * 16 * (size_t)n; }

cudaError_t launch_residual_df(int n, int q, const float* Ahi, const float* Alo,
                               const double* amaxA, const double* X, long ldx, const double* B,
                               long ldb, double* R, long ldr, float2* Xs, double* inv,
                               double* partial, cudaStream_t stream) {
  if (n <= 0 || q <= 0) return cudaSuccess;
  if (q > 16) return cudaErrorInvalidValue;
  const int Q = df_q(q);
  split_x_kernel<<<Q, 256, 0, stream>>>(X, ldx, n, q, Q, amaxA, Xs, inv);
  const int nch = df_chunks(n);
  const int kc = std::max(kDfStage, ceil_div(ceil_div(n, 16), kDfStage) * kDfStage);
  const dim3 grid(ceil_div(n, kDfRows), nch);
  switch (Q) {
    case 1: df_residual_partial_kernel<1><<<grid, kDfRows, 0, stream>>>(n, Ahi, Alo, Xs, kc, partial); break;
    case 2: df_residual_partial_kernel<2><<<grid, kDfRows, 0, stream>>>(n, Ahi, Alo, Xs, kc, partial); break;
    case 4: df_residual_partial_kernel<4><<<grid, kDfRows, 0, stream>>>(n, Ahi, Alo, Xs, kc, partial); break;
    case 8: df_residual_partial_kernel<8><<<grid, kDfRows, 0, stream>>>(n, Ahi, Alo, Xs, kc, partial); break;
    default: df_residual_partial_kernel<16><<<grid, kDfRows, 0, stream>>>(n, Ahi, Alo, Xs, kc, partial); break;
  }
  df_residual_finish_kernel<<<dim3(ceil_div(n, 256), q), 256, 0, stream>>>(n, q, Q, nch, partial,
                                                                          inv, B, ldb, R, ldr);
  return cudaGetLastError();
}

}  // namespace elgb
