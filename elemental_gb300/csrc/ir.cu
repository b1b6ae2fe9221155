// Mixed-precision solves: A X = B with A, B, X in FP64, the factorization
// done in FP32 storage with tensor-core updates (BF16, TF32 or TF32x3
// products), accuracy recovered by iterative refinement with an FP64
// residual.
//
//   LU-IR    follows the refinement loop of the reference's
//            refined_solve::Single (include/El/lapack_like/solve/Refined.hpp:44-119):
//            x = A^{-1} b; repeat r = b - A x, stop when small, dx = A^{-1} r,
//            accept x + dx only if the residual decreases.
//   GMRES-IR follows the reference's flexible GMRES, fgmres::Single
//            (include/El/lapack_like/solve/FGMRES.hpp:37-290): right
//            preconditioning by the low-precision LU solve, FP64 Arnoldi
//            (here classical Gram-Schmidt applied twice instead of modified
//            Gram-Schmidt: same span, one reduction per pass), Givens
//            rotations on the Hessenberg matrix, restarts with an explicit
//            FP64 residual.  All right-hand sides advance in lockstep.
// The stopping test is the normwise backward error
//   ||b - A x||_2 / (||A||_F ||x||_2 + ||b||_2) <= tol   (per column),
// and a plain FP64 LU (getrf / getrs) takes over when the low-precision
// factor is singular or refinement stalls.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/elgb300.h"
#include "driver.h"
#include "kernels.h"
#include "tc_gemm.h"
#include "trsv.h"

namespace elgb {

namespace {

constexpr int kRowChunk = 2048;  // rows per partial sum in the reductions

__global__ void cvt_f64_f32_kernel(const double* __restrict__ src, long lds, int m, int n,
                                   float* __restrict__ dst, long ldd) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  for (int j = blockIdx.y; j < n; j += gridDim.y) dst[i + (long)j * ldd] = (float)src[i + (long)j * lds];
}

// Per-column max |R(:, c)| over row chunks (partial), then finish.
__global__ void col_absmax_partial_kernel(const double* __restrict__ R, long ldr, int n,
                                          double* __restrict__ partial) {
  __shared__ double s[256];
  const int c = blockIdx.y, ch = blockIdx.x;
  const int r0 = ch * kRowChunk, r1 = min(r0 + kRowChunk, n);
  double v = 0.0;
  for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) v = fmax(v, fabs(R[r + (long)c * ldr]));
  s[threadIdx.x] = v;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] = fmax(s[threadIdx.x], s[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[(long)c * gridDim.x + ch] = s[0];
}

__global__ void col_absmax_finish_kernel(const double* __restrict__ partial, int nch, int q,
                                         double* __restrict__ scale) {
  const int c = threadIdx.x;
  if (c >= q) return;
  double v = 0.0;
  for (int ch = 0; ch < nch; ++ch) v = fmax(v, partial[(long)c * nch + ch]);
  scale[c] = (v > 0.0 && v < INFINITY) ? v : 1.0;
}

// Rf(i, c) = R(perm[i], c) / scale[c]  (row permutation P R fused with the
// FP64 -> FP32 scaling)
__global__ void scale_perm_to_f32_kernel(const double* __restrict__ R, long cstride, int n,
                                         const int* __restrict__ perm,
                                         const double* __restrict__ scale,
                                         float* __restrict__ Rf, long ldf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (i < n)
    Rf[i + (long)c * ldf] =
        (float)(R[perm[i] + (long)c * cstride] / (scale ? scale[c] : 1.0));
}

// Rf(:, c) = R(:, c) / scale[c]  (FP64 -> FP32); column c of R starts at
// R + c * cstride.
__global__ void scale_to_f32_kernel(const double* __restrict__ R, long cstride, int n,
                                    const double* __restrict__ scale, float* __restrict__ Rf,
                                    long ldf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (i < n) Rf[i + (long)c * ldf] = (float)(R[i + (long)c * cstride] / (scale ? scale[c] : 1.0));
}

// X(:, c) (+)= scale[c] * Rf(:, c)   (accumulate = 0 overwrites)
__global__ void f32_axpy_kernel(double* __restrict__ X, long cstride, int n,
                                const float* __restrict__ Rf, long ldf,
                                const double* __restrict__ scale, int accumulate) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (i >= n) return;
  const double v = (double)Rf[i + (long)c * ldf] * (scale ? scale[c] : 1.0);
  double* x = X + i + (long)c * cstride;
  *x = accumulate ? *x + v : v;
}

// Lockstep Gram-Schmidt pieces: column c owns the basis V_c (k vectors of
// length n, vector i at V + c * vcs + i * n) and the vector W(:, c).
// H[c * hld + i] = <V_c(:, i), W(:, c)>, deterministic two-stage.
constexpr int kMaxBasis = 64;

__global__ void __launch_bounds__(256)
multi_dot_partial_kernel(const double* __restrict__ V, long vcs, int n, int k,
                         const double* __restrict__ W, long ldw,
                         double* __restrict__ partial) {
  __shared__ double red[kMaxBasis][9];
  const int ch = blockIdx.x, c = blockIdx.y;
  const int r0 = ch * kRowChunk, r1 = min(r0 + kRowChunk, n);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const double* Vc = V + (long)c * vcs;
  for (int i0 = 0; i0 < k; i0 += 16) {
    double acc[16];
#pragma unroll
    for (int t = 0; t < 16; ++t) acc[t] = 0.0;
    for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
      const double w = W[r + (long)c * ldw];
#pragma unroll
      for (int t = 0; t < 16; ++t)
        if (i0 + t < k) acc[t] = fma(Vc[r + (long)(i0 + t) * n], w, acc[t]);
    }
#pragma unroll
    for (int t = 0; t < 16; ++t) {
      double v = acc[t];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0 && i0 + t < k) red[i0 + t][warp] = v;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < k; i += blockDim.x) {
    double v = 0.0;
    for (int w = 0; w < 8; ++w) v += red[i][w];
    partial[((long)c * gridDim.x + ch) * kMaxBasis + i] = v;
  }
}

__global__ void multi_dot_finish_kernel(const double* __restrict__ partial, int nch, int k,
                                        double* __restrict__ H, int hld, int accumulate) {
  const int c = blockIdx.x, i = threadIdx.x;
  if (i >= k) return;
  double v = 0.0;
  for (int ch = 0; ch < nch; ++ch) v += partial[((long)c * nch + ch) * kMaxBasis + i];
  H[(long)c * hld + i] = accumulate ? H[(long)c * hld + i] + v : v;
}

// W(:, c) -= sum_{i<k} V_c(:, i) * H[c * hld + i]
__global__ void multi_axpy_kernel(const double* __restrict__ V, long vcs, int n, int k,
                                  const double* __restrict__ H, int hld, double* __restrict__ W,
                                  long ldw, double sign) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (r >= n) return;
  const double* Vc = V + (long)c * vcs;
  double s = 0.0;
  for (int i = 0; i < k; ++i) s = fma(Vc[r + (long)i * n], H[(long)c * hld + i], s);
  W[r + (long)c * ldw] -= sign * s;
}

// dst(:, c) = src(:, c) * f[c]
__global__ void col_scale_copy_kernel(const double* __restrict__ src, long scs, int n,
                                      const double* __restrict__ f, double* __restrict__ dst,
                                      long dcs) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (r < n) dst[r + (long)c * dcs] = src[r + (long)c * scs] * f[c];
}

struct Ws {
  float* Af;
  int* ipiv;
  int* perm;
  double* R;
  double* Xprev;
  float* Rf;
  double* scale;
  double* part;      // col partials / residual partials
  double* rpart;
  double* sums;      // [4][q + 1]
  double* colout;    // [n + 1] column sums of squares of A
  double* V;         // GMRES
  double* Z;
  double* W;
  double* H;         // device [q][restart + 1]
  double* dpart;
  float* Dl;         // inverted 64 x 64 diagonal blocks of L (unit lower)
  float* Du;         // ... and of U
  unsigned long long* tags;  // words the one-launch triangular solves publish
  unsigned* ticket;
  unsigned epoch;
  // double-float residual (residual_df.cu): FP32 words of A, the scaled
  // split X, per-column unscaling, partial sums, ||A||_F^2 and max |a|
  float* Ahi;
  float* Alo;
  float2* Xs;
  double* xinv;
  double* dfpart;
  double* spart;
  double* astat;
  bool df;           // residuals in double-float arithmetic
};

size_t al(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace

// Host-side sums helper: sum of squares per column of an n x q block.
static cudaError_t colnorm2(Context* ctx, const double* X, long ld, int n, int q, double* dsum,
                            double* part, std::vector<double>& host) {
  cudaError_t e = launch_col_sumsq<double>(X, ld, n, q, dsum, part, ctx->stream);
  if (e != cudaSuccess) return e;
  ctx->launches += 2;
  host.resize(q + 1);
  e = cudaMemcpyAsync(host.data(), dsum, sizeof(double) * (q + 1), cudaMemcpyDeviceToHost,
                      ctx->stream);
  if (e != cudaSuccess) return e;
  e = cudaStreamSynchronize(ctx->stream);
  for (auto& v : host) v = std::sqrt(v);
  return e;
}

#define IR_CHECK(x)                        \
  do {                                     \
    cudaError_t e_ = (x);                  \
    if (e_ != cudaSuccess) return e_;      \
  } while (0)

// The low-precision preconditioner application: D = (P^T L U)^{-1} R in
// FP32 (columns scaled by their max-abs to stay in range), D into X either
// added (accumulate) or stored.
static cudaError_t lowprec_solve(Context* ctx, int n, int q, Ws& w, const double* R,
                                 long rcs, double* X, long xcs, bool accumulate, bool scale) {
  dim3 g((n + 255) / 256, q);
  const int nch = (n + kRowChunk - 1) / kRowChunk;
  if (scale) {
    col_absmax_partial_kernel<<<dim3(nch, q), 256, 0, ctx->stream>>>(R, rcs, n, w.part);
    col_absmax_finish_kernel<<<1, 32, 0, ctx->stream>>>(w.part, nch, q, w.scale);
    ctx->launches += 2;
  }
  scale_perm_to_f32_kernel<<<g, 256, 0, ctx->stream>>>(R, rcs, n, w.perm,
                                                       scale ? w.scale : nullptr, w.Rf, n);
  ctx->launches += 1;
  IR_CHECK(cudaGetLastError());
  // (P^T L U)^{-1}: L then U, each one launch
  const int pi = ctx->prof_begin(ctx->stream, ELGB_PROF_SOLVE);
  IR_CHECK(launch_trsv_persistent<float>(w.Af, n, w.Dl, w.Rf, n, n, q, true, w.ticket, w.tags,
                                         ++w.epoch, ctx->status, ctx->num_sms, ctx->stream));
  IR_CHECK(launch_trsv_persistent<float>(w.Af, n, w.Du, w.Rf, n, n, q, false, w.ticket,
                                         w.tags, ++w.epoch, ctx->status, ctx->num_sms,
                                         ctx->stream));
  ctx->launches += 2;
  ctx->prof_end(pi, ctx->stream, ELGB_PROF_SOLVE, 2.0 * n * (double)n * q,
                4.0 * n * (double)n);
  f32_axpy_kernel<<<g, 256, 0, ctx->stream>>>(X, xcs, n, w.Rf, n, scale ? w.scale : nullptr,
                                              accumulate ? 1 : 0);
  ctx->launches += 1;
  return cudaGetLastError();
}

static void backward_errors(const std::vector<double>& nr, const std::vector<double>& nx,
                            const std::vector<double>& nb, double nA, int q,
                            std::vector<double>& out) {
  out.resize(q);
  for (int c = 0; c < q; ++c) {
    const double den = nA * nx[c] + nb[c];
    out[c] = den > 0 ? nr[c] / den : (nr[c] > 0 ? INFINITY : 0.0);
  }
}

// R = B - A X (B == nullptr: R = A X) for q <= 16 columns: double-float on
// the FP32 pipe, or FP64.
static cudaError_t ir_residual(Context* ctx, const Ws& w, int n, int q, const double* A,
                               long lda, const double* X, long ldx, const double* B, long ldb,
                               double* R, long ldr) {
  const int pr = ctx->prof_begin(ctx->stream, ELGB_PROF_RESIDUAL);
  cudaError_t e;
  if (w.df) {
    e = launch_residual_df(n, q, w.Ahi, w.Alo, w.astat + 1, X, ldx, B, ldb, R, ldr, w.Xs,
                           w.xinv, w.dfpart, ctx->stream);
    ctx->launches += 3;
  } else {
    e = launch_residual_f64(n, q, A, lda, X, ldx, B, ldb, R, ldr, w.rpart, ctx->stream);
    ctx->launches += 2;
  }
  ctx->prof_end(pr, ctx->stream, ELGB_PROF_RESIDUAL, 2.0 * n * (double)n * q,
                8.0 * n * (double)n);
  return e;
}

cudaError_t refined_solve(Context* ctx, int n, const double* A, long lda, int nrhs,
                          const double* B, long ldb, double* X, long ldx,
                          const ElGBRefineCtrl& cin, ElGBRefineInfo* info) {
  ElGBRefineCtrl c = cin;
  if (c.tol <= 0) c.tol = n * 2.220446049250313e-16;
  if (c.max_iters <= 0) c.max_iters = 30;
  if (c.restart <= 0) c.restart = 20;
  if (c.restart > kMaxBasis - 1) c.restart = kMaxBasis - 1;
  if (c.nb <= 0) c.nb = 512;
  ElGBRefineInfo inf{};
  inf.precision = c.precision;
  IR_CHECK(cudaSetDevice(ctx->device));
  if (n == 0 || nrhs == 0) {
    inf.converged = 1;
    if (info) *info = inf;
    return cudaSuccess;
  }
  const int tc_kind = c.precision == ELGB_PREC_BF16   ? kTcBF16
                      : c.precision == ELGB_PREC_TF32 ? kTcTF32
                      : c.precision == ELGB_PREC_FP8  ? kTcFP8
                                                      : kTcTF32x3;
  const bool gm = c.method == 1;
  const int Q = std::min(nrhs, 16);
  const int nch = (n + kRowChunk - 1) / kRowChunk;
  const int rch = (n + 4095) / 4096;
  const int kb = c.restart + 1;
  size_t need = al((size_t)n * n * sizeof(float)) + 2 * al((size_t)n * sizeof(int)) +
                2 * al((size_t)n * Q * sizeof(double)) + al((size_t)n * Q * sizeof(float)) +
                al(Q * sizeof(double)) + al(((size_t)64 * (n + 1) + 8) * sizeof(double)) +
                al((size_t)rch * n * 16 * sizeof(double)) + al(4 * (Q + 1) * sizeof(double)) +
                al((size_t)(n + 1) * sizeof(double));
  const int nblk = trsv_blocks(n);
  need += 2 * al((size_t)nblk * 4096 * sizeof(float)) +
          al(trsv_tag_words(n) * sizeof(unsigned long long)) + al(sizeof(unsigned));
  // double-float residuals where the FP64 pipe bounds the residual (below
  // n = 2048 it costs little either way)
  const bool df = ctx->opt_residual_df != 0 && n >= 2048;
  const size_t xs_count = ((size_t)(n + 63) / 64 * 64 + 1) * 16;
  need += al(2 * df_split_parts(n) * sizeof(double)) + al(2 * sizeof(double));
  if (df)
    need += 2 * al((size_t)n * n * sizeof(float)) + al(xs_count * sizeof(float2)) +
            al(16 * sizeof(double)) + al(df_residual_partial_doubles(n) * sizeof(double));
  if (gm)
    need += al((size_t)Q * kb * n * sizeof(double)) + al((size_t)Q * c.restart * n * sizeof(double)) +
            al((size_t)n * Q * sizeof(double)) + al((size_t)Q * kb * sizeof(double)) +
            al((size_t)Q * nch * kMaxBasis * sizeof(double));
  if (c.precision != ELGB_PREC_FP64) IR_CHECK(ctx->ensure2(need));

  bool done = false;
  if (c.precision != ELGB_PREC_FP64) {
    char* p = static_cast<char*>(ctx->arena2);
    auto take = [&](size_t b) {
      char* r = p;
      p += al(b);
      return r;
    };
    Ws w{};
    w.Af = (float*)take((size_t)n * n * sizeof(float));
    w.ipiv = (int*)take((size_t)n * sizeof(int));
    w.perm = (int*)take((size_t)n * sizeof(int));
    w.R = (double*)take((size_t)n * Q * sizeof(double));
    w.Xprev = (double*)take((size_t)n * Q * sizeof(double));
    w.Rf = (float*)take((size_t)n * Q * sizeof(float));
    w.scale = (double*)take(Q * sizeof(double));
    w.part = (double*)take(((size_t)64 * (n + 1) + 8) * sizeof(double));
    w.rpart = (double*)take((size_t)rch * n * 16 * sizeof(double));
    w.sums = (double*)take(4 * (Q + 1) * sizeof(double));
    w.colout = (double*)take((size_t)(n + 1) * sizeof(double));
    w.Dl = (float*)take((size_t)nblk * 4096 * sizeof(float));
    w.Du = (float*)take((size_t)nblk * 4096 * sizeof(float));
    w.tags = (unsigned long long*)take(trsv_tag_words(n) * sizeof(unsigned long long));
    w.ticket = (unsigned*)take(sizeof(unsigned));
    w.epoch = 0;
    w.spart = (double*)take(2 * df_split_parts(n) * sizeof(double));
    w.astat = (double*)take(2 * sizeof(double));
    if (df) {
      w.Ahi = (float*)take((size_t)n * n * sizeof(float));
      w.Alo = (float*)take((size_t)n * n * sizeof(float));
      w.Xs = (float2*)take(xs_count * sizeof(float2));
      w.xinv = (double*)take(16 * sizeof(double));
      w.dfpart = (double*)take(df_residual_partial_doubles(n) * sizeof(double));
    }
    IR_CHECK(cudaMemsetAsync(w.tags, 0, trsv_tag_words(n) * sizeof(unsigned long long),
                             ctx->stream));
    if (gm) {
      w.V = (double*)take((size_t)Q * kb * n * sizeof(double));
      w.Z = (double*)take((size_t)Q * c.restart * n * sizeof(double));
      w.W = (double*)take((size_t)n * Q * sizeof(double));
      w.H = (double*)take((size_t)Q * kb * sizeof(double));
      w.dpart = (double*)take((size_t)Q * nch * kMaxBasis * sizeof(double));
    }
    // 1. low-precision factorization of an FP32 copy of A; the same pass over
    // A makes its FP32 words for the double-float residual and its norms
    const int pc = ctx->prof_begin(ctx->stream, ELGB_PROF_CONVERT);
    if (df) {
      IR_CHECK(launch_split_a(A, lda, n, w.Af, w.Ahi, w.Alo, w.spart, w.astat, ctx->stream));
      ctx->launches += 2;
    } else {
      cvt_f64_f32_kernel<<<dim3((n + 255) / 256, grid_y(n)), 256, 0, ctx->stream>>>(A, lda, n,
                                                                               n, w.Af, n);
      ctx->launches += 1;
      IR_CHECK(cudaGetLastError());
    }
    // bytes: A read, the FP32 copy (and the two words) written
    ctx->prof_end(pc, ctx->stream, ELGB_PROF_CONVERT, 0.0,
                  (df ? 20.0 : 12.0) * n * (double)n);
    IR_CHECK(getrf<float>(ctx, n, n, w.Af, n, w.ipiv, c.nb, tc_kind, c.pivoting == 1));
    IR_CHECK(cudaMemcpyAsync(ctx->h_status, ctx->status, sizeof(DevStatus),
                             cudaMemcpyDeviceToHost, ctx->stream));
    IR_CHECK(cudaStreamSynchronize(ctx->stream));
    const int finfo = ctx->h_status->info, ferr = ctx->h_status->err;
    if (ferr) return cudaErrorLaunchTimeout;
    if (finfo == 0) {
      IR_CHECK(launch_explicit_perm(w.ipiv, n, n, w.perm, ctx->stream));
      IR_CHECK(launch_trtri_diag<float>(w.Af, n, n, true, true, w.Dl, ctx->stream));
      IR_CHECK(launch_trtri_diag<float>(w.Af, n, n, false, false, w.Du, ctx->stream));
      ctx->launches += 3;
      // ||A||_F (and max |a|, from the split pass)
      double stat[2] = {0.0, 0.0};
      if (!df) {
        IR_CHECK(launch_col_sumsq<double>(A, lda, n, n, w.colout, w.part, ctx->stream));
        ctx->launches += 2;
        IR_CHECK(cudaMemcpyAsync(&stat[0], w.colout + n, sizeof(double), cudaMemcpyDeviceToHost,
                                 ctx->stream));
      } else {
        IR_CHECK(cudaMemcpyAsync(stat, w.astat, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                                 ctx->stream));
      }
      IR_CHECK(cudaStreamSynchronize(ctx->stream));
      const double nA = std::sqrt(stat[0]);
      // double-float words need max |a| well inside FP32's exponent range
      // (the scaled products then stay O(1)); otherwise FP64 residuals
      w.df = df && stat[1] > 0x1p-100 && stat[1] < 0x1p100;
      bool all_ok = true;
      int max_it = 0;
      double worst = 0.0;
      for (int c0 = 0; c0 < nrhs; c0 += 16) {
        const int q = std::min(16, nrhs - c0);
        const double* Bc = B + (long)c0 * ldb;
        double* Xc = X + (long)c0 * ldx;
        std::vector<double> nb, nr, nx, be, prev(q, INFINITY);
        IR_CHECK(colnorm2(ctx, Bc, ldb, n, q, w.sums, w.part, nb));
        // x0 = M^{-1} b
        IR_CHECK(lowprec_solve(ctx, n, q, w, Bc, ldb, Xc, ldx, false, true));
        int it = 0;
        bool conv = false;
        while (true) {
          IR_CHECK(ir_residual(ctx, w, n, q, A, lda, Xc, ldx, Bc, ldb, w.R, n));
          IR_CHECK(colnorm2(ctx, w.R, n, n, q, w.sums, w.part, nr));
          IR_CHECK(colnorm2(ctx, Xc, ldx, n, q, w.sums + 17, w.part, nx));
          backward_errors(nr, nx, nb, nA, q, be);
          double mx = 0.0;
          for (double v : be) mx = std::isfinite(v) ? std::max(mx, v) : INFINITY;
          if (mx <= c.tol) {
            conv = true;
            break;
          }
          if (it > 0) {
            bool improved = false;
            for (int j = 0; j < q; ++j) improved |= be[j] < prev[j];
            if (!improved || !std::isfinite(mx)) {
              // Refined.hpp keeps the previous iterate when the residual grew.
              IR_CHECK(cudaMemcpy2DAsync(Xc, ldx * sizeof(double), w.Xprev, n * sizeof(double),
                                         n * sizeof(double), q, cudaMemcpyDeviceToDevice,
                                         ctx->stream));
              break;
            }
          }
          if (it >= c.max_iters) break;
          prev = be;
          if (!gm) {
            IR_CHECK(cudaMemcpy2DAsync(w.Xprev, n * sizeof(double), Xc, ldx * sizeof(double),
                                       n * sizeof(double), q, cudaMemcpyDeviceToDevice,
                                       ctx->stream));
            IR_CHECK(lowprec_solve(ctx, n, q, w, w.R, n, Xc, ldx, true, true));
            ++it;
            continue;
          }
          // ---- one FGMRES cycle, right-preconditioned, all columns in lockstep
          IR_CHECK(cudaMemcpy2DAsync(w.Xprev, n * sizeof(double), Xc, ldx * sizeof(double),
                                     n * sizeof(double), q, cudaMemcpyDeviceToDevice,
                                     ctx->stream));
          const long vcs = (long)kb * n, zcs = (long)c.restart * n;
          std::vector<double> beta(q), f(q);
          for (int j = 0; j < q; ++j) {
            beta[j] = nr[j];
            f[j] = nr[j] > 0 ? 1.0 / nr[j] : 0.0;
          }
          IR_CHECK(cudaMemcpyAsync(w.scale, f.data(), q * sizeof(double), cudaMemcpyHostToDevice,
                                   ctx->stream));
          col_scale_copy_kernel<<<dim3((n + 255) / 256, q), 256, 0, ctx->stream>>>(
              w.R, n, n, w.scale, w.V, vcs);
          ctx->launches += 1;
          // Hessenberg, rotations and right-hand side per column (host)
          const int rs = c.restart;
          std::vector<double> Hh((size_t)q * (rs + 1) * rs, 0.0), cs((size_t)q * rs),
              sn((size_t)q * rs), g((size_t)q * (rs + 1), 0.0), hcol((size_t)q * kb);
          for (int j = 0; j < q; ++j) g[(size_t)j * (rs + 1)] = beta[j];
          std::vector<double> target(q);
          for (int j = 0; j < q; ++j) target[j] = 0.5 * c.tol * (nA * nx[j] + nb[j]);
          int jdone = 0;
          for (int j = 0; j < rs && it < c.max_iters; ++j) {
            // Z_c(:, j) = M^{-1} V_c(:, j)
            IR_CHECK(lowprec_solve(ctx, n, q, w, w.V + (long)j * n, vcs, w.Z + (long)j * n, zcs,
                                   false, false));
            // W = A Z(:, j)
            IR_CHECK(ir_residual(ctx, w, n, q, A, lda, w.Z + (long)j * n, zcs, nullptr, 0, w.W,
                                 n));
            // classical Gram-Schmidt, twice
            for (int pass = 0; pass < 2; ++pass) {
              multi_dot_partial_kernel<<<dim3(nch, q), 256, 0, ctx->stream>>>(w.V, vcs, n, j + 1,
                                                                             w.W, n, w.dpart);
              multi_dot_finish_kernel<<<q, 64, 0, ctx->stream>>>(w.dpart, nch, j + 1, w.H, kb,
                                                                 pass);
              ctx->launches += 2;
              // subtract only this pass's projection: recompute from the
              // accumulated H minus the previous pass is avoided by keeping
              // the pass-1 coefficients on the host
              if (pass == 0) {
                multi_axpy_kernel<<<dim3((n + 255) / 256, q), 256, 0, ctx->stream>>>(
                    w.V, vcs, n, j + 1, w.H, kb, w.W, n, 1.0);
                ctx->launches += 1;
                IR_CHECK(cudaMemcpyAsync(hcol.data(), w.H, (size_t)q * kb * sizeof(double),
                                         cudaMemcpyDeviceToHost, ctx->stream));
              }
            }
            // second pass: H now holds h1 + h2; subtract h2 = H - h1
            {
              std::vector<double> htot((size_t)q * kb);
              IR_CHECK(cudaMemcpyAsync(htot.data(), w.H, (size_t)q * kb * sizeof(double),
                                       cudaMemcpyDeviceToHost, ctx->stream));
              IR_CHECK(cudaStreamSynchronize(ctx->stream));
              std::vector<double> h2((size_t)q * kb, 0.0);
              for (int cc = 0; cc < q; ++cc)
                for (int i = 0; i <= j; ++i)
                  h2[(size_t)cc * kb + i] = htot[(size_t)cc * kb + i] - hcol[(size_t)cc * kb + i];
              IR_CHECK(cudaMemcpyAsync(w.H, h2.data(), (size_t)q * kb * sizeof(double),
                                       cudaMemcpyHostToDevice, ctx->stream));
              multi_axpy_kernel<<<dim3((n + 255) / 256, q), 256, 0, ctx->stream>>>(
                  w.V, vcs, n, j + 1, w.H, kb, w.W, n, 1.0);
              ctx->launches += 1;
              std::vector<double> hn;
              IR_CHECK(colnorm2(ctx, w.W, n, n, q, w.sums, w.part, hn));
              for (int cc = 0; cc < q; ++cc) {
                double* Hc = &Hh[(size_t)cc * (rs + 1) * rs];
                for (int i = 0; i <= j; ++i) Hc[i + (size_t)j * (rs + 1)] = htot[(size_t)cc * kb + i];
                Hc[(j + 1) + (size_t)j * (rs + 1)] = hn[cc];
                f[cc] = hn[cc] > 0 ? 1.0 / hn[cc] : 0.0;
                // apply previous rotations, then a new one (FGMRES.hpp:180-226)
                for (int i = 0; i < j; ++i) {
                  const double a = Hc[i + (size_t)j * (rs + 1)], b = Hc[i + 1 + (size_t)j * (rs + 1)];
                  const double ci = cs[(size_t)cc * rs + i], si = sn[(size_t)cc * rs + i];
                  Hc[i + (size_t)j * (rs + 1)] = ci * a + si * b;
                  Hc[i + 1 + (size_t)j * (rs + 1)] = -si * a + ci * b;
                }
                const double a = Hc[j + (size_t)j * (rs + 1)], b = Hc[j + 1 + (size_t)j * (rs + 1)];
                const double r = std::hypot(a, b);
                const double ci = r > 0 ? a / r : 1.0, si = r > 0 ? b / r : 0.0;
                cs[(size_t)cc * rs + j] = ci;
                sn[(size_t)cc * rs + j] = si;
                Hc[j + (size_t)j * (rs + 1)] = r;
                Hc[j + 1 + (size_t)j * (rs + 1)] = 0.0;
                double* gc = &g[(size_t)cc * (rs + 1)];
                gc[j + 1] = -si * gc[j];
                gc[j] = ci * gc[j];
              }
              IR_CHECK(cudaMemcpyAsync(w.scale, f.data(), q * sizeof(double),
                                       cudaMemcpyHostToDevice, ctx->stream));
              col_scale_copy_kernel<<<dim3((n + 255) / 256, q), 256, 0, ctx->stream>>>(
                  w.W, n, n, w.scale, w.V + (long)(j + 1) * n, vcs);
              ctx->launches += 1;
            }
            ++it;
            jdone = j + 1;
            bool all_small = true;
            for (int cc = 0; cc < q; ++cc)
              all_small &= std::fabs(g[(size_t)cc * (rs + 1) + j + 1]) <= target[cc];
            if (all_small) break;
          }
          // y = H^{-1} g (upper triangular), X += Z y
          std::vector<double> y((size_t)q * kb, 0.0);
          for (int cc = 0; cc < q; ++cc) {
            const double* Hc = &Hh[(size_t)cc * (rs + 1) * rs];
            const double* gc = &g[(size_t)cc * (rs + 1)];
            for (int i = jdone - 1; i >= 0; --i) {
              double s = gc[i];
              for (int l = i + 1; l < jdone; ++l) s -= Hc[i + (size_t)l * (rs + 1)] * y[(size_t)cc * kb + l];
              const double d = Hc[i + (size_t)i * (rs + 1)];
              y[(size_t)cc * kb + i] = d != 0 ? s / d : 0.0;
            }
          }
          IR_CHECK(cudaMemcpyAsync(w.H, y.data(), (size_t)q * kb * sizeof(double),
                                   cudaMemcpyHostToDevice, ctx->stream));
          multi_axpy_kernel<<<dim3((n + 255) / 256, q), 256, 0, ctx->stream>>>(
              w.Z, zcs, n, jdone, w.H, kb, Xc, ldx, -1.0);
          ctx->launches += 1;
          IR_CHECK(cudaGetLastError());
        }
        all_ok &= conv;
        max_it = std::max(max_it, it);
        worst = std::max(worst, be.empty() ? 0.0 : *std::max_element(be.begin(), be.end()));
      }
      inf.iterations = max_it;
      inf.converged = all_ok ? 1 : 0;
      inf.backward_error = worst;
      done = all_ok || !c.fallback;
    }
  }
  if (!done) {
    // FP64 LU (the plain path) takes over: factor a copy, solve.
    IR_CHECK(ctx->ensure2(al((size_t)n * n * sizeof(double)) + al((size_t)n * sizeof(int))));
    double* Ad = static_cast<double*>(ctx->arena2);
    int* ipiv = reinterpret_cast<int*>(static_cast<char*>(ctx->arena2) +
                                       al((size_t)n * n * sizeof(double)));
    IR_CHECK(cudaMemcpy2DAsync(Ad, n * sizeof(double), A, lda * sizeof(double),
                               n * sizeof(double), n, cudaMemcpyDeviceToDevice, ctx->stream));
    IR_CHECK(cudaMemcpy2DAsync(X, ldx * sizeof(double), B, ldb * sizeof(double),
                               n * sizeof(double), nrhs, cudaMemcpyDeviceToDevice, ctx->stream));
    IR_CHECK(getrf<double>(ctx, n, n, Ad, n, ipiv, 0, -1));
    IR_CHECK(getrs<double>(ctx, 0, n, Ad, n, ipiv, nrhs, X, ldx, nullptr));
    inf.fell_back = c.precision != ELGB_PREC_FP64 ? 1 : 0;
    inf.precision = ELGB_PREC_FP64;
    double be = 0;
    IR_CHECK(backward_error(ctx, n, nrhs, A, lda, X, ldx, B, ldb, &be));
    inf.backward_error = be;
    inf.converged = be <= c.tol ? 1 : 0;
  }
  if (info) *info = inf;
  return cudaSuccess;
}

// R = B - A X in double-float arithmetic for any nrhs (blocks of 16): the
// split of A into FP32 words, then the residual kernels.
cudaError_t residual_df(Context* ctx, int n, int nrhs, const double* A, long lda,
                        const double* X, long ldx, const double* B, long ldb, double* R,
                        long ldr) {
  IR_CHECK(cudaSetDevice(ctx->device));
  IR_CHECK(ctx->begin_call());
  if (n == 0 || nrhs == 0) return cudaSuccess;
  const size_t xs_count = ((size_t)(n + 63) / 64 * 64 + 1) * 16;
  // partial sums of either kernel set (FP64: one per 4096-column chunk)
  const size_t npart = std::max(df_residual_partial_doubles(n),
                                (size_t)((n + 4095) / 4096) * n * 16);
  IR_CHECK(ctx->ensure(2 * al((size_t)n * n * sizeof(float)) +
                       al(2 * df_split_parts(n) * sizeof(double)) + al(2 * sizeof(double)) +
                       al(xs_count * sizeof(float2)) + al(16 * sizeof(double)) +
                       al(npart * sizeof(double))));
  char* p = static_cast<char*>(ctx->arena);
  auto take = [&](size_t b) {
    char* r = p;
    p += al(b);
    return r;
  };
  float* Ahi = (float*)take((size_t)n * n * sizeof(float));
  float* Alo = (float*)take((size_t)n * n * sizeof(float));
  double* spart = (double*)take(2 * df_split_parts(n) * sizeof(double));
  double* astat = (double*)take(2 * sizeof(double));
  float2* Xs = (float2*)take(xs_count * sizeof(float2));
  double* inv = (double*)take(16 * sizeof(double));
  double* part = (double*)take(npart * sizeof(double));
  IR_CHECK(launch_split_a(A, lda, n, nullptr, Ahi, Alo, spart, astat, ctx->stream));
  ctx->launches += 2;
  // A's entries must sit well inside FP32's exponent range for the split;
  // otherwise the FP64 kernels (their partial sums fit in the same scratch)
  double amax = 0.0;
  IR_CHECK(cudaMemcpyAsync(&amax, astat + 1, sizeof(double), cudaMemcpyDeviceToHost,
                           ctx->stream));
  IR_CHECK(cudaStreamSynchronize(ctx->stream));
  if (!(amax > 0x1p-100 && amax < 0x1p100)) {
    for (int c = 0; c < nrhs; c += 16) {
      const int q = std::min(16, nrhs - c);
      IR_CHECK(launch_residual_f64(n, q, A, lda, X + (long)c * ldx, ldx,
                                   B ? B + (long)c * ldb : nullptr, ldb, R + (long)c * ldr, ldr,
                                   part, ctx->stream));
      ctx->launches += 2;
    }
    return cudaSuccess;
  }
  for (int c = 0; c < nrhs; c += 16) {
    const int q = std::min(16, nrhs - c);
    IR_CHECK(launch_residual_df(n, q, Ahi, Alo, astat + 1, X + (long)c * ldx, ldx,
                                B ? B + (long)c * ldb : nullptr, ldb, R + (long)c * ldr, ldr,
                                Xs, inv, part, ctx->stream));
    ctx->launches += 3;
  }
  return cudaSuccess;
}

}  // namespace elgb

extern "C" int ElGBResidualDF_d(ElGBContext ctx, int n, int nrhs, const double* A, int lda,
                                const double* X, int ldx, const double* B, int ldb, double* R,
                                int ldr) {
  if (!ctx || n < 0 || nrhs < 0 || lda < std::max(n, 1) || ldx < std::max(n, 1) ||
      ldb < std::max(n, 1) || ldr < std::max(n, 1))
    return elgb::kElArgError;
  auto* cx = static_cast<elgb::Context*>(ctx);
  return elgb::to_el_error(elgb::residual_df(cx, n, nrhs, A, lda, X, ldx, B, ldb, R, ldr));
}

extern "C" int ElGBRefinedSolve_d(ElGBContext ctx, int n, const double* A, int lda, int nrhs,
                                  const double* B, int ldb, double* X, int ldx,
                                  const ElGBRefineCtrl* ctrl, ElGBRefineInfo* info) {
  if (!ctx || n < 0 || nrhs < 0 || lda < std::max(n, 1) || ldb < std::max(n, 1) ||
      ldx < std::max(n, 1))
    return elgb::kElArgError;
  ElGBRefineCtrl c{};
  if (ctrl) c = *ctrl;
  else {
    c.precision = ELGB_PREC_FP32;
    c.fallback = 1;
  }
  if (c.pivoting < 0 || c.pivoting > 1 || c.precision < ELGB_PREC_FP64 ||
      c.precision > ELGB_PREC_FP8 || c.method < 0 ||
      c.method > 1)
    return elgb::kElArgError;
  auto* cx = static_cast<elgb::Context*>(ctx);
  return elgb::to_el_error(elgb::refined_solve(cx, n, A, lda, nrhs, B, ldb, X, ldx, c, info));
}
