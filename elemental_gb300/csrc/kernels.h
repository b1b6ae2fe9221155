// Launch wrappers for the GB300 dense factor-and-solve kernels (host side).
// All matrices are column-major: element (i, j) of a matrix with leading
// dimension ld sits at ptr[i + j * ld], the layout of El::Matrix
// (include/El/core/Matrix/decl.hpp:17-241).  Every wrapper enqueues work on
// `stream` and returns a cudaError_t from the launch.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace elgb {

// One CTA's published state for one panel column (see getf2_panel_kernel).
template <typename T>
struct alignas(16) PanelSlot {
  T val;        // |candidate|
  int row;      // candidate row (panel-relative), -1 = none
  int epoch;    // written last, with release semantics
  T cand[32];   // the candidate row
  T diag[32];   // row j (written by its owner only)
};

// Device scratch of the panel factorization: slots [2][maxG] (column
// parity x CTA), zeroed once per factorization.
template <typename T>
struct PanelScratch {
  PanelSlot<T>* slots;
  int maxG;
  int* cand;  // tournament pivoting: maxG x 33 candidate lists
  // panel trace (ElGBSetOption(ELGB_OPT_PANEL_TRACE)): when set, CTA 0 of a
  // leaf panel stamps %globaltimer four times per column at trace[4 j ..]
  // (before its candidate is published, after the previous step's deferred
  // update, once the exchange is complete, after the step's front half and
  // argmax); null: no trace
  unsigned long long* trace = nullptr;
};

// Tournament-pivoted leaf panel of the FP32 (preconditioner) LU, w <= 32
// (calu.cu): same outputs as launch_getf2_panel (ipiv, the factored panel,
// info), pivots chosen by a reduction tree.  cudaErrorNotSupported when the
// candidate set does not fit in shared memory (the caller then uses getf2).
size_t calu_scratch_ints(int max_ctas);
cudaError_t launch_calu_panel(float* A, long lda, int mp, int w, int* ipiv, int row_base,
                              int info_base, int* cand, int max_ctas, DevStatus* st,
                              int num_sms, cudaStream_t stream, int* nlaunch);

// Largest thread-block cluster the panel kernel may use (1: the cooperative
// kernel only); process-wide, ElGBSetOption(ELGB_OPT_PANEL_CLUSTER).
extern int g_panel_cluster;
// Rows per CTA the leaf-panel kernels aim for (ElGBSetOption(ELGB_OPT_PANEL_ROWS),
// default 512: the register kernel then holds one row a thread up to 8192 rows).
extern int g_panel_rows;
// FP32 panels with the rows in registers: 2 on one cluster (default), 1 on a
// cooperative grid, 0 in shared memory.
extern int g_panel_regs;
// register leaf panels: candidates pushed into every CTA with asynchronous
// DSMEM stores on an mbarrier (1) or read after a cluster barrier (0)
extern int g_panel_push;
// register leaf panels launched as programmatic dependents of the kernel
// before them on their stream (1) or normally (0)
extern int g_panel_pdl;

// getf2 on a w-wide panel (w <= 32): El's lu::Panel
// (src/lapack_like/factor/LU/Panel.hpp:15-59) as one cooperative launch.
// `A` points at the panel's top-left element, `mp` rows, `w` columns.
// ipiv[c] receives the absolute pivot row (row_base + panel row).  A zero
// pivot records info = info_base + c + 1 (first one wins) in st.
// epoch_base: columns published so far in this factorization (the slot
// epochs must keep growing across launches).  nopiv: no pivot search, the
// pivot of column c is row c (El::LU(A), ipiv[c] = row_base + c).
// swap_lo <= 0 <= w <= swap_hi: the leaf's row interchanges are also due on
// the columns [swap_lo, 0) and [w, swap_hi) of A (relative to the leaf's
// first column); a kernel that applies them itself sets *swaps_done, and the
// caller applies them otherwise.  sib_w > 0: the leaf is the left child of a
// recursion node whose right child is columns [w, w + sib_w); a kernel that
// also applies that node's TRSM and update (the same operations in the same
// order as launch_trsm_block and launch_gemm_simt) sets *node_done.
template <typename T>
cudaError_t launch_getf2_panel(T* A, long lda, int mp, int w, int* ipiv,
                               int row_base, int info_base, int epoch_base,
                               const PanelScratch<T>& s, DevStatus* st,
                               int num_sms, cudaStream_t stream, bool nopiv = false,
                               int swap_lo = 0, int swap_hi = 0, bool* swaps_done = nullptr,
                               int sib_w = 0, bool* node_done = nullptr);

// El::LU(A, P, Q) with full pivoting (src/lapack_like/factor/LU/Full.hpp):
// unblocked, two kernels per step.  fs / part: device scratch (one state,
// `grid` candidates); p / q receive the row / column swap destinations; an
// exact zero pivot records info = step + 1.  *nlaunch += kernels enqueued.
template <typename T>
struct FullPivState {
  int i, j;        // the next pivot (absolute row and column)
  T alpha;         // its value
  unsigned count;  // CTAs done with the current update
};
template <typename T>
struct FullPivCand {
  T v, s;  // |value| and value
  int i, j;
};
int fullpiv_grid(int num_sms);
// El::Cholesky(uplo, A, P) with diagonal pivoting: unblocked, two kernels per
// step; piv (n ints) receives the swap destinations.  Same scratch as
// launch_lu_full.  No error is raised for a non-positive pivot (the
// reference takes its square root).
template <typename T>
cudaError_t launch_cholesky_piv(T* A, long lda, int n, bool upper, int* piv,
                                FullPivState<T>* fs, FullPivCand<T>* part, int grid,
                                cudaStream_t stream, long long* nlaunch);
template <typename T>
cudaError_t launch_lu_full(T* A, long lda, int m, int n, int* p, int* q, FullPivState<T>* fs,
                           FullPivCand<T>* part, int grid, DevStatus* st, cudaStream_t stream,
                           long long* nlaunch);

// Converts the swap sequence ipiv[0..nb) (absolute destinations for rows
// k..k+nb) into an explicit list of (dst, src) row moves.  pairs must hold
// 4*nb ints ([dst..., src...] as 2*nb each); count receives the number of
// moves.
cudaError_t launch_build_swap_pairs(const int* ipiv, int k, int nb,
                                    int* pairs, int* count,
                                    cudaStream_t stream);

// Applies the row moves from launch_build_swap_pairs to columns
// [c0a, c1a) and [c0b, c1b) of A (the laswp of El's PB.PermuteRows,
// src/lapack_like/factor/LU.cpp:130-131).
template <typename T>
cudaError_t launch_apply_swap_pairs(T* A, long lda, int c0a, int c1a,
                                    int c0b, int c1b, const int* pairs,
                                    const int* count, int nb,
                                    cudaStream_t stream);

// Deferred interchanges of the blocked LU's left columns.  Block column b
// (columns [b nb, (b+1) nb)) must end up with every later panel's row
// interchanges applied; instead of swapping those rows after each panel,
// lab[b m + r] (r >= (b+1) nb) receives the original row whose content ends
// at row r after the interchanges ipiv[(b+1) nb .. mn), and the gather
// A(r, c) <- A(lab[r], c) applies them once per column (through shared
// memory when a column fits, coalesced both ways).  tmp: gridDim x m
// elements of scratch for columns that do not fit.  work (may be null: one
// serial replay a block column instead): defer_labels_work_ints ints.
size_t defer_labels_work_ints(int m, int mn, int nb);
cudaError_t launch_defer_labels(const int* ipiv, int m, int mn, int nb, int* lab, int* work,
                                cudaStream_t stream);
template <typename T>
cudaError_t launch_defer_gather(T* A, long lda, int m, int mn, int nb, const int* lab, T* tmp,
                                int grid, cudaStream_t stream);
int defer_gather_grid(int num_sms);

// Explicit permutation vector from a whole swap sequence:
// perm[i] = the original row that ends up at row i
// (Permutation::ExplicitVector, src/lapack_like/perm/Permutation.cpp:731-745).
cudaError_t launch_explicit_perm(const int* ipiv, int nswaps, int n,
                                 int* perm, cudaStream_t stream);

// Y(i, :) = X(perm[i], :) (inverse = false) or Y(perm[i], :) = X(i, :).
template <typename T>
cudaError_t launch_permute_rows(const T* X, long ldx, T* Y, long ldy, int n,
                                int ncols, const int* perm, bool inverse,
                                cudaStream_t stream);

// Small dense triangular solve on one diagonal block (nb <= 128):
//   op(A11) X = B   with B nb x ncols, solved in place.
// lower/upper and unit/non-unit refer to op(A11); trans_a loads A11
// transposed; trans_b means B is stored transposed (B^T is ncols x nb at
// Bm with leading dimension ldb).
// st (may be null): where a bounded wait reports a timeout; with it, A11's
// triangle is staged by bulk copies when its columns are 16-byte aligned.
template <typename T>
cudaError_t launch_trsm_block(const T* A11, long lda, T* Bm, long ldb, int nb,
                              int ncols, bool lower, bool unit, bool trans_a,
                              bool trans_b, cudaStream_t stream, DevStatus* st = nullptr);

// out (n x n) := the strictly lower triangle of A, zeros elsewhere.
template <typename T>
cudaError_t launch_copy_strict_lower(const T* A, long lda, int n, T* out, long ldo,
                                     cudaStream_t stream);

// C = alpha * op(A) * op(B) + beta * C on CUDA cores (SIMT FMA).
// uplo: 0 full, 1 lower triangle only (i >= j), 2 upper only (i <= j).
template <typename T>
cudaError_t launch_gemm_simt(bool ta, bool tb, int m, int n, int k, T alpha,
                             const T* A, long lda, const T* Bm, long ldb,
                             T beta, T* C, long ldc, int uplo,
                             cudaStream_t stream);

// Tall-skinny update C[m x q] -= op(A)[m x K] * X[K x q], K <= 256, q <= 16.
template <typename T>
cudaError_t launch_gemm_tall_sub(bool ta, int m, int q, int K, const T* A,
                                 long lda, const T* X, long ldx, T* C,
                                 long ldc, cudaStream_t stream);

// Cholesky of one diagonal block (nb <= 128) in place, El's
// LowerVariant3Unblocked / UpperVariant3Unblocked
// (src/lapack_like/factor/Cholesky/LowerVariant3.hpp:15-41).  A
// non-positive pivot records info = info_base + j + 1.
template <typename T>
cudaError_t launch_potf2_block(T* A, long lda, int nb, bool upper,
                               int info_base, DevStatus* st,
                               cudaStream_t stream);

// Residual R = B - A X in FP64 with a deterministic two-stage reduction
// (B == nullptr gives the product R = A X).
// partial must hold nchunks * n * q doubles, nchunks = ceil(n / 4096).
cudaError_t launch_residual_f64(int n, int q, const double* A, long lda,
                                const double* X, long ldx, const double* B,
                                long ldb, double* R, long ldr, double* partial,
                                cudaStream_t stream);

// The refinement's residual to FP64 accuracy on the FP32 pipe (double-float
// arithmetic, residual_df.cu).  launch_split_a makes, from the FP64 A (n x n),
// the FP32 copy Af, the FP32 words Ahi + Alo of A (all ld n) and out[0] =
// ||A||_F^2, out[1] = max |a_ij|; part holds 2 * df_split_parts(n) doubles.
// launch_residual_df computes R = B - A X (B == nullptr: R = A X), q <= 16,
// from Ahi, Alo and amaxA (= &out[1]); Xs holds (round_up(n, 64) + 1) * 16
// float2, inv 16 doubles, partial df_residual_partial_doubles(n) doubles.
size_t df_split_parts(int n);
size_t df_residual_partial_doubles(int n);
cudaError_t launch_split_a(const double* A, long lda, int n, float* Af, float* Ahi, float* Alo,
                           double* part, double* out, cudaStream_t stream);
cudaError_t launch_residual_df(int n, int q, const float* Ahi, const float* Alo,
                               const double* amaxA, const double* X, long ldx, const double* B,
                               long ldb, double* R, long ldr, float2* Xs, double* inv,
                               double* partial, cudaStream_t stream);

// Sum of squares of each column (out[j]) and of all entries (out[ncols]) of
// an m x ncols matrix, deterministic.  partial holds 64 * (ncols + 1) doubles
// followed by one zero-initialised unsigned counter (left zero on return).
template <typename T>
cudaError_t launch_col_sumsq(const T* A, long lda, int m, int ncols,
                             double* out, double* partial,
                             cudaStream_t stream);

// Measures the device's FP64 FMA rate: `iters` dependent-chain FMAs per
// thread over the given grid; out receives a checksum.
cudaError_t launch_fp64_fma_probe(double* out, int blocks, int threads,
                                  int iters, cudaStream_t stream);

}  // namespace elgb
