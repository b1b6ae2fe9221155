/*
 * ORACLE — test infrastructure only.  A CPU restatement of Elemental's
 * sequential factor-and-solve path, used by tests/ as the checker, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg.  Nothing in the
 * product links, imports or calls it.
 *
 * It follows the reference step by step, calling the same external BLAS
 * routines at the same places the reference calls them (Elemental's own code
 * on this path is the blocking, the pivot bookkeeping and the panel loop; its
 * arithmetic is external BLAS), so on the same BLAS build its outputs are the
 * reference's bit for bit.  BLAS comes from a shared library opened at
 * elo_init() (SciPy's bundled OpenBLAS in practice, LP64).
 *
 * Parity pinned: the outputs are checked against golden fixtures produced by
 * the reference itself (oracle/_ref/elref, built from the reference sources
 * by oracle/build_ref.sh) in tests/test_oracle_golden.py.
 *
 * Layout: column-major, element (i,j) at A[i + j*lda], 32-bit Int, swap
 * destinations 0-based (Permutation::SwapDestinations,
 * src/lapack_like/perm/Permutation.cpp:205-250).
 * Status: 0 ok, 3 singular (SingularMatrixException,
 * src/lapack_like/factor/LU/Panel.hpp:51-52), 4 not HPD
 * (NonHPDMatrixException, src/lapack_like/factor/Cholesky/LowerVariant3.hpp:29-30),
 * 2 bad arguments, 1 BLAS not loaded.
 */
#include <dlfcn.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef int bint;

/* Fortran-style BLAS entry points, resolved at elo_init(). */
typedef void (*gemm_fn)(const char*, const char*, const bint*, const bint*,
                        const bint*, const void*, const void*, const bint*,
                        const void*, const bint*, const void*, void*,
                        const bint*);
typedef void (*trsm_fn)(const char*, const char*, const char*, const char*,
                        const bint*, const bint*, const void*, const void*,
                        const bint*, void*, const bint*);
typedef void (*swap_fn)(const bint*, void*, const bint*, void*, const bint*);
typedef void (*scal_fn)(const bint*, const void*, void*, const bint*);
typedef void (*ger_fn)(const bint*, const bint*, const void*, const void*,
                       const bint*, const void*, const bint*, void*,
                       const bint*);
typedef bint (*iamax_fn)(const bint*, const void*, const bint*);
typedef void (*syrk_fn)(const char*, const char*, const bint*, const bint*,
                        const void*, const void*, const bint*, const void*,
                        void*, const bint*);
typedef void (*syr_fn)(const char*, const bint*, const void*, const void*,
                       const bint*, void*, const bint*);
typedef void (*setthreads_fn)(int);

static struct {
  gemm_fn gemm[2];
  trsm_fn trsm[2];
  swap_fn swap[2];
  scal_fn scal[2];
  ger_fn ger[2];
  iamax_fn iamax[2];
  syrk_fn syrk[2];
  syr_fn syr[2];
  setthreads_fn setthreads;
  int loaded;
} B;

static void* sym(void* h, const char* prefix, const char* name) {
  char buf[128];
  strcpy(buf, prefix);
  strcat(buf, name);
  strcat(buf, "_");
  void* p = dlsym(h, buf);
  if (!p) { /* plain Fortran name */
    strcpy(buf, name);
    strcat(buf, "_");
    p = dlsym(h, buf);
  }
  return p;
}

/* Opens the BLAS library at `path`; symbols are looked up as
 * <prefix><name>_ (e.g. "scipy_dgemm_") then <name>_.  Returns 0 on success. */
int elo_init(const char* path, const char* prefix, int nthreads) {
  void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!h) return 1;
  const char* t[2] = {"d", "s"};
  for (int i = 0; i < 2; ++i) {
    char nm[16];
#define LOAD(field, base)                                   \
    strcpy(nm, t[i]); strcat(nm, base);                      \
    B.field[i] = (typeof(B.field[i]))sym(h, prefix, nm);    \
    if (!B.field[i]) return 1;
    LOAD(gemm, "gemm") LOAD(trsm, "trsm") LOAD(swap, "swap")
    LOAD(scal, "scal") LOAD(ger, "ger") LOAD(syrk, "syrk") LOAD(syr, "syr")
#undef LOAD
    strcpy(nm, "i");
    strcat(nm, t[i]);
    strcat(nm, "amax");
    B.iamax[i] = (iamax_fn)sym(h, prefix, nm);
    if (!B.iamax[i]) return 1;
  }
  char buf[128];
  strcpy(buf, prefix);
  strcat(buf, "openblas_set_num_threads");
  B.setthreads = (setthreads_fn)dlsym(h, buf);
  if (!B.setthreads) B.setthreads = (setthreads_fn)dlsym(h, "openblas_set_num_threads");
  if (B.setthreads && nthreads > 0) B.setthreads(nthreads);
  B.loaded = 1;
  return 0;
}

int elo_set_threads(int nthreads) {
  if (!B.setthreads) return 1;
  B.setthreads(nthreads);
  return 0;
}

/* ---------------------------------------------------------------------- */
/* One body per precision: T = scalar type, P = BLAS table index (0 = d,   */
/* 1 = s), S = function-name suffix.                                       */
/* ---------------------------------------------------------------------- */
#define ELO_DEFINE(T, P, S)                                                    \
                                                                               \
/* El::RowSwap (src/blas_like/level1/Swap.cpp:99-115): dswap of two rows.  */  \
static void rowswap_##S(bint width, T* A, bint lda, bint to, bint from) {      \
  if (to == from || width == 0) return;                                        \
  B.swap[P](&width, A + to, &lda, A + from, &lda);                             \
}                                                                              \
                                                                               \
/* lu::Panel (src/lapack_like/factor/LU/Panel.hpp:15-59) on the m x n panel   \
 * A; swap destinations relative to the panel go to piv[0..n).            */   \
static int panel_##S(bint m, bint n, T* A, bint lda, bint* piv) {              \
  const bint one = 1;                                                          \
  const T mone = (T)-1;                                                        \
  for (bint k = 0; k < n; ++k) {                                               \
    bint horz = n - (k + 1), vert = m - (k + 1), len = vert + 1;               \
    bint maxInd = B.iamax[P](&len, A + k + k * lda, &one) - 1;                 \
    bint iPiv = maxInd + k;                                                    \
    piv[k] = iPiv;                                                             \
    if (iPiv != k) B.swap[P](&n, A + k, &lda, A + iPiv, &lda);                 \
    const T alpha = A[k + k * lda];                                            \
    if (alpha == (T)0) return 3;                                               \
    const T inv = (T)1 / alpha;                                                \
    if (vert > 0) B.scal[P](&vert, &inv, A + (k + 1) + k * lda, &one);         \
    if (vert > 0 && horz > 0)                                                  \
      B.ger[P](&vert, &horz, &mone, A + (k + 1) + k * lda, &one,               \
               A + k + (k + 1) * lda, &lda, A + (k + 1) + (k + 1) * lda,       \
               &lda);                                                          \
  }                                                                            \
  return 0;                                                                    \
}                                                                              \
                                                                               \
/* El::Gemm NN with alpha=-1, beta=1 (src/blas_like/level3/Gemm.cpp:19-71). */ \
static void gemm_sub_##S(bint m, bint n, bint k, const T* A, bint lda,         \
                         const T* Bm, bint ldb, T* C, bint ldc) {              \
  if (m == 0 || n == 0 || k == 0) return;                                      \
  const T mone = (T)-1, pone = (T)1;                                           \
  B.gemm[P]("N", "N", &m, &n, &k, &mone, A, &lda, Bm, &ldb, &pone, C, &ldc);   \
}                                                                              \
                                                                               \
/* El::Trsm (src/blas_like/level3/Trsm.cpp:23-61) -> dtrsm, alpha = 1.     */  \
static void trsm_##S(char side, char uplo, char trans, char diag, bint m,      \
                     bint n, const T* A, bint lda, T* Bm, bint ldb) {          \
  if (m == 0 || n == 0) return;                                                \
  const T pone = (T)1;                                                         \
  B.trsm[P](&side, &uplo, &trans, &diag, &m, &n, &pone, A, &lda, Bm, &ldb);    \
}                                                                              \
                                                                               \
/* El::LU(Matrix&, Permutation&) (src/lapack_like/factor/LU.cpp:104-138).    \
 * swapDests[0..min(m,n)) receives P.SwapDestinations().                   */  \
int elo_lu_##S(bint m, bint n, T* A, bint lda, bint bsize, bint* swapDests) {  \
  if (m < 0 || n < 0 || lda < (m > 1 ? m : 1) || bsize < 1) return 2;         \
  if (!B.loaded) return 1;                                                     \
  const bint minDim = m < n ? m : n;                                           \
  for (bint k = 0; k < minDim; k += bsize) {                                   \
    const bint nb = bsize < minDim - k ? bsize : minDim - k;                   \
    const bint mB = m - k, n2 = n - (k + nb), m2 = m - (k + nb);               \
    bint* pb = swapDests + k;                                                  \
    int st = panel_##S(mB, nb, A + k + k * lda, lda, pb);                      \
    if (st) { /* the panel threw: no further swaps or updates */               \
      for (bint j = 0; j < nb; ++j) pb[j] += k;                                \
      return st;                                                               \
    }                                                                          \
    /* PB.PermuteRows(AB0); PB.PermuteRows(AB2) (LU.cpp:130-131) */            \
    for (bint j = 0; j < nb; ++j) {                                            \
      rowswap_##S(k, A + k, lda, j, pb[j]);                                    \
      rowswap_##S(n2, A + k + (k + nb) * lda, lda, j, pb[j]);                  \
    }                                                                          \
    for (bint j = 0; j < nb; ++j) pb[j] += k; /* P.Swap(k+offset, ...) */      \
    trsm_##S('L', 'L', 'N', 'U', nb, n2, A + k + k * lda, lda,                 \
             A + k + (k + nb) * lda, lda);                                     \
    gemm_sub_##S(m2, n2, nb, A + (k + nb) + k * lda, lda,                      \
                 A + k + (k + nb) * lda, lda, A + (k + nb) + (k + nb) * lda,   \
                 lda);                                                         \
  }                                                                            \
  return 0;                                                                    \
}                                                                              \
                                                                               \
/* Permutation::PermuteRows / InversePermuteRows for a swap sequence with    \
 * implicit origins (src/lapack_like/perm/Permutation.cpp:544-631).        */  \
void elo_permute_rows_##S(int inverse, bint numSwaps, const bint* swapDests,   \
                          bint height, bint width, T* Bm, bint ldb) {          \
  if (height == 0 || width == 0) return;                                       \
  if (!inverse)                                                                \
    for (bint j = 0; j < numSwaps; ++j)                                        \
      rowswap_##S(width, Bm, ldb, j, swapDests[j]);                            \
  else                                                                         \
    for (bint j = numSwaps - 1; j >= 0; --j)                                   \
      rowswap_##S(width, Bm, ldb, j, swapDests[j]);                            \
}                                                                              \
                                                                               \
/* lu::SolveAfter(orientation, A, P, B)                                       \
 * (src/lapack_like/factor/LU/SolveAfter.hpp:66-92).  orient: 0 NORMAL,      \
 * 1 TRANSPOSE, 2 ADJOINT (same as TRANSPOSE for real scalars).          */    \
int elo_lu_solve_after_##S(int orient, bint n, const T* A, bint lda,           \
                           const bint* swapDests, bint nrhs, T* Bm,            \
                           bint ldb) {                                         \
  if (!B.loaded) return 1;                                                     \
  if (orient == 0) {                                                           \
    elo_permute_rows_##S(0, n, swapDests, n, nrhs, Bm, ldb);                   \
    trsm_##S('L', 'L', 'N', 'U', n, nrhs, A, lda, Bm, ldb);                    \
    trsm_##S('L', 'U', 'N', 'N', n, nrhs, A, lda, Bm, ldb);                    \
  } else {                                                                     \
    trsm_##S('L', 'U', 'T', 'N', n, nrhs, A, lda, Bm, ldb);                    \
    trsm_##S('L', 'L', 'T', 'U', n, nrhs, A, lda, Bm, ldb);                    \
    elo_permute_rows_##S(1, n, swapDests, n, nrhs, Bm, ldb);                   \
  }                                                                            \
  return 0;                                                                    \
}                                                                              \
                                                                               \
/* cholesky::LowerVariant3Unblocked / UpperVariant3Unblocked                  \
 * (src/lapack_like/factor/Cholesky/LowerVariant3.hpp:15-41,                  \
 *  UpperVariant3.hpp): sqrt, scal by 1/alpha, dsyr rank-1 update.       */    \
static int potf2_##S(char uplo, bint n, T* A, bint lda) {                      \
  const T mone = (T)-1;                                                        \
  for (bint j = 0; j < n; ++j) {                                               \
    T alpha = A[j + j * lda];                                                  \
    if (alpha <= (T)0) return 4;                                               \
    alpha = (T)sqrt((double)alpha);                                            \
    A[j + j * lda] = alpha;                                                    \
    bint rest = n - (j + 1);                                                   \
    if (rest == 0) continue;                                                   \
    const T inv = (T)1 / alpha;                                                \
    if (uplo == 'L') {                                                         \
      const bint one = 1;                                                      \
      B.scal[P](&rest, &inv, A + (j + 1) + j * lda, &one);                     \
      B.syr[P]("L", &rest, &mone, A + (j + 1) + j * lda, &one,                 \
               A + (j + 1) + (j + 1) * lda, &lda);                             \
    } else {                                                                   \
      B.scal[P](&rest, &inv, A + j + (j + 1) * lda, &lda);                     \
      B.syr[P]("U", &rest, &mone, A + j + (j + 1) * lda, &lda,                 \
               A + (j + 1) + (j + 1) * lda, &lda);                             \
    }                                                                          \
  }                                                                            \
  return 0;                                                                    \
}                                                                              \
                                                                               \
/* El::Cholesky(uplo, A) (src/lapack_like/factor/Cholesky.cpp:26-38):          \
 * LowerVariant3Blocked (Cholesky/LowerVariant3.hpp:43-68) or                  \
 * UpperVariant3Blocked (Cholesky/UpperVariant3.hpp:48-73).               */   \
int elo_cholesky_##S(char uplo, bint n, T* A, bint lda, bint bsize) {          \
  if (!B.loaded) return 1;                                                     \
  if (n < 0 || lda < (n > 1 ? n : 1) || bsize < 1) return 2;                   \
  const T mone = (T)-1, pone = (T)1;                                           \
  for (bint k = 0; k < n; k += bsize) {                                        \
    const bint nb = bsize < n - k ? bsize : n - k;                             \
    const bint n2 = n - (k + nb);                                              \
    T* A11 = A + k + k * lda;                                                  \
    int st = potf2_##S(uplo, nb, A11, lda);                                    \
    if (st) return st;                                                         \
    if (n2 == 0) continue;                                                     \
    if (uplo == 'L') {                                                         \
      T* A21 = A + (k + nb) + k * lda;                                         \
      trsm_##S('R', 'L', 'T', 'N', n2, nb, A11, lda, A21, lda);                \
      B.syrk[P]("L", "N", &n2, &nb, &mone, A21, &lda, &pone,                   \
                A + (k + nb) + (k + nb) * lda, &lda);                          \
    } else {                                                                   \
      T* A12 = A + k + (k + nb) * lda;                                         \
      trsm_##S('L', 'U', 'T', 'N', nb, n2, A11, lda, A12, lda);                \
      B.syrk[P]("U", "T", &n2, &nb, &mone, A12, &lda, &pone,                   \
                A + (k + nb) + (k + nb) * lda, &lda);                          \
    }                                                                          \
  }                                                                            \
  return 0;                                                                    \
}                                                                              \
                                                                               \
/* cholesky::SolveAfter(uplo, NORMAL, A, B)                                   \
 * (src/lapack_like/factor/Cholesky/SolveAfter.hpp:15-43); real scalars.  */   \
int elo_cholesky_solve_after_##S(char uplo, bint n, const T* A, bint lda,      \
                                 bint nrhs, T* Bm, bint ldb) {                 \
  if (!B.loaded) return 1;                                                     \
  if (uplo == 'L') {                                                           \
    trsm_##S('L', 'L', 'N', 'N', n, nrhs, A, lda, Bm, ldb);                    \
    trsm_##S('L', 'L', 'T', 'N', n, nrhs, A, lda, Bm, ldb);                    \
  } else {                                                                     \
    trsm_##S('L', 'U', 'T', 'N', n, nrhs, A, lda, Bm, ldb);                    \
    trsm_##S('L', 'U', 'N', 'N', n, nrhs, A, lda, Bm, ldb);                    \
  }                                                                            \
  return 0;                                                                    \
}                                                                              \
                                                                               \
/* El::LinearSolve(A, B) (src/lapack_like/solve/Linear.cpp:212-218): copy A,  \
 * RowEchelon(ACopy, B) (:30-77), then the upper solve (:176-183).        */   \
int elo_linear_solve_##S(bint n, const T* A, bint lda, bint nrhs, T* Bm,       \
                         bint ldb, bint bsize) {                               \
  if (!B.loaded) return 1;                                                     \
  if (n < 0 || lda < (n > 1 ? n : 1) || bsize < 1) return 2;                   \
  T* W = (T*)malloc(sizeof(T) * (size_t)(n ? n : 1) * (size_t)(n ? n : 1));    \
  bint* pb = (bint*)malloc(sizeof(bint) * (size_t)(bsize));                    \
  if (!W || !pb) { free(W); free(pb); return 2; }                              \
  for (bint j = 0; j < n; ++j) memcpy(W + (size_t)j * n, A + (size_t)j * lda,  \
                                      sizeof(T) * n);                          \
  int st = 0;                                                                  \
  for (bint k = 0; k < n && !st; k += bsize) {                                 \
    const bint nb = bsize < n - k ? bsize : n - k;                             \
    const bint mB = n - k, n2 = n - (k + nb), m2 = n - (k + nb);               \
    st = panel_##S(mB, nb, W + k + (size_t)k * n, n, pb);                      \
    if (st) break;                                                             \
    for (bint j = 0; j < nb; ++j) {                                            \
      rowswap_##S(n2, W + k + (size_t)(k + nb) * n, n, j, pb[j]);              \
      rowswap_##S(nrhs, Bm + k, ldb, j, pb[j]);                                \
    }                                                                          \
    trsm_##S('L', 'L', 'N', 'U', nb, n2, W + k + (size_t)k * n, n,             \
             W + k + (size_t)(k + nb) * n, n);                                 \
    trsm_##S('L', 'L', 'N', 'U', nb, nrhs, W + k + (size_t)k * n, n, Bm + k,   \
             ldb);                                                             \
    gemm_sub_##S(m2, n2, nb, W + (k + nb) + (size_t)k * n, n,                  \
                 W + k + (size_t)(k + nb) * n, n,                              \
                 W + (k + nb) + (size_t)(k + nb) * n, n);                      \
    gemm_sub_##S(m2, nrhs, nb, W + (k + nb) + (size_t)k * n, n, Bm + k, ldb,   \
                 Bm + (k + nb), ldb);                                          \
  }                                                                            \
  if (!st) trsm_##S('L', 'U', 'N', 'N', n, nrhs, W, n, Bm, ldb);               \
  free(W);                                                                     \
  free(pb);                                                                    \
  return st;                                                                   \
}                                                                              \
                                                                               \
/* El::HPDSolve(uplo, NORMAL, A, B) (src/lapack_like/solve/HPD.cpp:47-55):     \
 * copy A, Cholesky, cholesky::SolveAfter.                                */   \
int elo_hpd_solve_##S(char uplo, bint n, const T* A, bint lda, bint nrhs,      \
                      T* Bm, bint ldb, bint bsize) {                           \
  if (!B.loaded) return 1;                                                     \
  T* W = (T*)malloc(sizeof(T) * (size_t)(n ? n : 1) * (size_t)(n ? n : 1));    \
  if (!W) return 2;                                                            \
  for (bint j = 0; j < n; ++j) memcpy(W + (size_t)j * n, A + (size_t)j * lda,  \
                                      sizeof(T) * n);                          \
  int st = elo_cholesky_##S(uplo, n, W, n > 0 ? n : 1, bsize);                 \
  if (!st) st = elo_cholesky_solve_after_##S(uplo, n, W, n > 0 ? n : 1, nrhs,  \
                                             Bm, ldb);                         \
  free(W);                                                                     \
  return st;                                                                   \
}

ELO_DEFINE(double, 0, d)
ELO_DEFINE(float, 1, s)
