/*
 * El_gb300.h — the subset of Elemental's C interface that the dense
 * factor-and-solve path binds, exported by libelgb300.so with the same names,
 * handle types and error codes, so that a C caller or the reference's ctypes
 * layer (python/lapack_like/factor.py:525-560, python/lapack_like/solve.py)
 * can load this library in place of libEl for that path.
 *
 * Each declaration cites the reference declaration it replaces.  Handles are
 * opaque pointers to the El::Matrix<T> / El::Permutation of El_gb300.hpp;
 * matrices are host memory, column-major, 32-bit ElInt.
 */
#ifndef EL_GB300_C_H
#define EL_GB300_C_H

#include <stdbool.h>
#include <stddef.h>

#include "elgb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef int ElInt; /* include/El/core/types.h (EL_USE_64BIT_INTS off) */

/* include/El/core/types.h:45-54 */
typedef enum {
  EL_SUCCESS,
  EL_ALLOC_ERROR,
  EL_OUT_OF_BOUNDS_ERROR,
  EL_ARG_ERROR,
  EL_LOGIC_ERROR,
  EL_RUNTIME_ERROR,
  EL_ERROR = -1
} ElError;
/* include/El/core/types.h:55 */
const char* ElErrorString(ElError error);

/* include/El/core/types.h:211-228 */
typedef enum { EL_NORMAL, EL_TRANSPOSE, EL_ADJOINT } ElOrientation;
typedef enum { EL_LOWER, EL_UPPER } ElUpperOrLower;
/* include/El/core/types.h:237-251 (BINARY and BINARY_FLAT are supported) */
typedef enum {
  EL_AUTO, EL_ASCII, EL_ASCII_MATLAB, EL_BINARY, EL_BINARY_FLAT, EL_BMP, EL_JPG, EL_JPEG,
  EL_MATRIX_MARKET, EL_PNG, EL_PPM, EL_XBM, EL_XPM, EL_FileFormat_MAX
} ElFileFormat;

/* include/El/core/Matrix.h:20-31 */
typedef struct ElMatrix_iDummy* ElMatrix_i;
typedef struct ElMatrix_sDummy* ElMatrix_s;
typedef struct ElMatrix_dDummy* ElMatrix_d;
typedef const struct ElMatrix_iDummy* ElConstMatrix_i;
typedef const struct ElMatrix_sDummy* ElConstMatrix_s;
typedef const struct ElMatrix_dDummy* ElConstMatrix_d;

/* include/El/core/Permutation.h:50-54 */
typedef struct ElPermutationDummy* ElPermutation;
typedef const struct ElPermutationDummy* ElConstPermutation;

/* Matrix<T> (include/El/core/Matrix.h:36-260) */
#define EL_GB_MATRIX_DECLS(S, T)                                              \
  ElError ElMatrixCreate_##S(ElMatrix_##S* A);                                \
  ElError ElMatrixDestroy_##S(ElConstMatrix_##S A);                           \
  ElError ElMatrixEmpty_##S(ElMatrix_##S A);                                  \
  ElError ElMatrixResize_##S(ElMatrix_##S A, ElInt height, ElInt width);      \
  ElError ElMatrixResizeWithLDim_##S(ElMatrix_##S A, ElInt height,            \
                                     ElInt width, ElInt ldim);                \
  ElError ElMatrixAttach_##S(ElMatrix_##S A, ElInt height, ElInt width,       \
                             T* buffer, ElInt ldim);                          \
  ElError ElMatrixLockedAttach_##S(ElMatrix_##S A, ElInt height, ElInt width, \
                                   const T* buffer, ElInt ldim);              \
  ElError ElMatrixHeight_##S(ElConstMatrix_##S A, ElInt* height);             \
  ElError ElMatrixWidth_##S(ElConstMatrix_##S A, ElInt* width);               \
  ElError ElMatrixLDim_##S(ElConstMatrix_##S A, ElInt* ldim);                 \
  ElError ElMatrixBuffer_##S(ElMatrix_##S A, T** buffer);                     \
  ElError ElMatrixLockedBuffer_##S(ElConstMatrix_##S A, const T** buffer);    \
  ElError ElMatrixGet_##S(ElConstMatrix_##S A, ElInt i, ElInt j, T* val);     \
  ElError ElMatrixSet_##S(ElMatrix_##S A, ElInt i, ElInt j, T val);
EL_GB_MATRIX_DECLS(i, ElInt)
EL_GB_MATRIX_DECLS(s, float)
EL_GB_MATRIX_DECLS(d, double)
#undef EL_GB_MATRIX_DECLS

/* include/El/core/types.h:36 */
typedef struct { ElInt beg, end; } ElRange_i;

/* include/El/core/View.h:20-25, 42-47: A becomes a view of B's rows iRange and
 * columns jRange (end == -100, El::END, stands for the full extent) */
ElError ElView_i(ElMatrix_i A, ElMatrix_i B, ElRange_i iRange, ElRange_i jRange);
ElError ElView_s(ElMatrix_s A, ElMatrix_s B, ElRange_i iRange, ElRange_i jRange);
ElError ElView_d(ElMatrix_d A, ElMatrix_d B, ElRange_i iRange, ElRange_i jRange);
ElError ElLockedView_i(ElMatrix_i A, ElConstMatrix_i B, ElRange_i iRange, ElRange_i jRange);
ElError ElLockedView_s(ElMatrix_s A, ElConstMatrix_s B, ElRange_i iRange, ElRange_i jRange);
ElError ElLockedView_d(ElMatrix_d A, ElConstMatrix_d B, ElRange_i iRange, ElRange_i jRange);

/* Permutation (include/El/core/Permutation.h:55-199) */
ElError ElPermutationCreate(ElPermutation* P);
ElError ElPermutationDestroy(ElConstPermutation P);
ElError ElPermutationEmpty(ElPermutation P);
ElError ElPermutationMakeIdentity(ElPermutation P, ElInt size);
ElError ElPermutationReserveSwaps(ElPermutation P, ElInt maxSwaps);
ElError ElPermutationSwap(ElPermutation P, ElInt origin, ElInt dest);
/* include/El/core/Permutation.h:82-83: appends PAppend's swaps, shifted by offset */
ElError ElPermutationSwapSequence(ElPermutation P, ElConstPermutation PAppend,
                                  ElInt offset);
ElError ElPermutationHeight(ElConstPermutation P, ElInt* height);
ElError ElPermutationWidth(ElConstPermutation P, ElInt* width);
ElError ElPermutationParity(ElConstPermutation P, bool* parity);
ElError ElPermutationIsSwapSequence(ElConstPermutation P, bool* isSwap);
ElError ElPermutationIsImplicitSwapSequence(ElConstPermutation P,
                                            bool* isImplicit);
ElError ElPermutationPermuteRows_s(ElConstPermutation P, ElMatrix_s A,
                                   ElInt offset);
ElError ElPermutationPermuteRows_d(ElConstPermutation P, ElMatrix_d A,
                                   ElInt offset);
ElError ElPermutationExplicitVector(ElConstPermutation P, ElMatrix_i pVec);

/* Blocksize (include/El/core/environment.h:48-52) */
ElError ElBlocksize(ElInt* blocksize);
ElError ElSetBlocksize(ElInt blocksize);
ElError ElPushBlocksizeStack(ElInt blocksize);
ElError ElPopBlocksizeStack(void);

/* LU with partial pivoting (include/El/lapack_like/factor.h:500-516) */
ElError ElLUPartialPiv_s(ElMatrix_s A, ElPermutation P);
ElError ElLUPartialPiv_d(ElMatrix_d A, ElPermutation P);
ElError ElSolveAfterLUPartialPiv_s(ElOrientation orientation,
                                   ElConstMatrix_s A, ElConstPermutation P,
                                   ElMatrix_s B);
ElError ElSolveAfterLUPartialPiv_d(ElOrientation orientation,
                                   ElConstMatrix_d A, ElConstPermutation P,
                                   ElMatrix_d B);

/* Cholesky with diagonal pivoting and its solve (include/El/lapack_like/factor.h:80-105) */
ElError ElCholeskyPiv_s(ElUpperOrLower uplo, ElMatrix_s A, ElPermutation P);
ElError ElCholeskyPiv_d(ElUpperOrLower uplo, ElMatrix_d A, ElPermutation P);
ElError ElSolveAfterCholeskyPiv_s(ElUpperOrLower uplo, ElOrientation orientation,
                                  ElConstMatrix_s A, ElConstPermutation P, ElMatrix_s B);
ElError ElSolveAfterCholeskyPiv_d(ElUpperOrLower uplo, ElOrientation orientation,
                                  ElConstMatrix_d A, ElConstPermutation P, ElMatrix_d B);

/* LU with full pivoting and its solve (include/El/lapack_like/factor.h:538-563) */
ElError ElLUFullPiv_s(ElMatrix_s A, ElPermutation P, ElPermutation Q);
ElError ElLUFullPiv_d(ElMatrix_d A, ElPermutation P, ElPermutation Q);
ElError ElSolveAfterLUFullPiv_s(ElOrientation orientation, ElConstMatrix_s A,
                                ElConstPermutation P, ElConstPermutation Q, ElMatrix_s B);
ElError ElSolveAfterLUFullPiv_d(ElOrientation orientation, ElConstMatrix_d A,
                                ElConstPermutation P, ElConstPermutation Q, ElMatrix_d B);

/* LU without pivoting (include/El/lapack_like/factor.h:467-468) */
ElError ElLU_s(ElMatrix_s A);
ElError ElLU_d(ElMatrix_d A);

/* Inverse (include/El/lapack_like/funcs.h:99-100) and the 1-norm condition
 * number (include/El/lapack_like/props.h:81-82) */
ElError ElInverse_s(ElMatrix_s A);
ElError ElInverse_d(ElMatrix_d A);
ElError ElOneCondition_s(ElConstMatrix_s A, float* cond);
ElError ElOneCondition_d(ElConstMatrix_d A, double* cond);

/* Matrix files (include/El/io.h:145-151, 216-224) */
ElError ElRead_i(ElMatrix_i A, const char* filename, ElFileFormat format);
ElError ElRead_s(ElMatrix_s A, const char* filename, ElFileFormat format);
ElError ElRead_d(ElMatrix_d A, const char* filename, ElFileFormat format);
ElError ElWrite_i(ElConstMatrix_i A, const char* basename, ElFileFormat format,
                  const char* title);
ElError ElWrite_s(ElConstMatrix_s A, const char* basename, ElFileFormat format,
                  const char* title);
ElError ElWrite_d(ElConstMatrix_d A, const char* basename, ElFileFormat format,
                  const char* title);

/* Cholesky (include/El/lapack_like/factor.h:24-41) */
ElError ElCholesky_s(ElUpperOrLower uplo, ElMatrix_s A);
ElError ElCholesky_d(ElUpperOrLower uplo, ElMatrix_d A);
ElError ElSolveAfterCholesky_s(ElUpperOrLower uplo, ElOrientation orientation,
                               ElConstMatrix_s A, ElMatrix_s B);
ElError ElSolveAfterCholesky_d(ElUpperOrLower uplo, ElOrientation orientation,
                               ElConstMatrix_d A, ElMatrix_d B);

/* Dense solves (include/El/lapack_like/solve.h:21-22, 151-156) */
ElError ElLinearSolve_s(ElConstMatrix_s A, ElMatrix_s B);
ElError ElLinearSolve_d(ElConstMatrix_d A, ElMatrix_d B);
ElError ElHPDSolve_s(ElUpperOrLower uplo, ElOrientation orientation,
                     ElConstMatrix_s A, ElMatrix_s B);
ElError ElHPDSolve_d(ElUpperOrLower uplo, ElOrientation orientation,
                     ElConstMatrix_d A, ElMatrix_d B);

/* Added form, no counterpart in the reference's C interface: El::LinearSolve
 * on host matrices through the mixed-precision path of this library
 * (low-precision tensor-core LU + LU-IR / GMRES-IR with an FP64 residual,
 * FP64 LU fallback; see ElGBRefinedSolve_d).  A is left untouched, B is
 * overwritten by X; ctrl may be NULL (FP32 factors, LU-IR, fallback on). */
ElError ElLinearSolveMixed_d(ElConstMatrix_d A, ElMatrix_d B,
                             const ElGBRefineCtrl* ctrl, ElGBRefineInfo* info);

/* Added, no counterpart in the reference: the host-side phases of the last
 * completed call of this interface that takes host matrices (milliseconds):
 * the host -> device uploads, the device work with its synchronisation, and
 * the device -> host downloads.  Any pointer may be NULL. */
ElError ElGBLastHostCallTimes(double* upload_ms, double* compute_ms,
                              double* download_ms);

/* Added, no counterpart in the reference: host memory for matrices that
 * move to and from the GPU (the buffers a caller attaches El::Matrix /
 * ElMatrix_d handles to).  Anonymous pages (transparent huge pages where the
 * kernel offers them) registered with the CUDA driver (cudaHostRegister).
 * On GB300, copies from such memory keep ~200 GB/s after GPU compute,
 * where copies from cudaHostAlloc memory fell to 40-100 GB/s.  *ptr is
 * NULL for bytes == 0.  EL_ARG_ERROR for ptr == NULL, EL_ALLOC_ERROR if
 * the pages cannot be had, EL_RUNTIME_ERROR if CUDA refuses the
 * registration. */
ElError ElGBHostAlloc(size_t bytes, void** ptr);
/* Frees memory from ElGBHostAlloc (NULL is a no-op); EL_LOGIC_ERROR for a
 * pointer it did not return. */
ElError ElGBHostFree(void* ptr);

#ifdef __cplusplus
}
#endif

#endif /* EL_GB300_C_H */
