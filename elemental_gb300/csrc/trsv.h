// One-launch blocked triangular solves (trsv.cu); instantiated for float
// (the refinement loop's low-precision factors).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>

#include "common.cuh"

namespace elgb {

// Number of 64-row block rows (and of 64 x 64 inverse diagonal blocks).
int trsv_blocks(int n);

// Dinv[b] = inverse of the b-th 64 x 64 diagonal block of the lower (unit or
// not) or upper triangle of A; Dinv holds trsv_blocks(n) * 4096 elements.
template <typename T>
cudaError_t launch_trtri_diag(const T* A, long lda, int n, bool lower, bool unit, T* Dinv,
                              cudaStream_t stream);

// 64-bit words the solve publishes its block rows in (two 64 x 16 tiles
// per block row).
size_t trsv_tag_words(int n);

// op(A) X = B in place (B n x q, q <= 16) with op(A) the lower or upper
// triangle of A and Dinv its inverted diagonal blocks.  tags holds
// trsv_tag_words(n) words whose high halves never held `epoch` before this
// call (start them at zero and use a new epoch per call); ticket is one
// unsigned.
template <typename T>
cudaError_t launch_trsv_persistent(const T* A, long lda, const T* Dinv, T* X, long ldx, int n,
                                   int q, bool lower, unsigned* ticket, unsigned long long* tags,
                                   unsigned epoch, DevStatus* st, int num_sms,
                                   cudaStream_t stream);

}  // namespace elgb
