// Tensor-core (tcgen05) GEMM update used by the low-precision factorizations.
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"

namespace elgb {

// Operand precision of the tensor-core products (accumulation is FP32).
enum TcKind : int {
  kTcBF16 = 0,  // tcgen05.mma kind::f16 with BF16 operands
  kTcTF32 = 1,  // tcgen05.mma kind::tf32
  kTcTF32x3 = 2,  // kind::tf32, operands split hi + lo, three products (~FP32)
  kTcFP8 = 3,     // kind::f8f6f4 with E4M3 operands, each operand scaled per
                  // call (per panel) by a power of two that maps its largest
                  // magnitude near the E4M3 maximum 448; the scales are
                  // divided out in the epilogue
};

// Bytes of device workspace launch_tc_gemm_sub needs for its packed operands.
size_t tc_gemm_workspace_bytes(int kind, int m, int n, int K);

// C[m x n] -= A[m x K] * B[K x n]; A, B, C FP32 column-major.  Packs A and B
// into `ws` (tc_gemm_workspace_bytes) in the operand precision, then runs the
// tcgen05 kernel.  *nlaunch receives the number of kernels enqueued.
// If ev0/ev1 are given they are recorded immediately before and after the
// tensor-core kernel itself (not the packing), for live per-kernel timing.
// grid_mode: how many SMs the persistent kernel may hold (one CTA per SM).
enum TcGridMode : int {
  kGridFull = 0,      // every SM (up to one CTA per tile)
  kGridSpareGpc = 1,  // all GPCs but one (16-CTA clusters), for an update that
                      // runs beside the look-ahead panel stream
  kGridSmall = 2,     // at most kSmallGrid CTAs, for the look-ahead stream's own
                      // small updates while the trailing update holds the rest
  kGridTiles = 3,     // one CTA per tile: SMs are released tile by tile
};
constexpr int kSmallGrid = 32;
// a_packed: ws already holds A's packed words from an earlier call with the
// same A, lda, m, K and kind, and nothing has changed them since (not for
// FP8, whose scale covers A and B per call).
cudaError_t launch_tc_gemm_sub(int kind, int m, int n, int K, const float* A, long lda,
                               const float* B, long ldb, float* C, long ldc, void* ws,
                               DevStatus* st, cudaStream_t stream, int* nlaunch,
                               cudaEvent_t ev0 = nullptr, cudaEvent_t ev1 = nullptr,
                               int grid_mode = kGridFull, bool a_packed = false);

}  // namespace elgb
