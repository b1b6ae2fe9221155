// Batched uneven-size solves in one persistent launch (batched.cu).
#pragma once

#include <cuda_runtime.h>

#include "driver.h"

namespace elgb {

struct BatchResult {
  int iters, converged, fell_back, info;
  double berr;
  int gmres_iters, prec;  // FGMRES iterations; the precision the result came from
  long long ns;  // device time spent on the system (globaltimer)
  int choice, pad2;  // fused selection: the network's class (else 0)
};

struct BatchPlan;

// Builds descriptors (largest-first order), per-CTA workspaces and a CUDA
// graph holding the persistent launch.  A, B, X: packed column-major
// systems (A_i n_i x n_i, B_i / X_i n_i x q, consecutive).  kind: 0 LU,
// 1 Cholesky; prec: 0 FP64 factors, 1 FP32 factors + FP64 refinement, 2 the
// same with BF16 operand products (nullptr: all LU / all FP32).  nb_table: panel width per size bucket
// (n <= 32, 64, ..., 2048, larger), nullptr for 32 everywhere.
// fallback: FP64 refactorization when refinement does not converge; mode 1
// computes the selector's 16 features per system into feat instead of
// solving.  method: 0 LU-IR, then FGMRES-IR (restart kry_m, at most kry_max
// inner iterations per right-hand side; 0: max(16, n / 24), -d: max(16, n / d)) when LU-IR stalls; 1 LU-IR only;
// 2 FGMRES-IR only.  prec_dev (device, may be null): per-system precision
// read when the graph runs, overriding h_prec (the selector's output).
// phase_ns (device, may be null): count x 10 device times per system: panel,
// row swaps, U12 solve, trailing update (low-precision factorization),
// LU-IR, FGMRES-IR, FP64 path, features, and within LU-IR the FP64
// residuals and the low-precision solves.  mlp (device, may be null): with
// mode 0, fused selection -- each system's features (FP32 LU kept), the
// network's class, then the solve with that precision.  tc: FP32 / BF16
// trailing updates on the tensor cores (tcgen05), else SIMT FMAs.
cudaError_t batched_plan(Context* ctx, int count, const int* h_n, const int* h_kind,
                         const int* h_prec, int q, const double* A, const double* B, double* X,
                         const int* nb_table, int ctas_per_sm, double tol, int max_iters,
                         int fallback, int mode, float* feat, int method, int kry_m,
                         int kry_max, const int* prec_dev, unsigned long long* phase_ns,
                         const float* mlp, int tc, BatchPlan** out);
cudaError_t batched_execute(BatchPlan* P);
cudaError_t batched_results(BatchPlan* P, BatchResult* h_out);
void batched_destroy(BatchPlan* P);
double batched_flops(const BatchPlan* P);

}  // namespace elgb
