// FP64 residual R = B - A X for callers that cannot allocate device memory.
//
// Some callers of this library may not call cudaMalloc at all: real-time or
// embedded hosts whose device memory is budgeted up front, frameworks that
// own every byte of device memory through their own allocator, and code on a
// latency-critical path that must not let cudaMalloc / cudaFree synchronize
// the device.  ElGBResidual_d needs scratch for its
// partial sums and takes it from a context arena that grows with cudaMalloc;
// this entry point instead keeps that scratch in a fixed file-scope device
// array, so it allocates nothing, ever.
//
// The array costs 8 MiB on every GPU that loads the library, for the life of
// the process.  Every call shares it, so two calls that overlap on the GPU
// (different streams, or different host threads) race on it; calls on one
// stream are ordered and safe.  The partial sums are fully overwritten by
// each call, so nothing needs clearing between calls.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/elgb300.h"
#include "driver.h"
#include "kernels.h"

namespace {

// Partial sums of the residual: one per (row, right-hand side, 4096-column
// chunk of A) for up to 16 right-hand sides at a time.
constexpr size_t kNoAllocPartials = size_t(1) << 20;  // doubles (8 MiB)
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_partials[kNoAllocPartials];

std::mutex g_noalloc_mu;
double* g_noalloc_addr[kMaxDevices];

}  // namespace

extern "C" int ElGBResidualNoAlloc_d(int n, int nrhs, const double* A, int lda,
                                     const double* X, int ldx, const double* B, int ldb,
                                     double* R, int ldr, void* stream) {
  if (n < 0 || nrhs < 0 || lda < (n > 1 ? n : 1) || ldx < (n > 1 ? n : 1) ||
      ldb < (n > 1 ? n : 1) || ldr < (n > 1 ? n : 1))
    return elgb::kElArgError;
  if (n == 0 || nrhs == 0) return 0;
  const size_t chunks = (size_t)(n + 4095) / 4096;
  const size_t q = nrhs < 16 ? (size_t)nrhs : 16;
  if (chunks * (size_t)n * q > kNoAllocPartials) return elgb::kElArgError;  // too large
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return elgb::kElRuntimeError;
  double* partials = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
      // The symbol's host-side name is not a device address: look the
      // address up once per device, with that device current.
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_partials) != cudaSuccess)
        return elgb::kElRuntimeError;
      g_noalloc_addr[dev] = static_cast<double*>(p);
    }
    partials = g_noalloc_addr[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  for (int c = 0; c < nrhs; c += 16) {
    const int qc = nrhs - c < 16 ? nrhs - c : 16;
    cudaError_t e = elgb::launch_residual_f64(n, qc, A, lda, X + (long)c * ldx, ldx,
                                              B + (long)c * ldb, ldb, R + (long)c * ldr, ldr,
                                              partials, st);
    if (e != cudaSuccess) return elgb::kElRuntimeError;
  }
  return 0;
}
