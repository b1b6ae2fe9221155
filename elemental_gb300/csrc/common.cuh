// Shared device helpers for the GB300 dense factor-and-solve kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace elgb {

// Device-side status word layout (one int per call, in device scratch).
// 0 = ok.  Factorizations record the first failing column (1-based, like
// LAPACK's info) in `info`; kernels that wait on other CTAs record a timeout
// in `err` instead of trapping.
struct DevStatus {
  int info;      // first zero pivot / non-positive diagonal, 1-based; 0 = none
  int err;       // nonzero: a bounded wait gave up (see ErrCode)
  int err_where; // which kernel / barrier gave up
  int pad;
};

enum ErrCode : int {
  kErrNone = 0,
  kErrBarrierTimeout = 1,
  kErrMbarTimeout = 2,
};

// Upper bound for any spin-wait on another CTA, in nanoseconds of
// %globaltimer.  A wait that exceeds it records kErrBarrierTimeout and
// returns; the host turns that into an error status.
constexpr unsigned long long kSpinLimitNs = 2000000000ull;  // 2 s

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialization may start while its predecessor on the stream still runs;
// pdl_wait() blocks until that predecessor has completed and its memory is
// visible (a no-op for a kernel launched normally).  pdl_launch_dependents()
// lets such a successor start being scheduled (no effect on any other).
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid-wide barrier for a cooperative launch.  `counter` starts at 0 before
// the launch; barrier number `epoch` (1, 2, ...) waits until all `nblocks`
// CTAs have arrived `epoch` times.  Returns false (after recording the
// timeout) if the wait exceeded kSpinLimitNs.
__device__ __forceinline__ bool grid_barrier(unsigned* counter, unsigned epoch,
                                             unsigned nblocks, DevStatus* st,
                                             int where) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(counter, 1u);
    const unsigned target = epoch * nblocks;
    int ok = 1;
    if (ld_acquire_gpu(counter) < target) {
      const unsigned long long t0 = globaltimer_ns();
      while (ld_acquire_gpu(counter) < target) {
        if (globaltimer_ns() - t0 > kSpinLimitNs) {
          atomicCAS(&st->err, 0, (int)kErrBarrierTimeout);
          st->err_where = where;
          ok = 0;
          break;
        }
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

template <typename T>
__device__ __forceinline__ T shfl_xor(T v, int lane_mask) {
  return __shfl_xor_sync(0xffffffffu, v, lane_mask);
}

// (|value|, row) argmax pair; ties resolve to the LOWER row index, matching
// the first-index rule of idamax / blas::MaxInd
// (src/core/imports/blas/MaxInd.hpp:25-44 uses a strict `>` scan).
template <typename T>
struct ArgMax {
  T absval;
  int row;
};

template <typename T>
__device__ __forceinline__ bool argmax_better(T a, int ra, T b, int rb) {
  // a beats b if strictly larger, or equal and lower row.  Empty slots carry
  // (-1, -1), which every |value| beats.  A NaN beats nothing, as in the
  // strict `>` scan; an all-NaN column yields row -1 and the caller falls
  // back to the diagonal row (what idamax returns for it).
  return (a > b) || (a == b && ra < rb);
}

template <typename T>
__device__ __forceinline__ void warp_argmax(T& v, int& r) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    T ov = shfl_xor(v, o);
    int orr = shfl_xor(r, o);
    if (argmax_better(ov, orr, v, r)) {
      v = ov;
      r = orr;
    }
  }
}

// FP32: two warp reductions instead of five shuffle rounds.  Non-negative
// floats order as their bit patterns, so the largest |value| is a max over
// (bits + 1), with empty slots (-1) and NaN mapped to 0, which never wins;
// the row is then the lowest among the lanes holding that value.  Without
// NaN the result equals argmax_better's order; every lane gets it.
__device__ __forceinline__ void warp_argmax(float& v, int& r) {
  const unsigned key = v >= 0.f ? (__float_as_uint(v) & 0x7fffffffu) + 1u : 0u;
  const unsigned kmax = __reduce_max_sync(0xffffffffu, key);
  const unsigned rmin =
      __reduce_min_sync(0xffffffffu, key == kmax ? (unsigned)r : 0xffffffffu);
  if (kmax == 0u) {
    v = -1.f;
    r = -1;
  } else {
    v = __uint_as_float(kmax - 1u);
    r = (int)rmin;
  }
}

__host__ __device__ constexpr int ceil_div(int a, int b) { return (a + b - 1) / b; }
// grid.y of a launch with one column per y index: at most 65535, so the
// kernels loop over the columns j = blockIdx.y, blockIdx.y + gridDim.y, ...
__host__ __device__ constexpr int grid_y(int ncols) { return ncols < 65535 ? ncols : 65535; }

}  // namespace elgb
