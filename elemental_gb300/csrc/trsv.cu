// One-launch blocked triangular solve for a few right-hand sides, used by
// the refinement loop's low-precision solves (the Trsm(LEFT, LOWER/UPPER,
// NORMAL) pair of lu::SolveAfter, src/lapack_like/factor/LU/SolveAfter.hpp:84-86,
// applied with the preconditioner's factors).
//
// The n rows are cut into 64-row block rows.  CTAs draw block rows from an
// atomic ticket in solve order (top-down for lower, bottom-up for upper); the
// CTA holding block row i subtracts the contribution of every earlier block
// row j as soon as j's "done" flag carries this call's epoch, then applies
// the pre-inverted diagonal block and publishes X_i with a release store.  A
// ticket is only ever held by a running CTA and waits only on smaller
// tickets, so the chain always progresses; every wait is bounded anyway and
// a timeout (or another CTA's error) makes all CTAs bail out.
#include "trsv.h"

namespace elgb {

namespace {

constexpr int kB = 64;        // block rows
constexpr int kQ = 16;        // right-hand sides per launch
constexpr int kThreads = 256;

__device__ __forceinline__ void st_release_gpu(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_acquire_gpu_s32(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Inverse of each 64 x 64 diagonal block of the lower (unit or not) or upper
// triangle of A, column-major per block at Dinv + b * 4096.  Rows/columns
// past n are padded with the identity.
template <typename T>
__global__ void __launch_bounds__(kThreads)
trtri_diag_kernel(const T* __restrict__ A, long lda, int n, int lower, int unit,
                  T* __restrict__ Dinv) {
  __shared__ T sA[kB][kB + 1];
  __shared__ T sX[kB][kB + 1];
  const int b = blockIdx.x, i0 = b * kB, nb = min(kB, n - i0);
  for (int idx = threadIdx.x; idx < kB * kB; idx += blockDim.x) {
    const int r = idx % kB, c = idx / kB;
    T v;
    if (r < nb && c < nb)
      v = A[(i0 + r) + (long)(i0 + c) * lda];
    else
      v = (r == c) ? T(1) : T(0);
    if (unit && r == c) v = T(1);
    sA[r][c] = v;
    sX[r][c] = (r == c) ? T(1) : T(0);
  }
  for (int step = 0; step < kB; ++step) {
    const int k = lower ? step : kB - 1 - step;
    __syncthreads();
    if (!unit) {
      const T d = sA[k][k];
      for (int c = threadIdx.x; c < kB; c += blockDim.x) sX[k][c] = sX[k][c] / d;
      __syncthreads();
    }
    for (int idx = threadIdx.x; idx < kB * kB; idx += blockDim.x) {
      const int r = idx % kB, c = idx / kB;
      if (lower ? r > k : r < k) sX[r][c] = fma(-sA[r][k], sX[k][c], sX[r][c]);
    }
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < kB * kB; idx += blockDim.x) {
    const int r = idx % kB, c = idx / kB;
    Dinv[(long)b * kB * kB + r + c * kB] = sX[r][c];
  }
}

// Thread t owns row r = t % 64 of its block row and the k-slice
// [16 g, 16 g + 16) of every 64 x 64 tile (g = t / 64), with all q columns
// in registers; the four slices are summed once at the end.  The A tile of
// the next dependency is loaded before waiting for its flag, and the block
// row's inverted diagonal block sits in shared memory from the start, so a
// link of the dependency chain is: flag -> X_j tile -> 256 FMAs -> done.
template <typename T>
__global__ void __launch_bounds__(kThreads)
trsv_persistent_kernel(const T* __restrict__ A, long lda, const T* __restrict__ Dinv,
                       T* __restrict__ X, long ldx, int n, int q, int lower,
                       unsigned* __restrict__ ticket, int* __restrict__ flags, int epoch,
                       DevStatus* st) {
  __shared__ T sD[kB * kB];
  __shared__ T xs[2][kB][kQ + 1];
  __shared__ T red[4][kB][kQ + 1];
  __shared__ int s_blk, s_abort;
  const int nblk = (n + kB - 1) / kB;
  const int tid = threadIdx.x, r = tid & (kB - 1), g = tid >> 6;
  while (true) {
    __syncthreads();
    if (tid == 0) {
      s_blk = (int)atomicAdd(ticket, 1u);
      s_abort = 0;
    }
    __syncthreads();
    const int t = s_blk;
    if (t >= nblk) break;
    const int bi = lower ? t : nblk - 1 - t;
    const int i0 = bi * kB, nbi = min(kB, n - i0);
    for (int idx = tid; idx < kB * kB; idx += blockDim.x) sD[idx] = Dinv[(long)bi * kB * kB + idx];
    T acc[kQ];
#pragma unroll
    for (int c = 0; c < kQ; ++c) acc[c] = T(0);
    T a[16];
    auto load_tile = [&](int s) {
      const int bj = lower ? s : nblk - 1 - s;
      const int j0 = bj * kB, nbj = min(kB, n - j0);
      const T* ap = A + (i0 + r) + (long)(j0 + 16 * g) * lda;
#pragma unroll
      for (int u = 0; u < 16; ++u)
        a[u] = (r < nbi && 16 * g + u < nbj) ? ap[(long)u * lda] : T(0);
    };
    if (t > 0) load_tile(0);
    for (int s = 0; s < t; ++s) {
      const int bj = lower ? s : nblk - 1 - s;
      const int j0 = bj * kB, nbj = min(kB, n - j0);
      const int buf = s & 1;
      if (tid == 0) {
        if (ld_acquire_gpu_s32(flags + bj) != epoch) {
          const unsigned long long t0 = globaltimer_ns();
          while (ld_acquire_gpu_s32(flags + bj) != epoch) {
            if (*(volatile int*)&st->err != 0) {
              s_abort = 1;
              break;
            }
            if (globaltimer_ns() - t0 > kSpinLimitNs) {
              atomicCAS(&st->err, 0, (int)kErrBarrierTimeout);
              st->err_where = 30;
              s_abort = 1;
              break;
            }
          }
        }
      }
      __syncthreads();
      if (s_abort) break;
      for (int idx = tid; idx < kB * kQ; idx += blockDim.x) {
        const int rr = idx % kB, cc = idx / kB;
        xs[buf][rr][cc] = (rr < nbj && cc < q) ? __ldcg(X + (j0 + rr) + (long)cc * ldx) : T(0);
      }
      __syncthreads();
      T cur[16];
#pragma unroll
      for (int u = 0; u < 16; ++u) cur[u] = a[u];
      if (s + 1 < t) load_tile(s + 1);  // next tile in flight during the FMAs
#pragma unroll
      for (int u = 0; u < 16; ++u) {
        const T av = cur[u];
#pragma unroll
        for (int c = 0; c < kQ; ++c) acc[c] = fma(-av, xs[buf][16 * g + u][c], acc[c]);
      }
    }
    if (s_abort) break;
    // sum the four k-slices, add the right-hand side, apply inv(D_bi)
#pragma unroll
    for (int c = 0; c < kQ; ++c) red[g][r][c] = acc[c];
    __syncthreads();
    for (int idx = tid; idx < kB * kQ; idx += blockDim.x) {
      const int rr = idx % kB, cc = idx / kB;
      const T b = (rr < nbi && cc < q) ? X[(i0 + rr) + (long)cc * ldx] : T(0);
      xs[0][rr][cc] = b + red[0][rr][cc] + red[1][rr][cc] + red[2][rr][cc] + red[3][rr][cc];
    }
    __syncthreads();
    T out[4] = {T(0), T(0), T(0), T(0)};
    for (int kk = 0; kk < kB; ++kk) {
      const T d = sD[r + kk * kB];
#pragma unroll
      for (int c4 = 0; c4 < 4; ++c4) out[c4] = fma(d, xs[0][kk][g * 4 + c4], out[c4]);
    }
#pragma unroll
    for (int c4 = 0; c4 < 4; ++c4) {
      const int c = g * 4 + c4;
      if (r < nbi && c < q) X[(i0 + r) + (long)c * ldx] = out[c4];
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) st_release_gpu(flags + bi, epoch);
  }
}

}  // namespace

int trsv_blocks(int n) { return (n + kB - 1) / kB; }

template <typename T>
cudaError_t launch_trtri_diag(const T* A, long lda, int n, bool lower, bool unit, T* Dinv,
                              cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  trtri_diag_kernel<T><<<trsv_blocks(n), kThreads, 0, stream>>>(A, lda, n, lower ? 1 : 0,
                                                                unit ? 1 : 0, Dinv);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_trsv_persistent(const T* A, long lda, const T* Dinv, T* X, long ldx, int n,
                                   int q, bool lower, unsigned* ticket, int* flags, int epoch,
                                   DevStatus* st, int num_sms, cudaStream_t stream) {
  if (n <= 0 || q <= 0) return cudaSuccess;
  if (q > kQ) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(ticket, 0, sizeof(unsigned), stream);
  if (e != cudaSuccess) return e;
  const int nblk = trsv_blocks(n);
  const int grid = std::min(nblk, 4 * num_sms);
  trsv_persistent_kernel<T><<<grid, kThreads, 0, stream>>>(A, lda, Dinv, X, ldx, n, q,
                                                           lower ? 1 : 0, ticket, flags, epoch,
                                                           st);
  return cudaGetLastError();
}

template cudaError_t launch_trtri_diag<float>(const float*, long, int, bool, bool, float*,
                                              cudaStream_t);
template cudaError_t launch_trsv_persistent<float>(const float*, long, const float*, float*, long,
                                                   int, int, bool, unsigned*, int*, int,
                                                   DevStatus*, int, cudaStream_t);

}  // namespace elgb
