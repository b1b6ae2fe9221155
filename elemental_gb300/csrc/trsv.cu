// One-launch blocked triangular solve for a few right-hand sides, used by
// the refinement loop's low-precision solves (the Trsm(LEFT, LOWER/UPPER,
// NORMAL) pair of lu::SolveAfter, src/lapack_like/factor/LU/SolveAfter.hpp:84-86,
// applied with the preconditioner's factors).
//
// The n rows are cut into 64-row block rows.  CTAs draw block rows from an
// atomic ticket in solve order (top-down for lower, bottom-up for upper); the
// CTA holding block row i subtracts the contribution of every earlier block
// row as soon as that row's published words carry this call's epoch, then
// publishes its own.  A ticket is only ever held by a running CTA and waits
// only on smaller tickets, so the chain always progresses; every wait is
// bounded anyway and a timeout (or another CTA's error) makes all CTAs bail
// out.
#include "trsv.h"

namespace elgb {

namespace {

constexpr int kB = 64;        // block rows
constexpr int kQ = 16;        // right-hand sides per launch
constexpr int kThreads = 256;

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

__device__ __forceinline__ void st_tag(unsigned long long* p, float v, unsigned epoch) {
  const unsigned long long w = ((unsigned long long)epoch << 32) | __float_as_uint(v);
  asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(w) : "memory");
}
__device__ __forceinline__ unsigned long long ld_tag(const unsigned long long* p) {
  unsigned long long w;
  asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(w) : "l"(p) : "memory");
  return w;
}

// Waits until every word of a published 64 x 16 tile (word c * 64 + r)
// carries `epoch` and copies the values to xs[r][c].  A word is one 64-bit
// store of (epoch, value), so the value read with the current epoch is the
// one published with it: no flag, no fence, one round trip.  `tight`: the
// wait on the chain's predecessor spins; the others back off a little
// (many CTAs wait on the same tile).  Bounded; returns false (all threads)
// on a timeout or another CTA's error.
__device__ __forceinline__ bool wait_tile(const unsigned long long* tile, unsigned epoch,
                                          float (*xs)[kQ + 1], bool tight, DevStatus* st,
                                          int where, int* s_fail) {
  const int tid = threadIdx.x;
  unsigned long long w[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) w[k] = ld_tag(tile + tid + kThreads * k);
  auto ready = [&]() {
    bool r = true;
#pragma unroll
    for (int k = 0; k < 4; ++k) r = r && (unsigned)(w[k] >> 32) == epoch;
    return r;
  };
  if (!ready()) {
    const unsigned long long t0 = globaltimer_ns();
    while (true) {
      if (!tight) __nanosleep(64);
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if ((unsigned)(w[k] >> 32) != epoch) w[k] = ld_tag(tile + tid + kThreads * k);
      if (ready()) break;
      if (*(volatile int*)&st->err != 0) {
        *s_fail = 1;
        break;
      }
      if (globaltimer_ns() - t0 > kSpinLimitNs) {
        atomicCAS(&st->err, 0, (int)kErrBarrierTimeout);
        st->err_where = where;
        *s_fail = 1;
        break;
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int idx = tid + kThreads * k;
    xs[idx & (kB - 1)][idx >> 6] = __uint_as_float((unsigned)w[k]);
  }
  __syncthreads();
  return *s_fail == 0;
}

// Blocked forward (lower) or backward (upper) substitution.  With D_i the
// diagonal blocks, the CTA of block row i computes y_i = b_i - sum_j A_ij x_j
// and x_i = D_i^{-1} y_i.  It publishes y_i first: its successor s took
// M = A_si D_i^{-1} while waiting, so the chain's link from i to s is one
// 64 x 64 tile times y_i -- the inverse diagonal block is off the chain.
// Then x_i, which every later block row uses for its other tiles, and the
// solution itself in X.  Published words: tags[0][block][c * 64 + r] = y,
// tags[1][block][...] = x, each (epoch, value).
// Thread t owns row r = t % 64 of its block row and the k-slice
// [16 g, 16 g + 16) of every 64 x 64 tile (g = t / 64), with all q columns
// in registers; the four slices are summed once at the end.  The next A
// tile is loaded before waiting for its x.
template <typename T>
__global__ void __launch_bounds__(kThreads)
trsv_persistent_kernel(const T* __restrict__ A, long lda, const T* __restrict__ Dinv,
                       T* __restrict__ X, long ldx, int n, int q, int lower,
                       unsigned* __restrict__ ticket, unsigned long long* __restrict__ tags,
                       unsigned epoch, DevStatus* st) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sD = reinterpret_cast<T*>(smem_raw);                              // D_i^{-1}
  T(*sM)[kB + 1] = reinterpret_cast<T(*)[kB + 1]>(sD + kB * kB);       // A_ip D_p^{-1}
  T(*xs)[kB][kQ + 1] = reinterpret_cast<T(*)[kB][kQ + 1]>(&sM[kB][0]);  // 2 tiles
  T(*red)[kB][kQ + 1] = reinterpret_cast<T(*)[kB][kQ + 1]>(&xs[2][0][0]);  // 4 slices
  T* sDp = &red[0][0][0];  // D_p^{-1}, staged before the slices are written
  __shared__ int s_blk, s_fail;
  const int nblk = (n + kB - 1) / kB;
  const int tid = threadIdx.x, r = tid & (kB - 1), g = tid >> 6;
  const long tile_words = (long)kB * kQ;
  unsigned long long* ytags = tags;
  unsigned long long* xtags = tags + (long)nblk * tile_words;
  while (true) {
    __syncthreads();
    if (tid == 0) {
      s_blk = (int)atomicAdd(ticket, 1u);
      s_fail = 0;
    }
    __syncthreads();
    const int t = s_blk;
    if (t >= nblk) break;
    const int bi = lower ? t : nblk - 1 - t;
    const int i0 = bi * kB, nbi = min(kB, n - i0);
    for (int idx = tid; idx < kB * kB; idx += blockDim.x) sD[idx] = Dinv[(long)bi * kB * kB + idx];
    // M = A_ip D_p^{-1} for the predecessor p, before any wait
    const int bp = lower ? bi - 1 : bi + 1;
    if (t > 0) {
      const int p0 = bp * kB, nbp = min(kB, n - p0);
      for (int idx = tid; idx < kB * kB; idx += blockDim.x)
        sDp[idx] = Dinv[(long)bp * kB * kB + idx];
      __syncthreads();
      T m[16];
#pragma unroll
      for (int u = 0; u < 16; ++u) m[u] = T(0);
      const T* ap = A + (i0 + r) + (long)p0 * lda;
      for (int k0 = 0; k0 < kB; k0 += 8) {
        T tv[8];
#pragma unroll
        for (int e = 0; e < 8; ++e)
          tv[e] = (r < nbi && k0 + e < nbp) ? ap[(long)(k0 + e) * lda] : T(0);
#pragma unroll
        for (int e = 0; e < 8; ++e)
#pragma unroll
          for (int u = 0; u < 16; ++u)
            m[u] = fma(tv[e], sDp[(k0 + e) + (16 * g + u) * kB], m[u]);
      }
#pragma unroll
      for (int u = 0; u < 16; ++u) sM[r][16 * g + u] = m[u];
    }
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
    // every earlier block row but the predecessor, with its x
    const int nreg = t - 1;
    if (nreg > 0) load_tile(0);
    for (int s = 0; s < nreg; ++s) {
      const int bj = lower ? s : nblk - 1 - s;
      const int buf = s & 1;
      if (!wait_tile(xtags + (long)bj * tile_words, epoch, xs[buf], false, st, 30, &s_fail))
        break;
      T cur[16];
#pragma unroll
      for (int u = 0; u < 16; ++u) cur[u] = a[u];
      if (s + 1 < nreg) load_tile(s + 1);  // next tile in flight during the FMAs
#pragma unroll
      for (int u = 0; u < 16; ++u) {
        const T av = cur[u];
#pragma unroll
        for (int c = 0; c < kQ; ++c) acc[c] = fma(-av, xs[buf][16 * g + u][c], acc[c]);
      }
    }
    if (s_fail) break;  // uniform: read after wait_tile's barrier
    // the predecessor's y: the link of the chain
    if (t > 0) {
      const int buf = (nreg > 0 ? nreg : 0) & 1;
      if (!wait_tile(ytags + (long)bp * tile_words, epoch, xs[buf], true, st, 31, &s_fail))
        break;
#pragma unroll
      for (int u = 0; u < 16; ++u) {
        const T mv = sM[r][16 * g + u];
#pragma unroll
        for (int c = 0; c < kQ; ++c) acc[c] = fma(-mv, xs[buf][16 * g + u][c], acc[c]);
      }
    }
    // y_i = b_i + the four slices; publish it for the successor
#pragma unroll
    for (int c = 0; c < kQ; ++c) red[g][r][c] = acc[c];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int idx = tid + kThreads * k;
      const int rr = idx & (kB - 1), cc = idx >> 6;
      const bool ok = rr < nbi && cc < q;
      const T y = ok ? X[(i0 + rr) + (long)cc * ldx] + red[0][rr][cc] + red[1][rr][cc] +
                           red[2][rr][cc] + red[3][rr][cc]
                     : T(0);
      xs[0][rr][cc] = y;
      st_tag(ytags + (long)bi * tile_words + idx, y, epoch);
    }
    __syncthreads();
    // x_i = D_i^{-1} y_i: publish it and write the solution
    T out[4] = {T(0), T(0), T(0), T(0)};
    for (int kk = 0; kk < kB; ++kk) {
      const T d = sD[r + kk * kB];
#pragma unroll
      for (int c4 = 0; c4 < 4; ++c4) out[c4] = fma(d, xs[0][kk][g * 4 + c4], out[c4]);
    }
#pragma unroll
    for (int c4 = 0; c4 < 4; ++c4) {
      const int c = g * 4 + c4;
      st_tag(xtags + (long)bi * tile_words + c * kB + r, out[c4], epoch);
      if (r < nbi && c < q) X[(i0 + r) + (long)c * ldx] = out[c4];
    }
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

size_t trsv_tag_words(int n) { return (size_t)2 * trsv_blocks(n) * kB * kQ; }

template <typename T>
cudaError_t launch_trsv_persistent(const T* A, long lda, const T* Dinv, T* X, long ldx, int n,
                                   int q, bool lower, unsigned* ticket, unsigned long long* tags,
                                   unsigned epoch, DevStatus* st, int num_sms,
                                   cudaStream_t stream) {
  if (n <= 0 || q <= 0) return cudaSuccess;
  if (q > kQ) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(ticket, 0, sizeof(unsigned), stream);
  if (e != cudaSuccess) return e;
  const size_t smem = (size_t)(kB * kB + kB * (kB + 1) + 6 * kB * (kQ + 1)) * sizeof(T);
  auto kern = trsv_persistent_kernel<T>;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  // resident CTAs only: a CTA that is not yet running holds no ticket, but
  // it would only take its block rows late
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem) !=
          cudaSuccess ||
      per_sm < 1) {
    cudaGetLastError();
    per_sm = 1;
  }
  const int nblk = trsv_blocks(n);
  const int grid = std::min(nblk, per_sm * num_sms);
  kern<<<grid, kThreads, smem, stream>>>(A, lda, Dinv, X, ldx, n, q, lower ? 1 : 0, ticket, tags,
                                         epoch, st);
  return cudaGetLastError();
}

template cudaError_t launch_trtri_diag<float>(const float*, long, int, bool, bool, float*,
                                              cudaStream_t);
template cudaError_t launch_trsv_persistent<float>(const float*, long, const float*, float*, long,
                                                   int, int, bool, unsigned*, unsigned long long*,
                                                   unsigned, DevStatus*, int, cudaStream_t);

}  // namespace elgb
