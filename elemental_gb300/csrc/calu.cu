// Tournament pivoting for the low-precision (preconditioner) factorization:
// the w-column leaf panel of the FP32 LU chooses its w pivot rows by a
// reduction tree of small partial-pivoting eliminations (communication-
// avoiding LU, Grigori, Demmel and Xiang, "CALU", SIMAX 2011) instead of one
// grid-wide argmax exchange per column.  The result is an LU factorization
// with row interchanges -- same packed layout and swap-sequence convention
// as El::LU -- whose pivots may differ from partial pivoting's; the mixed-
// precision solve only needs a good preconditioner, and refinement to the
// FP64 backward error checks it.  The plain-precision El::LU path keeps
// partial pivoting (lu_kernels.cu, getf2_panel_kernel).
//
//   calu_local_kernel  G CTAs: each takes its rows (as getf2's partition),
//                      and reduces groups of 32 rows pairwise -- a warp
//                      eliminates 2 x 32 candidate rows with partial
//                      pivoting and keeps the w it picked -- down to one
//                      candidate list per CTA;
//   calu_final_kernel  one CTA: the same tree over the G lists (candidate
//                      rows re-read from A), then the swap sequence of the w
//                      winners (in pivot order), the interchanges on the
//                      panel's columns and the unpivoted LU of its top block;
//   calu_l21_kernel    every row below the top block: l = a U11^{-1}.
#include <algorithm>

#include "kernels.h"

namespace elgb {

namespace {

constexpr int kW = 32;        // panel width handled (w <= 32)
constexpr int kThreads = 256;
constexpr int kStride = kW + 1;  // shared-memory row stride (conflict-free)

// One warp picks up to w pivot rows out of n_c <= 64 candidates by partial
// pivoting on their (original) rows.  rows(i) -> pointer to candidate i's
// w values (stride `cs` between columns); ids[i] its global panel row.
// Ties: larger |a|, then the lower row id (idamax's first index).  Writes
// the picked ids in pivot order to out[0 .. min(w, n_c)) and returns the
// count.  Every lane of the warp must call it.
template <typename GetRow>
__device__ int warp_tournament(int n_c, const int* ids, int w, GetRow get, int* out) {
  const int lane = threadIdx.x & 31;
  float v0[kW], v1[kW];
  const bool h0 = lane < n_c, h1 = lane + 32 < n_c;
  const int id0 = h0 ? ids[lane] : 0x7fffffff, id1 = h1 ? ids[lane + 32] : 0x7fffffff;
#pragma unroll
  for (int c = 0; c < kW; ++c) {
    v0[c] = (h0 && c < w) ? get(lane, c) : 0.f;
    v1[c] = (h1 && c < w) ? get(lane + 32, c) : 0.f;
  }
  bool t0 = !h0, t1 = !h1;  // taken (or absent)
  const int picks = min(w, n_c);
#pragma unroll 1
  for (int j = 0; j < picks; ++j) {
    // this lane's best live candidate in column j
    float bv = -1.f;
    int bid = 0x7fffffff, bsel = -1;
    float a0 = 0.f, a1 = 0.f;
#pragma unroll
    for (int c = 0; c < kW; ++c)
      if (c == j) {
        a0 = v0[c];
        a1 = v1[c];
      }
    if (!t0) {
      bv = fabsf(a0);
      bid = id0;
      bsel = 0;
    }
    if (!t1) {
      const float v = fabsf(a1);
      if (v > bv || (v == bv && id1 < bid)) {
        bv = v;
        bid = id1;
        bsel = 1;
      }
    }
    int blane = lane;
    for (int o = 16; o > 0; o >>= 1) {
      const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
      const int oid = __shfl_xor_sync(0xffffffffu, bid, o);
      const int ol = __shfl_xor_sync(0xffffffffu, blane, o);
      const int os = __shfl_xor_sync(0xffffffffu, bsel, o);
      if (ov > bv || (ov == bv && oid < bid)) {
        bv = ov;
        bid = oid;
        blane = ol;
        bsel = os;
      }
    }
    if (lane == 0) out[j] = bid;
    const bool mine0 = lane == blane && bsel == 0, mine1 = lane == blane && bsel == 1;
    if (mine0) t0 = true;
    if (mine1) t1 = true;
    // pivot row broadcast and elimination of the live rows
    float piv = 0.f;
#pragma unroll
    for (int c = 0; c < kW; ++c) {
      const float mine = bsel == 0 ? v0[c] : v1[c];
      const float u = __shfl_sync(0xffffffffu, mine, blane);
      if (c == j) piv = u;
    }
    const float inv = piv != 0.f ? 1.f / piv : 0.f;
    const float l0 = t0 ? 0.f : a0 * inv, l1 = t1 ? 0.f : a1 * inv;
#pragma unroll
    for (int c = 0; c < kW; ++c) {
      const float mine = bsel == 0 ? v0[c] : v1[c];
      const float u = __shfl_sync(0xffffffffu, mine, blane);
      if (c > j) {
        v0[c] = fmaf(-l0, u, v0[c]);
        v1[c] = fmaf(-l1, u, v1[c]);
      }
    }
  }
  __syncwarp();
  return picks;
}

// Pairwise tree over `nl` candidate lists (lists[i][0..cnt[i])) in shared
// memory until one list remains in lists[0]; get(list, k, c) reads value c
// of list `list`'s k-th candidate's row.  All warps of the CTA take part.
template <typename Get>
__device__ void cta_tree(int nl, int* lists, int* cnt, int w, Get get) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __shared__ int s_ids[kThreads / 32][2 * kW];
  __shared__ int s_out[kThreads / 32][kW];
  for (int step = 1; step < nl; step *= 2) {
    // merge list i and i + step into i, for i multiple of 2*step
    const int npair = (nl + 2 * step - 1) / (2 * step);
    for (int p = warp; p < npair; p += kThreads / 32) {
      const int a = p * 2 * step, b = a + step;
      if (b >= nl) continue;  // odd one out: passes through
      const int na = cnt[a], nbc = cnt[b];
      if (lane < na) s_ids[warp][lane] = lists[a * kW + lane];
      if (lane < nbc) s_ids[warp][na + lane] = lists[b * kW + lane];
      __syncwarp();
      const int n_c = na + nbc;
      // candidate k's source: list a's k-th or list b's (k - na)-th
      auto getrow = [&](int k, int c) { return k < na ? get(a, k, c) : get(b, k - na, c); };
      const int picked = warp_tournament(n_c, s_ids[warp], w, getrow, s_out[warp]);
      __syncwarp();
      if (lane < picked) lists[a * kW + lane] = s_out[warp][lane];
      if (lane == 0) cnt[a] = picked;
      __syncwarp();
    }
    __syncthreads();
  }
}

struct CaluArgs {
  float* A;
  long lda;
  int mp, w, R;
  int* ipiv;
  int row_base, info_base;
  int* cand;  // G x (kW + 1): count, then the CTA's candidate panel rows
  DevStatus* st;
};

__global__ void __launch_bounds__(kThreads)
calu_local_kernel(CaluArgs p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* slab = reinterpret_cast<float*>(smem_raw);  // R rows x kStride
  const int b = blockIdx.x, R = p.R, w = p.w;
  const int rb = b * R, nr = max(min(rb + R, p.mp) - rb, 0);
  const int ng = (nr + kW - 1) / kW;
  int* lists = reinterpret_cast<int*>(slab + (size_t)R * kStride);  // ng x kW
  int* cnt = lists + (size_t)ng * kW;
  for (int c = 0; c < w; ++c)
    for (int r = threadIdx.x; r < nr; r += kThreads)
      slab[r * kStride + c] = p.A[(long)(rb + r) + (long)c * p.lda];
  for (int g = threadIdx.x; g < ng; g += kThreads) cnt[g] = min(kW, nr - g * kW);
  for (int i = threadIdx.x; i < ng * kW; i += kThreads) lists[i] = rb + i;  // panel row ids
  __syncthreads();
  // candidate value: row id -> local slab row
  cta_tree(ng, lists, cnt, w,
           [&](int l, int k, int c) { return slab[(lists[l * kW + k] - rb) * kStride + c]; });
  int* out = p.cand + (long)b * (kW + 1);
  if (threadIdx.x == 0) out[0] = ng > 0 ? cnt[0] : 0;
  if (ng > 0 && threadIdx.x < cnt[0]) out[1 + threadIdx.x] = lists[threadIdx.x];
}

// The winners of all CTAs, then the panel's interchanges and its top block.
__global__ void __launch_bounds__(kThreads)
calu_final_kernel(CaluArgs p, int G) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* rows = reinterpret_cast<float*>(smem_raw);  // G*kW candidate rows x kStride
  int* lists = reinterpret_cast<int*>(rows + (size_t)G * kW * kStride);  // G x kW
  int* cnt = lists + (size_t)G * kW;
  __shared__ int s_pos[2 * kW], s_org[2 * kW], s_n;
  __shared__ int s_q[kW];
  __shared__ float s_top[2 * kW][kStride];
  const int w = p.w;
  for (int g = threadIdx.x; g < G; g += kThreads) cnt[g] = p.cand[(long)g * (kW + 1)];
  for (int i = threadIdx.x; i < G * kW; i += kThreads) {
    const int g = i / kW, k = i % kW;
    lists[i] = k < p.cand[(long)g * (kW + 1)] ? p.cand[(long)g * (kW + 1) + 1 + k] : 0;
  }
  __syncthreads();
  // candidate rows' values, slot (g, k) at rows[(g*kW + k) * kStride]
  for (int i = threadIdx.x; i < G * kW * w; i += kThreads) {
    const int c = i / (G * kW), s = i % (G * kW);
    const int g = s / kW, k = s % kW;
    rows[s * kStride + c] = k < cnt[g] ? p.A[(long)lists[s] + (long)c * p.lda] : 0.f;
  }
  __syncthreads();
  // the tree moves ids, so keep a map id -> slot: candidate ids are unique
  // panel rows; look them up in the original slot layout by a linear probe
  // of this CTA's... simpler: carry (slot index) as the id during the tree.
  for (int i = threadIdx.x; i < G * kW; i += kThreads) lists[i] = i;  // slot ids
  __syncthreads();
  cta_tree(G, lists, cnt, w, [&](int l, int k, int c) {
    return rows[lists[l * kW + k] * kStride + c];
  });
  // slot ids -> panel rows, in pivot order
  if (threadIdx.x < kW) {
    const int s = threadIdx.x < cnt[0] ? lists[threadIdx.x] : 0;
    s_q[threadIdx.x] = threadIdx.x < cnt[0] ? p.cand[(long)(s / kW) * (kW + 1) + 1 + s % kW] : -1;
  }
  __syncthreads();
  // swap sequence: position j takes winner j; track the (position, original
  // row) pairs that moved
  if (threadIdx.x == 0) {
    int n = 0;
    const int picks = min(w, cnt[0]);
    for (int j = 0; j < picks; ++j) {
      const int want = s_q[j];
      int q = want;  // current position of original row `want`
      for (int t = 0; t < n; ++t)
        if (s_org[t] == want) {
          q = s_pos[t];
          break;
        }
      p.ipiv[j] = p.row_base + q;
      if (q != j) {
        // exchange the originals at positions j and q
        int oj = j, oq = q, tj = -1, tq = -1;
        for (int t = 0; t < n; ++t) {
          if (s_pos[t] == j) {
            oj = s_org[t];
            tj = t;
          }
          if (s_pos[t] == q) {
            oq = s_org[t];
            tq = t;
          }
        }
        if (tj < 0) {
          tj = n++;
          s_pos[tj] = j;
        }
        if (tq < 0) {
          tq = n++;
          s_pos[tq] = q;
        }
        s_org[tj] = oq;
        s_org[tq] = oj;
      }
    }
    for (int j = picks; j < w; ++j) p.ipiv[j] = p.row_base + j;  // (fewer rows than w)
    s_n = n;
  }
  __syncthreads();
  // apply to the panel's w columns: position t receives original row s_org
  const int n = s_n;
  for (int i = threadIdx.x; i < n * w; i += kThreads) {
    const int t = i % n, c = i / n;
    s_top[t][c] = p.A[(long)s_org[t] + (long)c * p.lda];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n * w; i += kThreads) {
    const int t = i % n, c = i / n;
    p.A[(long)s_pos[t] + (long)c * p.lda] = s_top[t][c];
  }
  __syncthreads();
  // unpivoted LU of the top w x w block (the winners, in pivot order)
  for (int i = threadIdx.x; i < w * w; i += kThreads) {
    const int r = i % w, c = i / w;
    s_top[r][c] = p.A[(long)r + (long)c * p.lda];
  }
  __syncthreads();
  for (int j = 0; j < w; ++j) {
    const float a = s_top[j][j];
    if (a == 0.f && threadIdx.x == 0) atomicCAS(&p.st->info, 0, p.info_base + j + 1);
    const float inv = a != 0.f ? 1.f / a : 0.f;
    __syncthreads();
    for (int r = j + 1 + threadIdx.x; r < w; r += kThreads) {
      const float l = s_top[r][j] * inv;
      s_top[r][j] = l;
      for (int c = j + 1; c < w; ++c) s_top[r][c] = fmaf(-l, s_top[j][c], s_top[r][c]);
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < w * w; i += kThreads) {
    const int r = i % w, c = i / w;
    p.A[(long)r + (long)c * p.lda] = s_top[r][c];
  }
}

// Rows below the top block: l U11 = a (U11 upper, from the factored top).
__global__ void __launch_bounds__(kThreads)
calu_l21_kernel(CaluArgs p) {
  __shared__ float U[kW][kStride];
  const int w = p.w;
  for (int i = threadIdx.x; i < w * w; i += kThreads) {
    const int r = i % w, c = i / w;
    U[r][c] = p.A[(long)r + (long)c * p.lda];
  }
  __syncthreads();
  for (long r = w + blockIdx.x * (long)kThreads + threadIdx.x; r < p.mp;
       r += (long)gridDim.x * kThreads) {
    float x[kW];
#pragma unroll
    for (int c = 0; c < kW; ++c) x[c] = c < w ? p.A[r + (long)c * p.lda] : 0.f;
#pragma unroll
    for (int c = 0; c < kW; ++c) {
      if (c < w) {
        float s = x[c];
#pragma unroll
        for (int k = 0; k < c; ++k) s = fmaf(-x[k], U[k][c], s);
        const float d = U[c][c];
        x[c] = d != 0.f ? s / d : 0.f;
      }
    }
#pragma unroll
    for (int c = 0; c < kW; ++c)
      if (c < w) p.A[r + (long)c * p.lda] = x[c];
  }
}

}  // namespace

size_t calu_scratch_ints(int max_ctas) { return (size_t)max_ctas * (kW + 1); }

cudaError_t launch_calu_panel(float* A, long lda, int mp, int w, int* ipiv, int row_base,
                              int info_base, int* cand, int max_ctas, DevStatus* st,
                              int num_sms, cudaStream_t stream, int* nlaunch) {
  *nlaunch = 0;
  if (w <= 0 || mp <= 0) return cudaSuccess;
  if (w > kW || mp < w) return cudaErrorInvalidValue;
  constexpr size_t kMaxSmem = 200 * 1024;
  // rows per CTA: ~1024, fewer CTAs only where shared memory forces more
  const int rows_cap = (int)(kMaxSmem / (kStride * sizeof(float) + 2 * sizeof(int))) - 64;
  int G = std::max(ceil_div(mp, 1024), ceil_div(mp, rows_cap));
  G = std::max(1, std::min({G, num_sms, max_ctas}));
  const int R = ceil_div(mp, G);
  G = ceil_div(mp, R);
  const int ng = ceil_div(R, kW);
  const size_t smem1 = (size_t)R * kStride * sizeof(float) + ((size_t)ng * kW + ng) * sizeof(int);
  const size_t smem2 = (size_t)G * kW * kStride * sizeof(float) + ((size_t)G * kW + G) * sizeof(int);
  if (smem1 > kMaxSmem || smem2 > kMaxSmem) return cudaErrorNotSupported;
  cudaError_t e = cudaFuncSetAttribute(calu_local_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(calu_final_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kMaxSmem);
  if (e != cudaSuccess) return e;
  CaluArgs a{A, lda, mp, w, R, ipiv, row_base, info_base, cand, st};
  calu_local_kernel<<<G, kThreads, smem1, stream>>>(a);
  calu_final_kernel<<<1, kThreads, smem2, stream>>>(a, G);
  const int rows = mp - w;
  if (rows > 0) {
    const int grid = std::max(1, std::min(ceil_div(rows, kThreads), 4 * num_sms));
    calu_l21_kernel<<<grid, kThreads, 0, stream>>>(a);
  }
  *nlaunch = rows > 0 ? 3 : 2;
  return cudaGetLastError();
}

}  // namespace elgb
