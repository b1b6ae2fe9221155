// CUDA-core kernels of the dense factor-and-solve path on GB300 (sm_103a):
// panel factorization with a warp-shuffle pivot search, row interchanges,
// small triangular solves, SIMT GEMM (the FP64 contraction: tcgen05 has no
// f64 kind), tall-skinny updates, the Cholesky diagonal block, the FP64
// residual and norms.  The tensor-core contractions live in tc_gemm.cu.
#include <cooperative_groups.h>

#include <algorithm>

#include "kernels.h"
#include "tcgen05.cuh"

namespace elgb {

// Largest thread-block cluster the panel may use (1: the cooperative kernel
// only); set by ElGBSetOption(ELGB_OPT_PANEL_CLUSTER).
int g_panel_cluster = 16;
// Rows per CTA the leaf-panel kernels aim for (ElGBSetOption(ELGB_OPT_PANEL_ROWS)).
int g_panel_rows = 512;
// FP32 panels with the rows in registers (ElGBSetOption(ELGB_OPT_PANEL_REGS)):
// 1 cooperative, 2 on a cluster where one fits (the default).
int g_panel_regs = 2;
int g_panel_push = 1;
int g_panel_pdl = 1;

template <typename T>
__device__ __forceinline__ T absv(T x) { return x < T(0) ? -x : x; }

// Block-wide (|value|, row) argmax over 8 warps; every thread gets the result.
template <typename T>
__device__ __forceinline__ void block_argmax(T& v, int& r, T* s_v, int* s_r) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  warp_argmax(v, r);
  __syncthreads();  // previous readers of s_v/s_r are done
  if (lane == 0) {
    s_v[warp] = v;
    s_r[warp] = r;
  }
  __syncthreads();
  if (warp == 0) {
    T wv = lane < nwarps ? s_v[lane] : T(-1);
    int wr = lane < nwarps ? s_r[lane] : -1;
    warp_argmax(wv, wr);
    if (lane == 0) {
      s_v[32] = wv;
      s_r[32] = wr;
    }
  }
  __syncthreads();
  v = s_v[32];
  r = s_r[32];
}

// The same without the leading barrier, for callers whose previous readers of
// s_v / s_r are already behind a barrier.
template <typename T>
__device__ __forceinline__ void block_argmax_nolead(T& v, int& r, T* s_v, int* s_r) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  warp_argmax(v, r);
  if (lane == 0) {
    s_v[warp] = v;
    s_r[warp] = r;
  }
  __syncthreads();
  // every warp reduces the per-warp results (no second broadcast barrier)
  T wv = lane < nwarps ? s_v[lane] : T(-1);
  int wr = lane < nwarps ? s_r[lane] : -1;
  warp_argmax(wv, wr);
  v = wv;
  r = wr;
}

// ---------------------------------------------------------------------------
// K1 + K3: panel factorization (lu::Panel, src/lapack_like/factor/LU/Panel.hpp:15-59)
// ---------------------------------------------------------------------------
// One cooperative launch factors a w-column panel (w <= W = 32).  CTA b owns
// panel rows [b*R, b*R + R) and keeps them in shared memory for the whole
// panel (column-major slab, slab[c * S + r], S = slab_stride(R)).  Per column j:
//   1. each CTA writes its slot: its best candidate (|a|, row) for column j
//      with that row, and (the owner of row j only) row j itself, then
//      publishes the slot with a release store of the column's epoch;
//   2. threads 0..G-1 poll the G slot epochs (acquire): seeing all of them is
//      the grid barrier, and the candidate headers arrive with it;
//   3. every warp reduces the candidates itself (ties -> lowest row,
//      idamax's rule); the winner's row and row j are already on chip;
//   4. the CTA writes the pivot row into row j if it owns row j, updates its
//      rows (the pivot row's position, if it owns it, starting from old row
//      j), scaling by the reciprocal of the pivot (El scales by alpha11Inv,
//      Panel.hpp:53-55) and applying the rank-1 update while computing its
//      candidate for column j+1.
// Four barriers per column: publish, exchange, and two in the argmax.
// Slots are double-buffered by column parity: a CTA can only rewrite a slot
// after every CTA has published the next column, i.e. finished reading this
// one.  Epochs grow across the launches of one factorization, so slots never
// need clearing between panels.
template <typename T>
struct PanelParams {
  T* A;
  long lda;
  int mp, w, R;
  int* ipiv;
  int row_base, info_base;
  int epoch_base;  // column j of this launch publishes epoch_base + j + 1
  PanelScratch<T> s;
  DevStatus* st;
  int nopiv;       // 1: El::LU without pivoting -- the pivot of column j is row j
  // the leaf's interchanges also applied to columns [swap_lo, 0) and
  // [w, swap_hi) (relative to A) by the kernels that do so (0, 0: none)
  int swap_lo, swap_hi;
  // > 0 (register cluster kernel): this leaf is the left child of a
  // recursion node whose right child is columns [w, w + sib_w); the kernel
  // also applies the node's update to them (U12 = L11^-1 A12 on rows
  // [0, w), A22 -= L21 U12 below), with trsm_block's and gemm_simt's
  // arithmetic in their order
  int sib_w;
};

constexpr int kPanelW = 32;
// Threads of a panel CTA: 512 for FP32 (two rows of a ~1024-row slab per
// thread halve the local update of each pivot step), 256 for FP64 (its
// candidate rows need the registers).
template <typename T>
__host__ __device__ constexpr int panel_threads() {
  return sizeof(T) == 4 ? 512 : 256;
}

__device__ __forceinline__ void st_release_s32(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_acquire_s32(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_relaxed_s32(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
// Spin (relaxed loads, bounded) until *flag == epoch, then one acquire
// fence orders the caller's later loads after the flag.  Returns false on a
// timeout or another CTA's error (recorded in st).
__device__ __forceinline__ bool wait_epoch(const int* flag, int epoch, DevStatus* st, int where) {
  bool ok = true;
  if (ld_relaxed_s32(flag) != epoch) {
    const unsigned long long t0 = globaltimer_ns();
    while (ld_relaxed_s32(flag) != epoch) {
      if (*(volatile int*)&st->err != 0 || globaltimer_ns() - t0 > kSpinLimitNs) {
        atomicCAS(&st->err, 0, (int)kErrBarrierTimeout);
        st->err_where = where;
        ok = false;
        break;
      }
    }
  }
  asm volatile("fence.acq_rel.gpu;" ::: "memory");
  return ok;
}

// Shared-memory slab of a CTA's panel rows: column c of local row r at
// slab[c * S + r], S = slab_stride(R) (R rounded up so that every column
// can start on the 16-byte phase of its rows in global memory), and slab =
// the 16-byte aligned shared base + mis, mis being the CTA's first row's
// offset from a 16-byte boundary in elements.  The slab takes
// slab_elems(R) elements from that base.
template <typename T>
__host__ __device__ constexpr int slab_stride(int R) {
  return (R + 2 * (16 / (int)sizeof(T)) - 2) / (16 / (int)sizeof(T)) * (16 / (int)sizeof(T));
}
template <typename T>
__host__ __device__ constexpr size_t slab_elems(int R) {
  return (size_t)slab_stride<T>(R) * kPanelW + 16 / sizeof(T);
}

// Stages the CTA's rows [rb, rb + nr) of the panel's w columns in the slab
// with the TMA engine: per column one bulk copy (cp.async.bulk) of the
// 16-byte aligned middle of its rows, completing on an mbarrier, and the
// at most 2 x (16 / sizeof(T) - 1) rows at either end by plain loads.  When
// a column's stride is not a multiple of 16 bytes, every entry goes by
// cp.async instead.  Returns the slab (shared base + mis).  A bounded wait:
// a timeout records an error and the kernel carries on (it must still meet
// every barrier of the other CTAs); the host then reports the failure.
template <typename T>
__device__ __forceinline__ T* panel_load_slab(unsigned char* smem, const T* A, long lda, int rb,
                                              int nr, int R, int w, uint64_t* mbar,
                                              DevStatus* st) {
  constexpr int E = 16 / (int)sizeof(T);
  const int S = slab_stride<T>(R);
  const T* src0 = A + rb;
  const int mis = (int)(((uintptr_t)src0 & 15u) / sizeof(T));
  T* slab = reinterpret_cast<T*>(smem) + mis;
  if (((size_t)lda * sizeof(T)) % 16 != 0) {
    for (int c = 0; c < w; ++c)
      for (int r = threadIdx.x; r < nr; r += blockDim.x)
        asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(
                         (unsigned)__cvta_generic_to_shared(slab + c * S + r)),
                     "l"(src0 + (long)r + (long)c * lda), "n"((int)sizeof(T))
                     : "memory");
    asm volatile("cp.async.wait_all;" ::: "memory");
    return slab;
  }
  const int h = (E - mis) % E;                      // rows before the first aligned one
  const int mid = nr > h ? (nr - h) / E * E : 0;    // rows in whole 16-byte units
  const uint32_t bytes = (uint32_t)(mid * sizeof(T));
  if (mid > 0) {
    if (threadIdx.x == 0) {
      tc::mbar_init(mbar, 1);
      tc::fence_mbar_init();
      tc::mbar_arrive_expect_tx(mbar, bytes * (uint32_t)w);
    }
    __syncthreads();
    if (threadIdx.x < w) {
      const int c = threadIdx.x;
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
          "[%3];" ::"r"((unsigned)__cvta_generic_to_shared(slab + c * S + h)),
          "l"(src0 + h + (long)c * lda), "r"(bytes), "r"(tc::smem_u32(mbar))
          : "memory");
    }
  }
  // the ends of each column
  const int tail0 = h + mid, ntail = nr - tail0;
  for (int idx = threadIdx.x; idx < w * E * 2; idx += blockDim.x) {
    const int c = idx / (2 * E), k = idx % (2 * E);
    const int r = k < E ? k : tail0 + (k - E);
    const bool in = k < E ? (r < min(h, nr)) : (k - E < ntail);
    if (in) slab[c * S + r] = src0[(long)r + (long)c * lda];
  }
  if (mid > 0 && !tc::mbar_wait(mbar, 0, st, 40)) {
    // the copies may still land: wait for them once more before going on
    tc::mbar_wait(mbar, 0, st, 41);
  }
  return slab;
}

// Step j of lu::Panel in two halves, so that the exchange of column j+1's
// pivot runs while most of step j's rank-1 update is still to do:
//   front: the multipliers of column j (scaled by the pivot's reciprocal,
//          Panel.hpp:53-55), the pivot row's old position pl in full (it
//          takes old row j from s_d), column j+1 of the other rows, and this
//          CTA's candidate for column j+1;
//   back:  columns j+2 .. w-1 of the other rows.
// Until the back half has run, pending_value() gives a row's entries as the
// whole step leaves them: every entry sees the same fma with the same
// operands as in one pass, so results are bit-identical.
template <typename T>
__device__ __forceinline__ void panel_step_front(T* slab, int S, int nr, int r0, int j, int w,
                                                 int pl, const T* s_d, const T* urow,
                                                 bool singular, T inv, int rb, T& bv,
                                                 int& br) {
  for (int r = r0 + threadIdx.x; r < nr; r += blockDim.x) {
    const bool pr = r == pl;
    T l = pr ? s_d[j] : slab[j * S + r];
    if (!singular) l *= inv;
    slab[j * S + r] = l;
    if (pr) {
      for (int c = j + 1; c < w; ++c) slab[c * S + r] = fma(-l, urow[c], s_d[c]);
    } else if (j + 1 < w) {
      slab[(j + 1) * S + r] = fma(-l, urow[j + 1], slab[(j + 1) * S + r]);
    }
    if (j + 1 < w) {
      const T v = absv(slab[(j + 1) * S + r]);
      if (argmax_better(v, rb + r, bv, br)) {
        bv = v;
        br = rb + r;
      }
    }
  }
}

template <typename T>
__device__ __forceinline__ void panel_step_back(T* slab, int S, int nr, int r0, int j, int w,
                                                int pl, const T* urow) {
  if (j + 2 >= w) return;
  for (int r = r0 + threadIdx.x; r < nr; r += blockDim.x) {
    if (r == pl) continue;
    const T l = slab[j * S + r];
    T* row = slab + r;
    int c = j + 2;
    for (; c + 7 < w; c += 8) {  // eight loads in flight, then eight fmas / stores
      T v[8];
#pragma unroll
      for (int e = 0; e < 8; ++e) v[e] = row[(c + e) * S];
#pragma unroll
      for (int e = 0; e < 8; ++e) v[e] = fma(-l, urow[c + e], v[e]);
#pragma unroll
      for (int e = 0; e < 8; ++e) row[(c + e) * S] = v[e];
    }
    for (; c + 3 < w; c += 4) {
      T v0 = row[c * S], v1 = row[(c + 1) * S], v2 = row[(c + 2) * S], v3 = row[(c + 3) * S];
      v0 = fma(-l, urow[c], v0);
      v1 = fma(-l, urow[c + 1], v1);
      v2 = fma(-l, urow[c + 2], v2);
      v3 = fma(-l, urow[c + 3], v3);
      row[c * S] = v0;
      row[(c + 1) * S] = v1;
      row[(c + 2) * S] = v2;
      row[(c + 3) * S] = v3;
    }
    for (; c < w; ++c) row[c * S] = fma(-l, urow[c], row[c * S]);
  }
}

// Entry (r, c) of the slab (local row r) as step pj leaves it, before
// panel_step_back(pj) has run (pj < 0: no step pending).  Only rows the step
// updates (global row > pj) are asked for.
template <typename T>
__device__ __forceinline__ T pending_value(const T* slab, int S, int r, int c, int pj, int plp,
                                           const T* urowp) {
  T v = slab[c * S + r];
  if (pj >= 0 && c >= pj + 2 && r != plp) v = fma(-slab[pj * S + r], urowp[c], v);
  return v;
}

template <typename T, int W>
__global__ void __launch_bounds__(panel_threads<T>())
getf2_panel_kernel(PanelParams<T> p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t s_mbar;
  __shared__ T s_d[W];
  __shared__ T s_rv[33];
  __shared__ int s_rr[33];
  __shared__ T s_gv[panel_threads<T>()];
  __shared__ int s_gr[panel_threads<T>()];
  T* s_rows = reinterpret_cast<T*>(smem_raw) + slab_elems<T>(p.R);  // [G][W] candidate rows
  __shared__ int s_abort;

  const int G = gridDim.x, b = blockIdx.x, tid = threadIdx.x;
  const int lane = tid & 31;
  const int R = p.R, w = p.w, maxG = p.s.maxG;
  const int S = slab_stride<T>(R);
  const int rb = b * R;
  const int re = min(rb + R, p.mp);
  const int nr = max(re - rb, 0);

  T* slab = panel_load_slab(smem_raw, p.A, p.lda, rb, nr, R, w, &s_mbar, p.st);
  if (tid == 0) s_abort = 0;
  __syncthreads();

  T bv = T(-1);
  int br = -1;
  for (int r = tid; r < nr; r += blockDim.x) {
    const T v = absv(slab[r]);
    if (argmax_better(v, rb + r, bv, br)) {
      bv = v;
      br = rb + r;
    }
  }
  block_argmax(bv, br, s_rv, s_rr);

  // the step whose back half is still to run (pj < 0: none)
  int pj = -1, plp = -1, r0p = 0;
  const T* urowp = nullptr;
  for (int j = 0; j < w; ++j) {
    if (p.nopiv) {  // the only candidate is row j (lu::Unb, LU/Local.hpp:42-61)
      br = (j >= rb && j < re) ? j : -1;
      bv = br >= 0 ? T(1) : T(-1);
    }
    const int epoch = p.epoch_base + j + 1;
    const int par = epoch & 1;
    PanelSlot<T>* my = p.s.slots + (long)par * maxG + b;
    unsigned long long* tr = (p.s.trace && b == 0 && tid == 0) ? p.s.trace + 4 * (long)j : nullptr;
    if (tr) tr[0] = globaltimer_ns();
    // 1. publish (the release store orders the CTA's slot writes, which
    // the barrier makes visible to the publishing thread); the rows carry
    // the pending step's update
    if (br >= 0 && tid < w) my->cand[tid] = pending_value(slab, S, br - rb, tid, pj, plp, urowp);
    if (j >= rb && j < re && tid < w)
      my->diag[tid] = pending_value(slab, S, j - rb, tid, pj, plp, urowp);
    if (tid == 0) {
      my->val = bv;
      my->row = br;
    }
    __syncthreads();
    if (tid == 0) st_release_s32(&my->epoch, epoch);
    // the rest of the previous step's update while the other CTAs publish
    if (pj >= 0) panel_step_back<T>(slab, S, nr, r0p, pj, w, plp, urowp);
    __syncthreads();  // urowp (s_rows / s_d) is read before the exchange refills them
    if (tr) tr[1] = globaltimer_ns();
    // 2. the barrier: every slot carries this epoch.  The thread that polled
    // slot g copies g's candidate row (and, for the owner of row j, row j)
    // right away, so the winner's row is already on chip after the barrier.
    if (tid < G) {
      const PanelSlot<T>* sl = p.s.slots + (long)par * maxG + tid;
      if (!wait_epoch(&sl->epoch, epoch, p.st, 1)) s_abort = 1;
      // all loads of the slot issued together (one round trip)
      const int gr = __ldcg(&sl->row);
      const T gv = __ldcg(&sl->val);
      const bool own = tid == j / R;
      T cr[W], dr[W];
#pragma unroll
      for (int c = 0; c < W; ++c) {
        cr[c] = c < w ? __ldcg(&sl->cand[c]) : T(0);
        dr[c] = (own && c < w) ? __ldcg(&sl->diag[c]) : T(0);
      }
      s_gv[tid] = gv;
      s_gr[tid] = gr;
#pragma unroll
      for (int c = 0; c < W; ++c) s_rows[tid * W + c] = cr[c];
      if (own)
#pragma unroll
        for (int c = 0; c < W; ++c) s_d[c] = dr[c];
    }
    __syncthreads();
    if (s_abort) return;
    if (tr) tr[2] = globaltimer_ns();
    // 3. reduce (every warp, identical result)
    int piv;
    {
      T v = T(-1);
      int r = -1;
      for (int g = lane; g < G; g += 32) {
        if (argmax_better(s_gv[g], s_gr[g], v, r)) {
          v = s_gv[g];
          r = s_gr[g];
        }
      }
      warp_argmax(v, r);
      piv = (r < 0) ? j : r;
    }
    const T* urow = (piv == j) ? s_d : s_rows + (piv / R) * W;  // the pivot row
    if (b == 0 && tid == 0) p.ipiv[j] = p.row_base + piv;
    const T alpha = urow[j];
    const bool singular = (alpha == T(0));
    if (singular && b == 0 && tid == 0) atomicCAS(&p.st->info, 0, p.info_base + j + 1);
    const T inv = singular ? T(1) : T(1) / alpha;
    // 4. row j takes the pivot row (row j is not updated below); the pivot
    // row's position takes old row j, updated from s_d
    if (piv != j && tid < w && j >= rb && j < re) slab[tid * S + (j - rb)] = urow[tid];
    bv = T(-1);
    br = -1;
    const int r0 = max(j + 1 - rb, 0);
    const int pl = (piv != j && piv >= rb && piv < re) ? piv - rb : -1;
    // the pivot row's position: old row j's multipliers of the earlier
    // columns move with it (columns j.. come from the update below)
    if (pl >= 0 && tid < j) slab[tid * S + pl] = s_d[tid];
    panel_step_front<T>(slab, S, nr, r0, j, w, pl, s_d, urow, singular, inv, rb, bv, br);
    block_argmax_nolead(bv, br, s_rv, s_rr);
    if (tr) tr[3] = globaltimer_ns();
    pj = j;
    plp = pl;
    r0p = r0;
    urowp = urow;
  }
  __syncthreads();
  for (int c = 0; c < w; ++c)
    for (int r = tid; r < nr; r += blockDim.x)
      p.A[(long)(rb + r) + (long)c * p.lda] = slab[c * S + r];
}

// ---------------------------------------------------------------------------
// FP32 panel with the rows in registers.  512 threads per CTA, thread t owns
// panel rows rb + t and rb + t + 512 with all w values in registers, so the
// rank-1 update of a column is register FMAs (no shared-memory traffic) and
// the per-column time is the exchange.  The exchange, slots, epochs, pivot
// choice and arithmetic order are those of getf2_panel_kernel: same pivots,
// same results.
constexpr int kRegThreads = 512, kRegRows = 2;

template <int W>
__global__ void __launch_bounds__(kRegThreads, 1)
getf2_panel_reg_kernel(PanelParams<float> p) {
  __shared__ float s_d[W];
  __shared__ float s_rv[33];
  __shared__ int s_rr[33];
  __shared__ float s_gv[kRegThreads];
  __shared__ int s_gr[kRegThreads];
  __shared__ float s_rows[kRegThreads / 2][W];  // candidate rows of up to 256 CTAs
  __shared__ int s_abort;

  const int G = gridDim.x, b = blockIdx.x, tid = threadIdx.x;
  const int lane = tid & 31;
  const int R = p.R, w = p.w, maxG = p.s.maxG;
  const int rb = b * R;
  const int re = min(rb + R, p.mp);
  const int nr = max(re - rb, 0);

  float a[kRegRows][W];
  int lr[kRegRows];  // local rows (or -1)
#pragma unroll
  for (int i = 0; i < kRegRows; ++i) {
    const int r = tid + i * kRegThreads;
    lr[i] = r < nr ? r : -1;
#pragma unroll
    for (int c = 0; c < W; ++c)
      a[i][c] = (lr[i] >= 0 && c < w) ? p.A[(long)(rb + r) + (long)c * p.lda] : 0.f;
  }
  if (tid == 0) s_abort = 0;

  auto col = [&](int i, int j) {  // a[i][j] for a run-time j
    float v = 0.f;
#pragma unroll
    for (int c = 0; c < W; ++c)
      if (c == j) v = a[i][c];
    return v;
  };

  float bv = -1.f;
  int br = -1;
#pragma unroll
  for (int i = 0; i < kRegRows; ++i)
    if (lr[i] >= 0) {
      const float v = fabsf(a[i][0]);
      if (argmax_better(v, rb + lr[i], bv, br)) {
        bv = v;
        br = rb + lr[i];
      }
    }
  block_argmax(bv, br, s_rv, s_rr);

  for (int j = 0; j < w; ++j) {
    const int epoch = p.epoch_base + j + 1;
    const int par = epoch & 1;
    PanelSlot<float>* my = p.s.slots + (long)par * maxG + b;
    // 1. publish: the owners of the candidate row and of row j write them
#pragma unroll
    for (int i = 0; i < kRegRows; ++i) {
      if (lr[i] >= 0 && rb + lr[i] == br)
#pragma unroll
        for (int c = 0; c < W; ++c)
          if (c < w) my->cand[c] = a[i][c];
      if (lr[i] >= 0 && rb + lr[i] == j)
#pragma unroll
        for (int c = 0; c < W; ++c)
          if (c < w) my->diag[c] = a[i][c];
    }
    if (tid == 0) {
      my->val = bv;
      my->row = br;
    }
    __syncthreads();
    if (tid == 0) st_release_s32(&my->epoch, epoch);
    // 2. the barrier and the candidates (as getf2_panel_kernel)
    if (tid < G) {
      const PanelSlot<float>* sl = p.s.slots + (long)par * maxG + tid;
      if (!wait_epoch(&sl->epoch, epoch, p.st, 3)) s_abort = 1;
      const int gr = __ldcg(&sl->row);
      const float gv = __ldcg(&sl->val);
      const bool own = tid == j / R;
      float cr[W], dr[W];
#pragma unroll
      for (int c = 0; c < W; ++c) {
        cr[c] = c < w ? __ldcg(&sl->cand[c]) : 0.f;
        dr[c] = (own && c < w) ? __ldcg(&sl->diag[c]) : 0.f;
      }
      s_gv[tid] = gv;
      s_gr[tid] = gr;
#pragma unroll
      for (int c = 0; c < W; ++c) s_rows[tid][c] = cr[c];
      if (own)
#pragma unroll
        for (int c = 0; c < W; ++c) s_d[c] = dr[c];
    }
    __syncthreads();
    if (s_abort) break;  // uniform: read after the barrier
    // 3. reduce (every warp)
    int piv;
    {
      float v = -1.f;
      int r = -1;
      for (int g = lane; g < G; g += 32)
        if (argmax_better(s_gv[g], s_gr[g], v, r)) {
          v = s_gv[g];
          r = s_gr[g];
        }
      warp_argmax(v, r);
      piv = (r < 0) ? j : r;
    }
    const float* urow = (piv == j) ? s_d : s_rows[piv / R];
    if (b == 0 && tid == 0) p.ipiv[j] = p.row_base + piv;
    const float alpha = urow[j];
    const bool singular = (alpha == 0.f);
    if (singular && b == 0 && tid == 0) atomicCAS(&p.st->info, 0, p.info_base + j + 1);
    const float inv = singular ? 1.f : 1.f / alpha;
    // 4. interchange: row j takes the pivot row, the pivot row's position
    // takes old row j; then the update of the rows after j
    bv = -1.f;
    br = -1;
#pragma unroll
    for (int i = 0; i < kRegRows; ++i) {
      if (lr[i] < 0) continue;
      const int row = rb + lr[i];
      if (piv != j && row == j) {
#pragma unroll
        for (int c = 0; c < W; ++c) a[i][c] = urow[c];
        continue;  // row j is not updated
      }
      if (piv != j && row == piv)
#pragma unroll
        for (int c = 0; c < W; ++c) a[i][c] = s_d[c];
      if (row <= j) continue;
      float l = col(i, j);
      if (!singular) l *= inv;
#pragma unroll
      for (int c = 0; c < W; ++c) {
        if (c == j) a[i][c] = l;
        if (c > j && c < w) a[i][c] = fmaf(-l, urow[c], a[i][c]);
      }
      if (j + 1 < w) {
        const float v = fabsf(col(i, j + 1));
        if (argmax_better(v, row, bv, br)) {
          bv = v;
          br = row;
        }
      }
    }
    block_argmax_nolead(bv, br, s_rv, s_rr);
  }
#pragma unroll
  for (int i = 0; i < kRegRows; ++i)
    if (lr[i] >= 0)
#pragma unroll
      for (int c = 0; c < W; ++c)
        if (c < w) p.A[(long)(rb + lr[i]) + (long)c * p.lda] = a[i][c];
}

// ---------------------------------------------------------------------------
// The same panel on one thread-block cluster: the per-column exchange goes
// through distributed shared memory and the cluster's hardware barrier
// instead of global-memory slots and polling.  CTA b of the cluster keeps
// rows [b R, b R + R) in its shared memory as above; per column j it writes
// its candidate (|a|, row, the row's w values, and row j if it owns it) to
// its own shared slot, all threads arrive at the cluster barrier (release /
// acquire), and thread g < C reads CTA g's slot with ld.shared::cluster.
// Slots are double-buffered by column parity: a CTA rewrites a slot only
// after the next column's barrier, which every CTA reaches after its reads.
// Same arithmetic, in the same order, as getf2_panel_kernel.
template <typename T>
struct ClusterSlot {
  T val;
  int row;
  T cand[kPanelW];
  T diag[kPanelW];
};

// The .aligned cluster barriers must be executed by every thread of a warp
// together; the callers reach them right after thread-divergent stores, so
// each first reconverges its warp explicitly.
__device__ __forceinline__ void cluster_barrier() {
  __syncwarp();
  asm volatile("barrier.cluster.arrive.release.aligned;\n"
               "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_arrive() {
  __syncwarp();
  asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_wait() {
  __syncwarp();
  asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ uint32_t cluster_map(const void* local, unsigned rank) {
  uint32_t a = static_cast<uint32_t>(__cvta_generic_to_shared(local)), r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}

__device__ __forceinline__ float ld_cluster(uint32_t addr, float*) {
  float v;
  asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(addr) : "memory");
  return v;
}
__device__ __forceinline__ double ld_cluster(uint32_t addr, double*) {
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(addr) : "memory");
  return v;
}
__device__ __forceinline__ int ld_cluster_s32(uint32_t addr) {
  int v;
  asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(addr) : "memory");
  return v;
}

template <typename T, int W>
__global__ void __launch_bounds__(panel_threads<T>())
getf2_panel_cluster_kernel(PanelParams<T> p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t s_mbar;
  __shared__ ClusterSlot<T> slots[2];
  __shared__ T s_d[W];
  __shared__ T s_rv[33];
  __shared__ int s_rr[33];
  __shared__ T s_gv[32];
  __shared__ int s_gr[32];
  T* s_rows = reinterpret_cast<T*>(smem_raw) + slab_elems<T>(p.R);  // [C][W] candidate rows

  const int G = gridDim.x, b = blockIdx.x, tid = threadIdx.x;
  const int lane = tid & 31;
  const int R = p.R, w = p.w;
  const int S = slab_stride<T>(R);
  const int rb = b * R;
  const int re = min(rb + R, p.mp);
  const int nr = max(re - rb, 0);

  T* slab = panel_load_slab(smem_raw, p.A, p.lda, rb, nr, R, w, &s_mbar, p.st);
  __syncthreads();

  T bv = T(-1);
  int br = -1;
  for (int r = tid; r < nr; r += blockDim.x) {
    const T v = absv(slab[r]);
    if (argmax_better(v, rb + r, bv, br)) {
      bv = v;
      br = rb + r;
    }
  }
  block_argmax(bv, br, s_rv, s_rr);
  cluster_barrier();  // every CTA of the cluster is running

  int pj = -1, plp = -1, r0p = 0;  // the step whose back half is still to run
  const T* urowp = nullptr;
  for (int j = 0; j < w; ++j) {
    ClusterSlot<T>* my = &slots[j & 1];
    unsigned long long* tr = (p.s.trace && b == 0 && tid == 0) ? p.s.trace + 4 * (long)j : nullptr;
    if (tr) tr[0] = globaltimer_ns();
    // 1. publish in this CTA's shared memory (rows with the pending update)
    if (br >= 0 && tid < w) my->cand[tid] = pending_value(slab, S, br - rb, tid, pj, plp, urowp);
    if (j >= rb && j < re && tid < w)
      my->diag[tid] = pending_value(slab, S, j - rb, tid, pj, plp, urowp);
    if (tid == 0) {
      my->val = bv;
      my->row = br;
    }
    cluster_arrive();
    // the rest of the previous step's update while the cluster gathers
    if (pj >= 0) panel_step_back<T>(slab, S, nr, r0p, pj, w, plp, urowp);
    __syncthreads();  // urowp (s_rows / s_d) is read before the exchange refills them
    if (tr) tr[1] = globaltimer_ns();
    cluster_wait();
    // 2. thread g < C reads CTA g's slot
    if (tid < G) {
      const uint32_t base = cluster_map(my, (unsigned)tid);
      const uint32_t o_val = (uint32_t)offsetof(ClusterSlot<T>, val);
      const uint32_t o_row = (uint32_t)offsetof(ClusterSlot<T>, row);
      const uint32_t o_cand = (uint32_t)offsetof(ClusterSlot<T>, cand);
      const uint32_t o_diag = (uint32_t)offsetof(ClusterSlot<T>, diag);
      const bool own = tid == j / R;
      T cr[W], dr[W];
      const T gv = ld_cluster(base + o_val, (T*)nullptr);
      const int gr = ld_cluster_s32(base + o_row);
#pragma unroll
      for (int c = 0; c < W; ++c) {
        cr[c] = c < w ? ld_cluster(base + o_cand + c * (uint32_t)sizeof(T), (T*)nullptr) : T(0);
        dr[c] = (own && c < w) ? ld_cluster(base + o_diag + c * (uint32_t)sizeof(T), (T*)nullptr)
                               : T(0);
      }
      s_gv[tid] = gv;
      s_gr[tid] = gr;
#pragma unroll
      for (int c = 0; c < W; ++c) s_rows[tid * W + c] = cr[c];
      if (own)
#pragma unroll
        for (int c = 0; c < W; ++c) s_d[c] = dr[c];
    }
    __syncthreads();
    if (tr) tr[2] = globaltimer_ns();
    // 3. reduce (every warp, identical result)
    int piv;
    {
      T v = T(-1);
      int r = -1;
      if (lane < G && argmax_better(s_gv[lane], s_gr[lane], v, r)) {
        v = s_gv[lane];
        r = s_gr[lane];
      }
      warp_argmax(v, r);
      piv = (r < 0) ? j : r;
    }
    const T* urow = (piv == j) ? s_d : s_rows + (piv / R) * W;
    if (b == 0 && tid == 0) p.ipiv[j] = p.row_base + piv;
    const T alpha = urow[j];
    const bool singular = (alpha == T(0));
    if (singular && b == 0 && tid == 0) atomicCAS(&p.st->info, 0, p.info_base + j + 1);
    const T inv = singular ? T(1) : T(1) / alpha;
    // 4. swap, the front of the update, next candidate (as getf2_panel_kernel)
    if (piv != j && tid < w && j >= rb && j < re) slab[tid * S + (j - rb)] = urow[tid];
    bv = T(-1);
    br = -1;
    const int r0 = max(j + 1 - rb, 0);
    const int pl = (piv != j && piv >= rb && piv < re) ? piv - rb : -1;
    if (pl >= 0 && tid < j) slab[tid * S + pl] = s_d[tid];
    panel_step_front<T>(slab, S, nr, r0, j, w, pl, s_d, urow, singular, inv, rb, bv, br);
    block_argmax_nolead(bv, br, s_rv, s_rr);
    if (tr) tr[3] = globaltimer_ns();
    pj = j;
    plp = pl;
    r0p = r0;
    urowp = urow;
  }
  __syncthreads();
  for (int c = 0; c < w; ++c)
    for (int r = tid; r < nr; r += blockDim.x)
      p.A[(long)(rb + r) + (long)c * p.lda] = slab[c * S + r];
  cluster_barrier();  // no CTA leaves while another may still read its slots
}

// The cluster panel with the rows in registers (FP32).  512 threads; thread
// t holds local rows t, t + 512, ... (RPT of them) of its CTA's R <= 512 RPT
// rows, all W values of each in registers (W x RPT <= 64: 32 columns and 2
// rows, or 16 columns and 4 rows for panels of up to 32768 rows on 16 CTAs),
// and the column loop is unrolled so every register index is fixed.  Per column: publish (candidate row and row j
// from registers into the CTA's own slot), the cluster barrier, thread
// g < C reads CTA g's slot, every warp picks the pivot, then the whole
// rank-1 update of the thread's two rows and the next column's candidate.
// No shared-memory traffic per entry, so a step is the exchange plus a few
// dozen register FMAs.  Same slots, exchange, pivot choice and arithmetic
// (l = a_j * (1 / pivot), a_c = fma(-l, u_c, a_c)) as the kernels above:
// same pivots, same factors.
constexpr int kRcThreads = 512;

// The register kernel's slot: 16-byte aligned rows, read with vector
// distributed-shared-memory loads.
struct __align__(16) RcSlot {
  float cand[kPanelW];
  float diag[kPanelW];
  float val;
  int row;
};

__device__ __forceinline__ float4 ld_cluster_v4(uint32_t addr) {
  float4 v;
  asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "r"(addr));
  return v;
}
__device__ __forceinline__ void ld_cluster_head(uint32_t addr, float& v, int& r) {
  asm volatile("ld.shared::cluster.v2.b32 {%0, %1}, [%2];" : "=f"(v), "=r"(r) : "r"(addr));
}

// Push exchange: every CTA sends its candidate (and the owner of row j that
// row) into every CTA's receive buffer with asynchronous distributed-shared-
// memory stores that complete on the receiver's mbarrier, so a step waits
// for its data once (no cluster barrier, no remote read round trip).
struct __align__(16) PushSlot {
  float cand[kPanelW];
  float val;
  int row;
  int pad[2];
};

__device__ __forceinline__ void st_async_v4(uint32_t addr, float x, float y, float z, float w,
                                            uint32_t bar) {
  asm volatile(
      "st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.f32 [%0], {%1, %2, %3, %4}, "
      "[%5];" ::"r"(addr),
      "f"(x), "f"(y), "f"(z), "f"(w), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void st_async_head(uint32_t addr, float v, int r, uint32_t bar) {
  asm volatile(
      "st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.b32 [%0], {%1, %2}, [%3];" ::"r"(
          addr),
      "r"(__float_as_uint(v)), "r"(r), "r"(bar)
      : "memory");
}
// test_wait does not suspend the thread: the waiting warps leave the moment
// the phase completes (a suspended try_wait was seen to wake late)
__device__ __forceinline__ bool mbar_try_wait_cluster(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "mbarrier.test_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Sends W values (a row held in registers) to slot `slot_off` of every CTA's
// buffer at `buf` (same layout in every CTA), completing on each CTA's `bar`.
template <int W>
__device__ __forceinline__ void push_row(const float (&v)[W], const void* buf, uint32_t slot_off,
                                         const uint64_t* bar, int G) {
  for (int d = 0; d < G; ++d) {
    const uint32_t dst = cluster_map(buf, (unsigned)d) + slot_off;
    const uint32_t rb = cluster_map(bar, (unsigned)d);
#pragma unroll
    for (int c = 0; c < W; c += 4) st_async_v4(dst + 4u * c, v[c], v[c + 1], v[c + 2], v[c + 3], rb);
  }
}

template <int W, int RPT, bool PUSH>
__global__ void __launch_bounds__(kRcThreads, 1)
getf2_panel_cluster_reg_kernel(PanelParams<float> p) {
  static_assert(W <= kPanelW && W % 4 == 0 && W * RPT <= 64, "slot layout, registers");
  __shared__ RcSlot slots[2];
  // PUSH: receive buffers (slot g = CTA g's candidate), row j, their mbarriers
  __shared__ PushSlot s_in[PUSH ? 2 : 1][PUSH ? 16 : 1];
  __shared__ __align__(16) float s_din[PUSH ? 2 : 1][W];
  __shared__ __align__(16) float s_stage[PUSH ? 2 : 1][2][W];  // rows being sent
  __shared__ __align__(8) uint64_t s_mbar[2];
  __shared__ __align__(16) float s_d[W];
  __shared__ __align__(16) float s_rows[16][W];
  __shared__ float s_gv[32];
  __shared__ int s_gr[32];
  // per-step CTA argmax buffers, alternating by column: with the push
  // exchange nothing else keeps a fast warp from the next column's writes
  // while a slow one still reads
  __shared__ float s_rv[2][33];
  __shared__ int s_rr[2][33];
  __shared__ int s_piv[W];                     // the pivot of each column (panel row)
  __shared__ __align__(16) float s_u[W][W];    // sib_w: the node's U12 (w x sib_w)
  __shared__ int s_dst[2 * W], s_src[2 * W];   // the interchanges' net row moves
  __shared__ int s_nmove;

  pdl_wait();  // (launched as the side stream's programmatic dependent)
  const int G = gridDim.x, b = blockIdx.x, tid = threadIdx.x;
  const int lane = tid & 31;
  const int R = p.R, w = p.w;
  const int rb = b * R;
  const int re = min(rb + R, p.mp);
  const int nr = max(re - rb, 0);

  float a[RPT][W];
  int grow[RPT];  // global panel row of each register row, -1 past the CTA's rows
#pragma unroll
  for (int i = 0; i < RPT; ++i) {
    const int r = tid + i * kRcThreads;
    grow[i] = r < nr ? rb + r : -1;
#pragma unroll
    for (int c = 0; c < W; ++c)
      a[i][c] = (grow[i] >= 0 && c < w) ? p.A[(long)grow[i] + (long)c * p.lda] : 0.f;
  }

  float bv = -1.f;
  int br = -1;
#pragma unroll
  for (int i = 0; i < RPT; ++i)
    if (grow[i] >= 0) {
      const float v = fabsf(a[i][0]);
      if (argmax_better(v, grow[i], bv, br)) {
        bv = v;
        br = grow[i];
      }
    }
  if (PUSH && tid == 0) {
    tc::mbar_init(&s_mbar[0], 1);
    tc::mbar_init(&s_mbar[1], 1);
    tc::fence_mbar_init();
  }
  block_argmax(bv, br, s_rv[0], s_rr[0]);
  cluster_barrier();  // every CTA of the cluster is running (and its mbarriers set)
  bool dead = false;  // PUSH: a wait timed out (recorded); later waits are skipped
  (void)dead;

#pragma unroll
  for (int j = 0; j < W; ++j) {
    if (j < w) {
      RcSlot* my = &slots[j & 1];
      const int bb = j & 1;
      (void)bb;
      unsigned long long* tr =
          (p.s.trace && b == 0 && tid == 0) ? p.s.trace + 4 * (long)j : nullptr;
      if (tr) tr[0] = globaltimer_ns();
      if constexpr (PUSH) {
        // 1. every CTA's candidate (zeros with an empty head if it has none)
        // and row j go straight into every CTA's buffer bb: the owner stages
        // its row in shared memory, then lane d of its warp sends it to CTA d
        if (tid == 0)
          tc::mbar_arrive_expect_tx(&s_mbar[bb], (uint32_t)(G * (8 + 4 * W) + 4 * W));
#pragma unroll
        for (int i = 0; i < RPT; ++i) {
          if (grow[i] >= 0 && grow[i] == br)
#pragma unroll
            for (int c = 0; c < W; ++c) s_stage[bb][0][c] = a[i][c];
          if (grow[i] == j)
#pragma unroll
            for (int c = 0; c < W; ++c) s_stage[bb][1][c] = a[i][c];
        }
        if (br < 0 && tid == 0)
#pragma unroll
          for (int c = 0; c < W; ++c) s_stage[bb][0][c] = 0.f;
        __syncwarp();
        const int warp = tid >> 5;
        const int cand_warp = br >= 0 ? ((br - rb) & (kRcThreads - 1)) >> 5 : 0;
        const int diag_warp = (j >= rb && j < re) ? ((j - rb) & (kRcThreads - 1)) >> 5 : -1;
        if (lane < G && (warp == cand_warp || warp == diag_warp)) {
          const uint32_t rbar = cluster_map(&s_mbar[bb], (unsigned)lane);
          if (warp == cand_warp) {
            const uint32_t dst =
                cluster_map(&s_in[bb][0], (unsigned)lane) + (uint32_t)(b * sizeof(PushSlot));
#pragma unroll
            for (int c = 0; c < W; c += 4) {
              const float4 v = *reinterpret_cast<const float4*>(&s_stage[bb][0][c]);
              st_async_v4(dst + 4u * c, v.x, v.y, v.z, v.w, rbar);
            }
            st_async_head(dst + (uint32_t)offsetof(PushSlot, val), bv, br, rbar);
          }
          if (warp == diag_warp) {
            const uint32_t dst = cluster_map(&s_din[bb][0], (unsigned)lane);
#pragma unroll
            for (int c = 0; c < W; c += 4) {
              const float4 v = *reinterpret_cast<const float4*>(&s_stage[bb][1][c]);
              st_async_v4(dst + 4u * c, v.x, v.y, v.z, v.w, rbar);
            }
          }
        }
        if (tr) tr[1] = globaltimer_ns();
        // 2. this step's buffer is complete (bounded wait)
        const uint32_t mb = tc::smem_u32(&s_mbar[bb]), par = (uint32_t)((j >> 1) & 1);
        if (!dead && !mbar_try_wait_cluster(mb, par)) {
          const unsigned long long t0 = globaltimer_ns();
          while (!mbar_try_wait_cluster(mb, par)) {
            if (globaltimer_ns() - t0 > kSpinLimitNs) {
              atomicCAS(&p.st->err, 0, (int)kErrMbarTimeout);
              p.st->err_where = 40;
              dead = true;
              break;
            }
          }
        }
        if (tr) tr[2] = globaltimer_ns();
      } else {
        // 1. publish from the registers of the rows' owners
  #pragma unroll
        for (int i = 0; i < RPT; ++i) {
          if (grow[i] >= 0 && grow[i] == br)
  #pragma unroll
            for (int c = 0; c < W; ++c) my->cand[c] = a[i][c];
          if (grow[i] == j)
  #pragma unroll
            for (int c = 0; c < W; ++c) my->diag[c] = a[i][c];
        }
        if (tid == 0) {
          my->val = bv;
          my->row = br;
        }
        cluster_arrive();
        if (tr) tr[1] = globaltimer_ns();
        cluster_wait();
        // 2. thread g < C reads CTA g's slot: head and candidate row in one
        // round trip, row j (its owner's slot only) in a second
        // (row j comes from its owner's slot through thread 32, in warp 1, at
        // the same time)
        if (tid < G || tid == 32) {
          const unsigned src = tid < G ? (unsigned)tid : (unsigned)(j / R);
          const uint32_t base = cluster_map(my, src);
          float4 cr[W / 4];
          if (tid < G) {
            float gv;
            int gr;
            ld_cluster_head(base + (uint32_t)offsetof(RcSlot, val), gv, gr);
  #pragma unroll
            for (int c = 0; c < W / 4; ++c)
              cr[c] = ld_cluster_v4(base + (uint32_t)offsetof(RcSlot, cand) + 16u * c);
            s_gv[tid] = gv;
            s_gr[tid] = gr;
  #pragma unroll
            for (int c = 0; c < W / 4; ++c) reinterpret_cast<float4*>(s_rows[tid])[c] = cr[c];
          } else {
  #pragma unroll
            for (int c = 0; c < W / 4; ++c)
              cr[c] = ld_cluster_v4(base + (uint32_t)offsetof(RcSlot, diag) + 16u * c);
  #pragma unroll
            for (int c = 0; c < W / 4; ++c) reinterpret_cast<float4*>(s_d)[c] = cr[c];
          }
        }
        __syncthreads();
        if (tr) tr[2] = globaltimer_ns();
      }
      // 3. the pivot (every warp, identical result)
      int piv;
      {
        float v = -1.f;
        int r = -1;
        const float hv = PUSH ? (lane < G ? s_in[bb & (PUSH ? 1 : 0)][lane & 15].val : -1.f)
                              : (lane < G ? s_gv[lane] : -1.f);
        const int hr = PUSH ? (lane < G ? s_in[bb & (PUSH ? 1 : 0)][lane & 15].row : -1)
                            : (lane < G ? s_gr[lane] : -1);
        if (lane < G && argmax_better(hv, hr, v, r)) {
          v = hv;
          r = hr;
        }
        warp_argmax(v, r);
        piv = (r < j || r >= p.mp) ? j : r;  // (r < 0: no candidate; else r >= j)
      }
      const float* drow = PUSH ? s_din[bb & (PUSH ? 1 : 0)] : s_d;
      const float* urow = (piv == j)
                              ? drow
                              : (PUSH ? s_in[bb & (PUSH ? 1 : 0)][(piv / R) & 15].cand
                                      : s_rows[piv / R]);
      // (the pivots go to global memory after the last column: a global store
      // here would hold up the release of thread 0's next cluster arrive)
      if (tid == 0) s_piv[j] = piv;
      const float alpha = urow[j];
      const bool singular = (alpha == 0.f);
      if (singular && b == 0 && tid == 0) atomicCAS(&p.st->info, 0, p.info_base + j + 1);
      const float inv = singular ? 1.f : 1.f / alpha;
      // 4. interchange, multipliers, rank-1 update, next candidate
      bv = -1.f;
      br = -1;
#pragma unroll
      for (int i = 0; i < RPT; ++i) {
        const int row = grow[i];
        if (row < 0) continue;
        if (piv != j && row == j) {  // row j takes the pivot row; not updated
#pragma unroll
          for (int c = 0; c < W; ++c) a[i][c] = urow[c];
          continue;
        }
        if (piv != j && row == piv)  // the pivot row's position takes old row j
#pragma unroll
          for (int c = 0; c < W; ++c) a[i][c] = drow[c];
        if (row <= j) continue;
        float l = a[i][j];
        if (!singular) l *= inv;
        a[i][j] = l;
#pragma unroll
        for (int c = j + 1; c < W; ++c) a[i][c] = fmaf(-l, urow[c], a[i][c]);
        if (j + 1 < w) {
          const float v = fabsf(a[i][j + 1 < W ? j + 1 : j]);
          if (argmax_better(v, row, bv, br)) {
            bv = v;
            br = row;
          }
        }
      }
      // every warp reduces the CTA's candidates itself (one barrier).  Its
      // buffers alternate by column; the exchange buffers of this column are
      // refilled only after every CTA has passed this barrier (cluster
      // barrier: each thread reads before it arrives, the gather writes
      // after the wait; push: the next-but-one column's data is sent only
      // after the sender has received this CTA's next column).
      block_argmax_nolead(bv, br, s_rv[bb], s_rr[bb]);
      if (tr) tr[3] = globaltimer_ns();
    }
  }
  if (b == 0 && tid < w) p.ipiv[tid] = p.row_base + s_piv[tid];
#pragma unroll
  for (int i = 0; i < RPT; ++i)
    if (grow[i] >= 0)
#pragma unroll
      for (int c = 0; c < W; ++c)
        if (c < w) p.A[(long)grow[i] + (long)c * p.lda] = a[i][c];
  // The leaf's interchanges (rows j and s_piv[j], j = 0 .. w-1, in order) on
  // the other columns of its block: their net row moves (at most 2w rows),
  // then each warp takes a few columns at a time and reads every moved row
  // of them before writing any.
  const int nleft = -p.swap_lo, nright = max(p.swap_hi - w, 0);
  if (nleft + nright > 0) {
    if (tid < 32) {
      // warp 0: slots 0 .. w-1 are rows 0 .. w-1; each distinct pivot row
      // >= w gets the next slot in the order of its first use
      const int pv = lane < w ? s_piv[lane] : lane;
      const bool ext = lane < w && pv >= w;
      const unsigned grp = __match_any_sync(0xffffffffu, ext ? pv : -1 - lane);
      const int leader = __ffs(grp) - 1;
      const unsigned firsts = __ballot_sync(0xffffffffu, ext && leader == lane);
      const int slot = ext ? w + __popc(firsts & ((1u << leader) - 1u)) : pv;
      const int nslot = w + __popc(firsts);
      if (ext && leader == lane) s_dst[slot] = pv;  // the row of each extra slot
      __syncwarp();
      const int key0 = lane < w ? lane : (lane < nslot ? s_dst[lane] : -1);
      const int key1 = lane + 32 < nslot ? s_dst[lane + 32] : -1;
      __syncwarp();
      // the swaps in order on the slots' contents (slot q: lane q & 31,
      // register q >> 5)
      int v0 = key0, v1 = key1;
#pragma unroll
      for (int j = 0; j < W; ++j) {
        if (j < w) {
          const int sj = __shfl_sync(0xffffffffu, slot, j);
          const int x = __shfl_sync(0xffffffffu, v0, j);
          const int y = __shfl_sync(0xffffffffu, sj < 32 ? v0 : v1, sj & 31);
          if (lane == j) v0 = y;
          if (sj < 32) {
            if (lane == sj) v0 = x;
          } else if (lane == sj - 32) {
            v1 = x;
          }
        }
      }
      const bool mv0 = lane < nslot && key0 != v0;
      const bool mv1 = lane + 32 < nslot && key1 != v1;
      const unsigned m0 = __ballot_sync(0xffffffffu, mv0);
      const unsigned m1 = __ballot_sync(0xffffffffu, mv1);
      const unsigned lt = (1u << lane) - 1u;
      if (mv0) {
        const int o = __popc(m0 & lt);
        s_dst[o] = key0;
        s_src[o] = v0;
      }
      if (mv1) {
        const int o = __popc(m0) + __popc(m1 & lt);
        s_dst[o] = key1;
        s_src[o] = v1;
      }
      if (lane == 0) s_nmove = __popc(m0) + __popc(m1);
    }
    __syncthreads();
    const int nmove = s_nmove;
    const int nw = kRcThreads / 32, warp = tid >> 5;
    const int d0 = lane < nmove ? s_dst[lane] : 0, s0 = lane < nmove ? s_src[lane] : 0;
    const int d1 = lane + 32 < nmove ? s_dst[lane + 32] : 0;
    const int s1 = lane + 32 < nmove ? s_src[lane + 32] : 0;
    constexpr int kCB = 4;  // columns a warp moves together
    const int ncol = nleft + nright, stride = G * nw;
    for (int q0 = b * nw + warp; q0 < ncol; q0 += kCB * stride) {
      float x0[kCB], x1[kCB];
#pragma unroll
      for (int u = 0; u < kCB; ++u) {
        const int q = q0 + u * stride;
        x0[u] = x1[u] = 0.f;
        if (q < ncol) {
          const int c = q < nleft ? p.swap_lo + q : w + (q - nleft);
          const float* col = p.A + (long)c * p.lda;
          if (lane < nmove) x0[u] = col[s0];
          if (lane + 32 < nmove) x1[u] = col[s1];
        }
      }
      __syncwarp();
#pragma unroll
      for (int u = 0; u < kCB; ++u) {
        const int q = q0 + u * stride;
        if (q < ncol) {
          const int c = q < nleft ? p.swap_lo + q : w + (q - nleft);
          float* col = p.A + (long)c * p.lda;
          if (lane < nmove) col[d0] = x0[u];
          if (lane + 32 < nmove) col[d1] = x1[u];
        }
      }
    }
  }
  cluster_barrier();  // no CTA leaves while another may still read its slots;
                      // every CTA's write-back and interchanges are visible
  if (p.sib_w > 0) {
    // The recursion node: U12 = L11^-1 A12 by warp 0 of CTA 0 (rows 0 .. w-1
    // are its threads' register rows 0), column by column of U12 in chunks
    // of 8 (each entry sees trsm_block's fma(-l_rc, u_c, u_r), c = 0 .. r-1);
    // then every CTA takes U12 and subtracts L21 U12 from its rows below w
    // (gemm_simt's sum from 0 over c, then one fma(-1, sum, a)).
    const int sw = p.sib_w;
    if (b == 0 && tid < 32) {
      const int r = tid;
#pragma unroll
      for (int c0 = 0; c0 < W; c0 += 8) {
        if (c0 < sw) {
          float u[8];
#pragma unroll
          for (int k = 0; k < 8; ++k)
            u[k] = (r < w && c0 + k < sw) ? p.A[(long)r + (long)(w + c0 + k) * p.lda] : 0.f;
#pragma unroll
          for (int c = 0; c < W; ++c) {
            if (c < w) {
              if (r == c)
#pragma unroll
                for (int k = 0; k < 8; ++k) s_u[c][c0 + k] = u[k];
              __syncwarp();
              if (r > c && r < w) {
                const float l = a[0][c];
#pragma unroll
                for (int k = 0; k < 8; ++k) u[k] = fmaf(-l, s_u[c][c0 + k], u[k]);
              }
            }
          }
          if (r < w)
#pragma unroll
            for (int k = 0; k < 8; ++k)
              if (c0 + k < sw) p.A[(long)r + (long)(w + c0 + k) * p.lda] = u[k];
        }
      }
    }
    cluster_barrier();  // CTA 0's U12 complete
    if (b != 0) {
      static_assert((W * W) % 4 == 0, "U12 in 16-byte pieces");
      const uint32_t src = cluster_map(&s_u[0][0], 0u);
      for (int v = tid; v < W * W / 4; v += kRcThreads)
        reinterpret_cast<float4*>(&s_u[0][0])[v] = ld_cluster_v4(src + 16u * v);
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < RPT; ++i) {
      const int row = grow[i];
      if (row < w) continue;  // (and rows past the CTA's)
#pragma unroll
      for (int c0 = 0; c0 < W; c0 += 8) {
        if (c0 < sw) {
          float acc[8];
#pragma unroll
          for (int k = 0; k < 8; ++k) acc[k] = 0.f;
#pragma unroll
          for (int c = 0; c < W; ++c)
            if (c < w)
#pragma unroll
              for (int k = 0; k < 8; ++k) acc[k] = fmaf(a[i][c], s_u[c][c0 + k], acc[k]);
#pragma unroll
          for (int k = 0; k < 8; ++k)
            if (c0 + k < sw) {
              float* pc = p.A + (long)row + (long)(w + c0 + k) * p.lda;
              *pc = fmaf(-1.f, acc[k], *pc);
            }
        }
      }
    }
    cluster_barrier();  // no CTA leaves while another may still read CTA 0's U12
  }
}

// Cluster size for a panel of mp rows: the power of two giving about
// g_panel_rows rows per CTA (at least 2 CTAs, at most max_cluster), or 0
// when one cluster cannot hold the panel in shared memory or the panel is
// too small for one (the caller then uses the cooperative kernel).
template <typename T>
static int cluster_ctas(int mp, int max_cluster) {
  constexpr int kMaxSmem = 200 * 1024;
  // the slab's row padding (slab_elems) comes out of the cap
  const int rows_cap = (int)(kMaxSmem / (kPanelW * sizeof(T))) - 32 - 16;
  if (mp < 128) return 0;
  int C = 2;
  while (C < max_cluster && (mp + C - 1) / C > g_panel_rows) C *= 2;
  if (C > max_cluster || (mp + C - 1) / C > rows_cap) return 0;
  return C;
}

template <typename T>
static cudaError_t launch_getf2_panel_cluster(T* A, long lda, int mp, int w, int* ipiv,
                                              int row_base, int info_base, DevStatus* st,
                                              int C, unsigned long long* trace,
                                              cudaStream_t stream) {
  const int R = ceil_div(mp, C);
  const size_t smem = (slab_elems<T>(R) + (size_t)C * kPanelW) * sizeof(T);
  auto kern = getf2_panel_cluster_kernel<T, kPanelW>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e == cudaSuccess && C > 8)
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(C);
  cfg.blockDim = dim3(panel_threads<T>());
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int nclusters = 0;
  e = cudaOccupancyMaxActiveClusters(&nclusters, (void*)kern, &cfg);
  if (e != cudaSuccess || nclusters < 1) {
    cudaGetLastError();
    return cudaErrorNotSupported;
  }
  PanelScratch<T> ps{};
  ps.trace = trace;
  PanelParams<T> prm{A, lda, mp, w, R, ipiv, row_base, info_base, 0, ps, st};
  return cudaLaunchKernelEx(&cfg, kern, prm);
}

// The register cluster kernel for an FP32 panel of mp rows on C CTAs
// (ceil(mp / C) <= 1024); cudaErrorNotSupported when the cluster cannot be
// placed.
static cudaError_t launch_getf2_panel_cluster_reg(float* A, long lda, int mp, int w, int* ipiv,
                                                  int row_base, int info_base, DevStatus* st,
                                                  int C, unsigned long long* trace,
                                                  cudaStream_t stream, int swap_lo, int swap_hi,
                                                  int sib_w) {
  const int R = ceil_div(mp, C);
  const bool narrow = w <= 16 && R > 2 * kRcThreads;  // 16 columns, 4 rows a thread
  if (R > (narrow ? 4 : 2) * kRcThreads) return cudaErrorNotSupported;
  const bool push = C <= 16 && (g_panel_push == 1 || (g_panel_push == 2 && !narrow));
  // at most one row a thread: the one-row instance (half the step code, which
  // is what the unrolled kernel waits on when fetching instructions)
  const bool single = !narrow && R <= kRcThreads && push;
  auto kern = narrow ? (push ? getf2_panel_cluster_reg_kernel<16, 4, true>
                             : getf2_panel_cluster_reg_kernel<16, 4, false>)
              : single ? getf2_panel_cluster_reg_kernel<kPanelW, 1, true>
                       : (push ? getf2_panel_cluster_reg_kernel<kPanelW, 2, true>
                               : getf2_panel_cluster_reg_kernel<kPanelW, 2, false>);
  cudaError_t e = cudaSuccess;
  if (C > 8) e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(C);
  cfg.blockDim = dim3(kRcThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = stream;
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  // whether a cluster of C fits, asked once per device, variant and C
  static signed char fits[64][5][17] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  signed char* f = (dev >= 0 && dev < 64 && C <= 16)
                       ? &fits[dev][single ? 4 : (narrow ? 2 : 0) + (push ? 1 : 0)][C]
                       : nullptr;
  bool ok = f && *f > 0;
  if (!f || *f == 0) {
    int nclusters = 0;
    e = cudaOccupancyMaxActiveClusters(&nclusters, (void*)kern, &cfg);
    if (e != cudaSuccess) cudaGetLastError();
    ok = e == cudaSuccess && nclusters >= 1;
    if (f) *f = ok ? 1 : -1;
  }
  if (!ok) return cudaErrorNotSupported;
  PanelScratch<float> ps{};
  ps.trace = trace;
  PanelParams<float> prm{A, lda, mp, w, R, ipiv, row_base, info_base, 0, ps, st, 0,
                         swap_lo, swap_hi, sib_w};
  if (g_panel_pdl) {
    // the leaf may be placed while the update before it on the stream
    // finishes; it waits for that update (pdl_wait) before touching memory
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.numAttrs = 2;
  }
  return cudaLaunchKernelEx(&cfg, kern, prm);
}

template <typename T>
cudaError_t launch_getf2_panel(T* A, long lda, int mp, int w, int* ipiv, int row_base,
                               int info_base, int epoch_base, const PanelScratch<T>& s,
                               DevStatus* st, int num_sms, cudaStream_t stream, bool nopiv,
                               int swap_lo, int swap_hi, bool* swaps_done, int sib_w,
                               bool* node_done) {
  if (swaps_done) *swaps_done = false;
  if (node_done) *node_done = false;
  if (w <= 0 || mp <= 0) return cudaSuccess;
  if (w > kPanelW || mp < w) return cudaErrorInvalidValue;
  if constexpr (sizeof(T) == 4) {
    if (g_panel_regs == 2 && g_panel_cluster > 1 && !nopiv) {
      // rows in registers on a cluster where one fits (<= 1024 rows per CTA;
      // narrow leaves of taller panels: 16 CTAs of up to 2048 rows)
      int C = cluster_ctas<T>(mp, g_panel_cluster);
      if (w <= 16 && g_panel_cluster == 16 && mp > 16 * 2 * kRcThreads &&
          mp <= 16 * 4 * kRcThreads)
        C = 16;
      if (C > 0 && ceil_div(mp, C) <= (w <= 16 ? 4 : 2) * kRcThreads) {
        const bool fuse = swaps_done != nullptr && (swap_lo < 0 || swap_hi > w);
        // the node update needs the sibling's interchanges done first, here
        const int sw = (fuse && node_done && sib_w > 0 && sib_w <= w && w + sib_w <= swap_hi)
                           ? sib_w
                           : 0;
        const cudaError_t e = launch_getf2_panel_cluster_reg(
            reinterpret_cast<float*>(A), lda, mp, w, ipiv, row_base, info_base, st, C, s.trace,
            stream, fuse ? swap_lo : 0, fuse ? swap_hi : 0, sw);
        if (e == cudaSuccess && fuse) *swaps_done = true;
        if (e == cudaSuccess && sw > 0) *node_done = true;
        if (e != cudaErrorNotSupported) return e;
      }
    }
    if (g_panel_regs == 1 && !nopiv) {
      // ~1024 rows per CTA (512 threads x 2 rows in registers)
      const int Rr = kRegThreads * kRegRows;
      int G = ceil_div(mp, Rr);
      if (G <= std::min({num_sms, s.maxG, kRegThreads / 2})) {
        PanelParams<float> prm{reinterpret_cast<float*>(A), lda, mp, w, Rr, ipiv, row_base,
                               info_base, epoch_base,
                               PanelScratch<float>{reinterpret_cast<PanelSlot<float>*>(s.slots),
                                                   s.maxG, s.cand},
                               st};
        void* args[] = {&prm};
        return cudaLaunchCooperativeKernel((const void*)getf2_panel_reg_kernel<kPanelW>, dim3(G),
                                           dim3(kRegThreads), args, 0, stream);
      }
    }
  }
  if (g_panel_cluster > 1 && !nopiv) {
    const int C = cluster_ctas<T>(mp, g_panel_cluster);
    if (C > 0) {
      const cudaError_t e =
          launch_getf2_panel_cluster<T>(A, lda, mp, w, ipiv, row_base, info_base, st, C, s.trace,
                                        stream);
      if (e != cudaErrorNotSupported) return e;
    }
  }
  constexpr int kMaxSmem = 200 * 1024;
  // About g_panel_rows rows per CTA: fewer CTAs make the per-column
  // exchange cheap (every CTA copies every candidate row), more make the
  // local update short; shared memory sets the fewest.
  const int rows_cap = (int)(kMaxSmem / (kPanelW * sizeof(T))) - 64 - 16;
  int G = std::max(ceil_div(mp, g_panel_rows), ceil_div(mp, rows_cap));
  if (G > num_sms) G = num_sms;
  if (G > s.maxG) G = s.maxG;
  if (G > panel_threads<T>()) G = panel_threads<T>();
  if (G < 1) G = 1;
  int R = ceil_div(mp, G);
  G = ceil_div(mp, R);  // no CTA without rows
  size_t smem = (slab_elems<T>(R) + (size_t)G * kPanelW) * sizeof(T);  // slab + candidate rows
  if (smem > (size_t)kMaxSmem) return cudaErrorInvalidValue;
  auto kern = getf2_panel_kernel<T, kPanelW>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       kMaxSmem);
  if (e != cudaSuccess) return e;
  PanelParams<T> prm{A, lda, mp, w, R, ipiv, row_base, info_base, epoch_base, s, st,
                     nopiv ? 1 : 0};
  void* args[] = {&prm};
  return cudaLaunchCooperativeKernel((const void*)kern, dim3(G), dim3(panel_threads<T>()),
                                     args, smem, stream);
}

template cudaError_t launch_getf2_panel<double>(double*, long, int, int, int*, int, int, int,
                                                const PanelScratch<double>&, DevStatus*,
                                                int, cudaStream_t, bool, int, int, bool*, int,
                                                bool*);
template cudaError_t launch_getf2_panel<float>(float*, long, int, int, int*, int, int, int,
                                               const PanelScratch<float>&, DevStatus*,
                                               int, cudaStream_t, bool, int, int, bool*, int,
                                               bool*);

// ---------------------------------------------------------------------------
// El::LU(A, P, Q) with full pivoting (src/lapack_like/factor/LU/Full.hpp:15-59)
// ---------------------------------------------------------------------------
// Unblocked, as the reference: per step k the pivot is the entry of largest
// magnitude of the trailing block -- on equal magnitudes the first in
// column-major order (MaxAbsLoc's strict '>' scan from 0 at the block's
// corner, src/blas_like/level1/MaxAbsLoc.cpp:131-163) -- then RowSwap and
// ColSwap over the whole matrix, a21 *= 1/alpha and the rank-1 update.
// Two kernels per step: fullpiv_swap (swaps + scaling) and fullpiv_update
// (rank-1 update of the trailing block fused with the next step's pivot
// search; the last CTA to finish reduces the per-CTA candidates, so no CTA
// ever waits on another).
template <typename T>
__device__ __forceinline__ bool fp_better(T v, int i, int j, T bv, int bi, int bj) {
  if (v != bv) return v > bv;  // NaN never wins (as MaxAbsLoc's '>')
  return j < bj || (j == bj && i < bi);
}

template <typename T>
__global__ void fullpiv_swap_kernel(T* __restrict__ A, long lda, int m, int n, int k,
                                    FullPivState<T>* __restrict__ fs, int* __restrict__ p,
                                    int* __restrict__ q, DevStatus* st) {
  const int ip = fs->i, jp = fs->j;
  const T alpha = fs->alpha;  // the pivot's value, recorded by the search
  const bool singular = alpha == T(0);
  const T inv = singular ? T(1) : T(1) / alpha;
  const long tid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long nth = (long)gridDim.x * blockDim.x;
  if (tid == 0) {
    p[k] = ip;
    q[k] = jp;
    if (singular) atomicCAS(&st->info, 0, k + 1);
    // the four entries both swaps move: row swap, then column swap
    const T kk = A[k + (long)k * lda], kj = A[k + (long)jp * lda];
    const T ik = A[ip + (long)k * lda], ij = A[ip + (long)jp * lda];
    A[k + (long)k * lda] = ij;
    A[k + (long)jp * lda] = ik;
    A[ip + (long)jp * lda] = kk;
    A[ip + (long)k * lda] = ip > k ? kj * inv : kj;  // below the diagonal: scaled
  }
  // row swap on every other column
  if (ip != k)
    for (long c = tid; c < n; c += nth) {
      if (c == k || c == jp) continue;
      T* a = A + k + c * lda;
      T* b = A + ip + c * lda;
      const T t = *a;
      *a = *b;
      *b = t;
    }
  // column swap on every other row; rows below k take the scaling
  for (long r = tid; r < m; r += nth) {
    if (r == k || r == ip) continue;
    T* a = A + r + (long)k * lda;
    T* b = A + r + (long)jp * lda;
    const T t = *a;
    *a = r > k ? *b * inv : *b;
    if (jp != k) *b = t;
  }
}

constexpr int kFpThreads = 256, kFpCols = 16;

// Rank-1 update of the trailing block A[k+1:m, k+1:n] (skipped for the
// initial search, k = -1) and the next pivot: one row per thread, kFpCols
// columns per CTA tile, tiles grid-strided.
template <typename T>
__global__ void __launch_bounds__(kFpThreads)
fullpiv_update_kernel(T* __restrict__ A, long lda, int m, int n, int k,
                      FullPivState<T>* __restrict__ fs, FullPivCand<T>* __restrict__ part) {
  __shared__ T s_v[kFpThreads / 32];
  __shared__ T s_s[kFpThreads / 32];
  __shared__ int s_i[kFpThreads / 32], s_j[kFpThreads / 32];
  __shared__ bool s_last;
  const int r0 = k + 1;
  const int rows = m - r0, cols = n - r0;
  const int rt = (rows + kFpThreads - 1) / kFpThreads, ct = (cols + kFpCols - 1) / kFpCols;
  const long tiles = (long)rt * ct;
  T bv = T(-1), bs = T(0);
  int bi = 0x7fffffff, bj = 0x7fffffff;
  for (long t = blockIdx.x; t < tiles; t += gridDim.x) {
    const int ti = (int)(t % rt), tj = (int)(t / rt);
    const int i = r0 + ti * kFpThreads + threadIdx.x;
    if (i >= m) continue;
    const T l = k >= 0 ? A[i + (long)k * lda] : T(0);
    const int j1 = min(r0 + (tj + 1) * kFpCols, n);
    for (int j = r0 + tj * kFpCols; j < j1; ++j) {
      T* a = A + i + (long)j * lda;
      T v = *a;
      if (k >= 0) {
        v = fma(l, -A[k + (long)j * lda], v);  // Geru(-1, a21, a12, A22)
        *a = v;
      }
      const T av = v < T(0) ? -v : v;
      if (fp_better(av, i, j, bv, bi, bj)) {
        bv = av;
        bs = v;
        bi = i;
        bj = j;
      }
    }
  }
  // the CTA's candidate
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    const T ov = __shfl_xor_sync(0xffffffffu, bv, o);
    const T os = __shfl_xor_sync(0xffffffffu, bs, o);
    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
    const int oj = __shfl_xor_sync(0xffffffffu, bj, o);
    if (fp_better(ov, oi, oj, bv, bi, bj)) {
      bv = ov;
      bs = os;
      bi = oi;
      bj = oj;
    }
  }
  if (lane == 0) {
    s_v[warp] = bv;
    s_s[warp] = bs;
    s_i[warp] = bi;
    s_j[warp] = bj;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < kFpThreads / 32; ++w)
      if (fp_better(s_v[w], s_i[w], s_j[w], s_v[0], s_i[0], s_j[0])) {
        s_v[0] = s_v[w];
        s_s[0] = s_s[w];
        s_i[0] = s_i[w];
        s_j[0] = s_j[w];
      }
    part[blockIdx.x] = FullPivCand<T>{s_v[0], s_s[0], s_i[0], s_j[0]};
    __threadfence();
    s_last = atomicAdd(&fs->count, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return;
  // the last CTA: every candidate is published (fence before each count)
  __threadfence();
  bv = T(-1);
  bs = T(0);
  bi = bj = 0x7fffffff;
  for (int b = threadIdx.x; b < gridDim.x; b += kFpThreads) {
    const volatile FullPivCand<T>* c = part + b;  // written by other CTAs
    const T cv = c->v, cs = c->s;
    const int ci = c->i, cj = c->j;
    if (fp_better(cv, ci, cj, bv, bi, bj)) {
      bv = cv;
      bs = cs;
      bi = ci;
      bj = cj;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const T ov = __shfl_xor_sync(0xffffffffu, bv, o);
    const T os = __shfl_xor_sync(0xffffffffu, bs, o);
    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
    const int oj = __shfl_xor_sync(0xffffffffu, bj, o);
    if (fp_better(ov, oi, oj, bv, bi, bj)) {
      bv = ov;
      bs = os;
      bi = oi;
      bj = oj;
    }
  }
  if (lane == 0) {
    s_v[warp] = bv;
    s_s[warp] = bs;
    s_i[warp] = bi;
    s_j[warp] = bj;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < kFpThreads / 32; ++w)
      if (fp_better(s_v[w], s_i[w], s_j[w], s_v[0], s_i[0], s_j[0])) {
        s_v[0] = s_v[w];
        s_s[0] = s_s[w];
        s_i[0] = s_i[w];
        s_j[0] = s_j[w];
      }
    // all candidates zero (or the block empty): the block's corner, as
    // MaxAbsLoc's scan starting from 0 at (0, 0)
    const bool none = !(s_v[0] > T(0));
    fs->i = none ? r0 : s_i[0];
    fs->j = none ? r0 : s_j[0];
    fs->alpha = none ? T(0) : s_s[0];
    fs->count = 0;
  }
}

// ---------------------------------------------------------------------------
// El::Cholesky(uplo, A, P) with diagonal pivoting (src/lapack_like/factor/
// Cholesky.cpp:44-52, Cholesky/Pivoted{Lower,Upper}Variant3.hpp)
// ---------------------------------------------------------------------------
// Right-looking and unblocked here (the reference's lazy panels compute the
// same updated diagonals): per step the updated diagonal's largest magnitude
// (the first on ties, VectorMaxAbsLoc) is the pivot, SymmetricSwap(LOWER)
// moves it to (k, k) (src/blas_like/level1/Swap.cpp:243-301), the column is
// scaled by 1/sqrt(pivot) and the trailing lower triangle takes the rank-1
// update fused with the next pivot search.  The upper variant runs the same
// steps on the transpose (element (i, j) of the lower view is A(j, i)).
template <typename T>
__device__ __forceinline__ T* pc_at(T* A, long lda, bool upper, int i, int j) {
  return upper ? A + j + (long)i * lda : A + i + (long)j * lda;
}

template <typename T>
__global__ void pchol_swap_kernel(T* __restrict__ A, long lda, int n, int k, int upper,
                                  const FullPivState<T>* __restrict__ fs, int* __restrict__ piv) {
  const int frm = fs->i;
  const T delta = sqrt(fs->alpha);  // NaN for a negative pivot, as the reference's Sqrt
  const T inv = T(1) / delta;
  const bool up = upper != 0;
  const long tid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long nth = (long)gridDim.x * blockDim.x;
  if (tid == 0) {
    piv[k] = frm;
    if (frm != k) {
      *pc_at(A, lda, up, frm, frm) = *pc_at(A, lda, up, k, k);  // diagonal swap
      T* c = pc_at(A, lda, up, frm, k);                          // the corner stays,
      *c = *c * inv;                                             // below the diagonal: scaled
    }
    *pc_at(A, lda, up, k, k) = delta;
  }
  if (frm != k)
    for (long j = tid; j < k; j += nth) {  // left: rows k and frm
      T* a = pc_at(A, lda, up, k, (int)j);
      T* b = pc_at(A, lda, up, frm, (int)j);
      const T t = *a;
      *a = *b;
      *b = t;
    }
  for (long i = k + 1 + tid; i < frm; i += nth) {  // inner: column k <-> row frm
    T* a = pc_at(A, lda, up, (int)i, k);
    T* b = pc_at(A, lda, up, frm, (int)i);
    const T t = *a;
    *a = *b * inv;
    *b = t;
  }
  for (long i = (long)max(frm, k) + 1 + tid; i < n; i += nth) {  // bottom: columns k, frm
    T* a = pc_at(A, lda, up, (int)i, k);
    T* b = pc_at(A, lda, up, (int)i, frm);
    const T t = *a;
    *a = *b * inv;
    if (frm != k) *b = t;
  }
}

// Rank-1 update of the trailing lower triangle (skipped for the initial
// search, k = -1) and the next pivot among its diagonal entries.
template <typename T>
__global__ void __launch_bounds__(kFpThreads)
pchol_update_kernel(T* __restrict__ A, long lda, int n, int k, int upper,
                    FullPivState<T>* __restrict__ fs, FullPivCand<T>* __restrict__ part) {
  __shared__ T s_v[kFpThreads / 32];
  __shared__ T s_s[kFpThreads / 32];
  __shared__ int s_i[kFpThreads / 32];
  __shared__ bool s_last;
  const bool up = upper != 0;
  const int r0 = k + 1, rows = n - r0;
  const int rt = (rows + kFpThreads - 1) / kFpThreads, ct = (rows + kFpCols - 1) / kFpCols;
  const long tiles = (long)rt * ct;
  T bv = T(-1), bs = T(0);
  int bi = 0x7fffffff;
  for (long t = blockIdx.x; t < tiles; t += gridDim.x) {
    const int ti = (int)(t % rt), tj = (int)(t / rt);
    const int j0 = r0 + tj * kFpCols, j1 = min(j0 + kFpCols, n);
    if (r0 + (ti + 1) * kFpThreads - 1 < j0) continue;  // entirely above the diagonal
    const int i = r0 + ti * kFpThreads + threadIdx.x;
    if (i >= n || i < j0) continue;
    const T l = k >= 0 ? *pc_at(A, lda, up, i, k) : T(0);
    const int jl = min(j1, i + 1);  // the lower triangle: j <= i
    for (int j = j0; j < jl; ++j) {
      T* a = pc_at(A, lda, up, i, j);
      T v = *a;
      if (k >= 0) {
        v = fma(l, -*pc_at(A, lda, up, j, k), v);  // Her(LOWER, -1, a21, A22)
        *a = v;
      }
      if (j == i) {
        const T av = v < T(0) ? -v : v;
        if (fp_better(av, i, i, bv, bi, bi)) {
          bv = av;
          bs = v;
          bi = i;
        }
      }
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  auto reduce_warp = [&]() {
    for (int o = 16; o > 0; o >>= 1) {
      const T ov = __shfl_xor_sync(0xffffffffu, bv, o);
      const T os = __shfl_xor_sync(0xffffffffu, bs, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (fp_better(ov, oi, oi, bv, bi, bi)) {
        bv = ov;
        bs = os;
        bi = oi;
      }
    }
  };
  auto reduce_cta = [&]() {
    if (lane == 0) {
      s_v[warp] = bv;
      s_s[warp] = bs;
      s_i[warp] = bi;
    }
    __syncthreads();
    if (threadIdx.x == 0)
      for (int w = 1; w < kFpThreads / 32; ++w)
        if (fp_better(s_v[w], s_i[w], s_i[w], s_v[0], s_i[0], s_i[0])) {
          s_v[0] = s_v[w];
          s_s[0] = s_s[w];
          s_i[0] = s_i[w];
        }
  };
  reduce_warp();
  reduce_cta();
  if (threadIdx.x == 0) {
    part[blockIdx.x] = FullPivCand<T>{s_v[0], s_s[0], s_i[0], s_i[0]};
    __threadfence();
    s_last = atomicAdd(&fs->count, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  bv = T(-1);
  bs = T(0);
  bi = 0x7fffffff;
  for (int b = threadIdx.x; b < gridDim.x; b += kFpThreads) {
    const volatile FullPivCand<T>* c = part + b;
    const T cv = c->v, cs = c->s;
    const int ci = c->i;
    if (fp_better(cv, ci, ci, bv, bi, bi)) {
      bv = cv;
      bs = cs;
      bi = ci;
    }
  }
  reduce_warp();
  __syncthreads();
  reduce_cta();
  if (threadIdx.x == 0) {
    const bool none = !(s_v[0] > T(0));  // VectorMaxAbsLoc: index 0 at value 0
    fs->i = fs->j = none ? r0 : s_i[0];
    fs->alpha = none ? T(0) : s_s[0];
    fs->count = 0;
  }
}

template <typename T>
cudaError_t launch_cholesky_piv(T* A, long lda, int n, bool upper, int* piv,
                                FullPivState<T>* fs, FullPivCand<T>* part, int grid,
                                cudaStream_t stream, long long* nlaunch) {
  if (n == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(fs, 0, sizeof(FullPivState<T>), stream);
  if (e != cudaSuccess) return e;
  const int up = upper ? 1 : 0;
  pchol_update_kernel<T><<<grid, kFpThreads, 0, stream>>>(A, lda, n, -1, up, fs, part);
  *nlaunch += 1;
  const int sgrid = std::max(1, std::min(ceil_div(n, 256), 64));
  for (int k = 0; k < n; ++k) {
    pchol_swap_kernel<T><<<sgrid, 256, 0, stream>>>(A, lda, n, k, up, fs, piv);
    *nlaunch += 1;
    if (k + 1 < n) {
      pchol_update_kernel<T><<<grid, kFpThreads, 0, stream>>>(A, lda, n, k, up, fs, part);
      *nlaunch += 1;
    }
    if ((k & 255) == 0 && (e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

template cudaError_t launch_cholesky_piv<double>(double*, long, int, bool, int*,
                                                 FullPivState<double>*, FullPivCand<double>*,
                                                 int, cudaStream_t, long long*);
template cudaError_t launch_cholesky_piv<float>(float*, long, int, bool, int*,
                                                FullPivState<float>*, FullPivCand<float>*, int,
                                                cudaStream_t, long long*);

int fullpiv_grid(int num_sms) { return 4 * num_sms; }

template <typename T>
cudaError_t launch_lu_full(T* A, long lda, int m, int n, int* p, int* q, FullPivState<T>* fs,
                           FullPivCand<T>* part, int grid, DevStatus* st, cudaStream_t stream,
                           long long* nlaunch) {
  const int mn = std::min(m, n);
  if (mn == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(fs, 0, sizeof(FullPivState<T>), stream);
  if (e != cudaSuccess) return e;
  fullpiv_update_kernel<T><<<grid, kFpThreads, 0, stream>>>(A, lda, m, n, -1, fs, part);
  *nlaunch += 1;
  const int sgrid = std::max(1, std::min(ceil_div(std::max(m, n), 256), 64));
  for (int k = 0; k < mn; ++k) {
    fullpiv_swap_kernel<T><<<sgrid, 256, 0, stream>>>(A, lda, m, n, k, fs, p, q, st);
    *nlaunch += 1;
    if (k + 1 < m && k + 1 < n) {
      fullpiv_update_kernel<T><<<grid, kFpThreads, 0, stream>>>(A, lda, m, n, k, fs, part);
      *nlaunch += 1;
    }
    if ((k & 255) == 0 && (e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

template cudaError_t launch_lu_full<double>(double*, long, int, int, int*, int*,
                                            FullPivState<double>*, FullPivCand<double>*, int,
                                            DevStatus*, cudaStream_t, long long*);
template cudaError_t launch_lu_full<float>(float*, long, int, int, int*, int*,
                                           FullPivState<float>*, FullPivCand<float>*, int,
                                           DevStatus*, cudaStream_t, long long*);

// ---------------------------------------------------------------------------
// K2: row interchanges (PB.PermuteRows, src/lapack_like/factor/LU.cpp:130-131)
// ---------------------------------------------------------------------------
// The nb swaps (k+i <-> ipiv[i], applied in order) become the list of rows
// whose contents change and the original row each one receives; applying
// that list touches every affected element once (read all, then write all)
// instead of replaying nb dependent swaps.  The list is built in parallel:
//   * E(t), the original row sitting at row k+t just before swap t, is
//     E(t') for the last earlier swap t' whose target was row k+t, else k+t
//     itself (resolved for all t at once by pointer jumping, the links
//     point to earlier swaps only);
//   * row k+i ends with what swap i brings in: E(i) if ipiv[i] = k+i, else
//     E(t) of the last earlier swap t with the same target, else the
//     untouched original row ipiv[i];
//   * a row below the block ends with E(t) of the last swap t targeting it.
// Targets are found through an open-addressing hash table in shared memory,
// each slot with the chain of swaps that target its row.
__device__ __forceinline__ int swap_hash(int row, int mask) {
  return (int)(((unsigned)row * 2654435761u) >> 7) & mask;
}

// Slot of `key` (inserted beforehand), or -1 when absent.
__device__ __forceinline__ int swap_find(const int* keys, int key, int mask) {
  int h = swap_hash(key, mask);
  while (true) {
    const int v = keys[h];
    if (v == key) return h;
    if (v == -1) return -1;
    h = (h + 1) & mask;
  }
}

__global__ void __launch_bounds__(1024)
build_swap_pairs_kernel(const int* __restrict__ ipiv, int k, int nb, int tbits,
                        int* __restrict__ pairs, int* __restrict__ count) {
  extern __shared__ int sh[];
  __shared__ int s_wsum[32];
  const int tsize = 1 << tbits, mask = tsize - 1;
  const int tid = threadIdx.x, bd = blockDim.x;
  int* p = sh;             // targets
  int* nxt = p + nb;       // next swap of the same target's chain (-1 ends)
  int* prv = nxt + nb;     // last earlier swap with the same target (-1)
  int* lst = prv + nb;     // 1: no later swap has the same target
  int* E0 = lst + nb;      // pointer jumping: resolved E(t) or -1 ...
  int* E1 = E0 + nb;
  int* P0 = E1 + nb;       // ... and the swap whose E is still needed
  int* P1 = P0 + nb;
  int* keys = P1 + nb;     // hash: target row (-1 empty)
  int* head = keys + tsize;  // first swap of the slot's chain (-1)
  for (int t = tid; t < nb; t += bd) p[t] = ipiv[t];
  for (int h = tid; h < tsize; h += bd) {
    keys[h] = -1;
    head[h] = -1;
  }
  __syncthreads();
  for (int t = tid; t < nb; t += bd) {
    const int key = p[t];
    int h = swap_hash(key, mask);
    while (true) {
      const int old = atomicCAS(&keys[h], -1, key);
      if (old == -1 || old == key) break;
      h = (h + 1) & mask;
    }
    nxt[t] = atomicExch(&head[h], t);
  }
  __syncthreads();
  for (int t = tid; t < nb; t += bd) {
    int pv = -1, mx = -1;
    for (int q = head[swap_find(keys, p[t], mask)]; q >= 0; q = nxt[q]) {
      mx = max(mx, q);
      if (q < t) pv = max(pv, q);
    }
    prv[t] = pv;
    lst[t] = mx == t;
    int lk = -1;  // last earlier swap that targeted row k+t
    const int h = swap_find(keys, k + t, mask);
    if (h >= 0)
      for (int q = head[h]; q >= 0; q = nxt[q])
        if (q < t) lk = max(lk, q);
    E0[t] = lk < 0 ? k + t : -1;
    P0[t] = lk;
  }
  __syncthreads();
  int* Ec = E0;
  int* Pc = P0;
  int* En = E1;
  int* Pn = P1;
  for (int span = 1; span < 2 * nb; span *= 2) {
    for (int t = tid; t < nb; t += bd) {
      int e = Ec[t], q = Pc[t];
      if (e < 0) {
        if (Ec[q] >= 0) {
          e = Ec[q];
          q = -1;
        } else {
          q = Pc[q];
        }
      }
      En[t] = e;
      Pn[t] = q;
    }
    __syncthreads();
    int* x = Ec;
    Ec = En;
    En = x;
    x = Pc;
    Pc = Pn;
    Pn = x;
  }
  // the changed rows: count per thread, block-wide scan, then write
  auto fin_in = [&](int t) {
    return p[t] == k + t ? Ec[t] : (prv[t] >= 0 ? Ec[prv[t]] : p[t]);
  };
  auto out_row = [&](int t) { return lst[t] && p[t] >= k + nb && Ec[t] != p[t]; };
  int mine = 0;
  for (int t = tid; t < nb; t += bd) mine += (fin_in(t) != k + t) + out_row(t);
  const int lane = tid & 31, warp = tid >> 5;
  int incl = mine;
  for (int o = 1; o < 32; o *= 2) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) s_wsum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const int nw = (bd + 31) >> 5;
    int v = lane < nw ? s_wsum[lane] : 0;
    for (int o = 1; o < 32; o *= 2) {
      const int u = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += u;
    }
    if (lane < nw) s_wsum[lane] = v;  // inclusive per warp
  }
  __syncthreads();
  int off = incl - mine + (warp > 0 ? s_wsum[warp - 1] : 0);
  int* dst = pairs;
  int* src = pairs + 2 * nb;
  for (int t = tid; t < nb; t += bd) {
    const int f = fin_in(t);
    if (f != k + t) {
      dst[off] = k + t;
      src[off] = f;
      ++off;
    }
    if (out_row(t)) {
      dst[off] = p[t];
      src[off] = Ec[t];
      ++off;
    }
  }
  if (tid == bd - 1) *count = off;
}

cudaError_t launch_build_swap_pairs(const int* ipiv, int k, int nb, int* pairs, int* count,
                                    cudaStream_t stream) {
  if (nb <= 0) return cudaMemsetAsync(count, 0, sizeof(int), stream);
  int tbits = 5;
  while ((1 << tbits) < 2 * nb) ++tbits;
  const size_t smem = (8 * (size_t)nb + 2 * ((size_t)1 << tbits)) * sizeof(int);
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  // the kernel's static shared memory (s_wsum) counts against the same 48 KB
  // default: at nb = 1024 the dynamic part alone is exactly 48 KB
  if (smem + sizeof(int) * 32 > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(build_swap_pairs_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
  }
  const int threads = std::min(1024, (nb + 31) / 32 * 32);
  build_swap_pairs_kernel<<<1, threads, smem, stream>>>(ipiv, k, nb, tbits, pairs, count);
  return cudaGetLastError();
}

constexpr int kSwapThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kSwapThreads)
apply_swap_pairs_kernel(T* __restrict__ A, long lda, int c0a, int c1a, int c0b, int c1b,
                        const int* __restrict__ pairs, const int* __restrict__ count,
                        int nb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int* s_dst = reinterpret_cast<int*>(smem_raw);
  int* s_src = s_dst + 2 * nb;
  T* buf = reinterpret_cast<T*>(s_src + 2 * nb);
  const int cnt = *count;
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    s_dst[e] = pairs[e];
    s_src[e] = pairs[2 * nb + e];
  }
  __syncthreads();
  if (cnt == 0) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T* wbuf = buf + (size_t)warp * 2 * nb;
  const int na = c1a - c0a, ncols = na + (c1b - c0b);
  const int gw = blockIdx.x * (blockDim.x >> 5) + warp;
  const int nw = gridDim.x * (blockDim.x >> 5);
  for (int q = gw; q < ncols; q += nw) {
    const int col = q < na ? c0a + q : c0b + (q - na);
    T* colp = A + (long)col * lda;
#pragma unroll 8
    for (int e = lane; e < cnt; e += 32) wbuf[e] = colp[s_src[e]];
    __syncwarp();
#pragma unroll 8
    for (int e = lane; e < cnt; e += 32) colp[s_dst[e]] = wbuf[e];
    __syncwarp();
  }
}

// The same with each lane's moved entries of a column in registers (at most
// 32 x PER moves): every load of the column is in flight at once before the
// stores, and shared memory holds only the pairs.  The moved rows are
// scattered over the column (one 32-byte sector each), so the kernel is
// bound by the number of DRAM sectors in flight, not by bytes.
template <typename T, int PER>
__global__ void __launch_bounds__(kSwapThreads)
apply_swap_pairs_reg_kernel(T* __restrict__ A, long lda, int c0a, int c1a, int c0b, int c1b,
                            const int* __restrict__ pairs, const int* __restrict__ count,
                            int nb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int* s_dst = reinterpret_cast<int*>(smem_raw);
  int* s_src = s_dst + 32 * PER;
  const int cnt = min(*count, 32 * PER);
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    s_dst[e] = pairs[e];
    s_src[e] = pairs[2 * nb + e];
  }
  __syncthreads();
  if (cnt == 0) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int na = c1a - c0a, ncols = na + (c1b - c0b);
  const int gw = blockIdx.x * (blockDim.x >> 5) + warp;
  const int nw = gridDim.x * (blockDim.x >> 5);
  for (int q = gw; q < ncols; q += nw) {
    const int col = q < na ? c0a + q : c0b + (q - na);
    T* colp = A + (long)col * lda;
    T v[PER];
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int e = lane + 32 * u;
      if (e < cnt) v[u] = colp[s_src[e]];
    }
    __syncwarp();
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int e = lane + 32 * u;
      if (e < cnt) colp[s_dst[e]] = v[u];
    }
  }
}

template <typename T>
cudaError_t launch_apply_swap_pairs(T* A, long lda, int c0a, int c1a, int c0b, int c1b,
                                    const int* pairs, const int* count, int nb,
                                    cudaStream_t stream) {
  const int ncols = max(c1a - c0a, 0) + max(c1b - c0b, 0);
  if (ncols == 0 || nb <= 0) return cudaSuccess;
  if (c1a < c0a) c1a = c0a;
  if (c1b < c0b) c1b = c0b;
  if (2 * nb <= 32 * 32) {  // at most 2 nb moves a column
    const int per = 2 * nb <= 32 * 8 ? 8 : 2 * nb <= 32 * 16 ? 16 : 32;
    auto kern = per == 8    ? apply_swap_pairs_reg_kernel<T, 8>
                : per == 16 ? apply_swap_pairs_reg_kernel<T, 16>
                            : apply_swap_pairs_reg_kernel<T, 32>;
    const size_t smem = 2 * 32 * (size_t)per * sizeof(int);
    int blocks = ceil_div(ncols, kSwapThreads / 32);
    if (blocks > 8192) blocks = 8192;
    kern<<<blocks, kSwapThreads, smem, stream>>>(A, lda, c0a, c1a, c0b, c1b, pairs, count, nb);
    return cudaGetLastError();
  }
  const size_t smem = 4 * (size_t)nb * sizeof(int) +
                      (size_t)(kSwapThreads / 32) * 2 * nb * sizeof(T);
  auto kern = apply_swap_pairs_kernel<T>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
  }
  int blocks = ceil_div(ncols, kSwapThreads / 32);
  if (blocks > 4096) blocks = 4096;
  kern<<<blocks, kSwapThreads, smem, stream>>>(A, lda, c0a, c1a, c0b, c1b, pairs, count, nb);
  return cudaGetLastError();
}

template cudaError_t launch_apply_swap_pairs<double>(double*, long, int, int, int, int,
                                                     const int*, const int*, int,
                                                     cudaStream_t);
template cudaError_t launch_apply_swap_pairs<float>(float*, long, int, int, int, int,
                                                    const int*, const int*, int,
                                                    cudaStream_t);

// ---- deferred left interchanges ----------------------------------------------
// One CTA per block column b: replay the interchanges of every later panel
// on row labels (shared memory when they fit, else in place in global
// memory), serially in one thread -- the replay is inherently ordered.
constexpr int kDeferChunk = 2048;

__global__ void defer_labels_kernel(const int* __restrict__ ipiv, int m, int mn, int nb,
                                    int* __restrict__ lab, int use_smem) {
  extern __shared__ int sl[];
  const int b = blockIdx.x;
  const int base = (b + 1) * nb;
  if (base >= m || base >= mn) return;
  const int rows = m - base;
  int* L = use_smem ? sl : lab + (long)b * m + base;
  for (int i = threadIdx.x; i < rows; i += blockDim.x) L[i] = base + i;
  __syncthreads();
  // the swaps come through shared memory a chunk at a time, so thread 0's
  // serial replay waits on shared memory only
  __shared__ int s_p[kDeferChunk];
  for (int t0 = base; t0 < mn; t0 += kDeferChunk) {
    const int nc = min(kDeferChunk, mn - t0);
    for (int i = threadIdx.x; i < nc; i += blockDim.x) s_p[i] = ipiv[t0 + i];
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int i = 0; i < nc; ++i) {
        const int t = t0 + i, p = s_p[i];  // partial pivoting: p >= t >= base
        if (p != t) {
          const int a = L[t - base];
          L[t - base] = L[p - base];
          L[p - base] = a;
        }
      }
    }
    __syncthreads();
  }
  if (use_smem)
    for (int i = threadIdx.x; i < rows; i += blockDim.x) lab[(long)b * m + base + i] = L[i];
}

// Columns c < (last block start): A(r, c) <- A(lab_b[r], c) for r >= base_b.
// With STAGE the CTA reads rows base_b .. m of the column into shared memory
// (coalesced) and writes them back permuted (coalesced; the random reads hit
// shared memory); otherwise through the CTA's own m-element slice of tmp (the
// gather from global memory is then one DRAM sector a row).
template <typename T, bool STAGE>
__global__ void __launch_bounds__(1024)
defer_gather_kernel(T* __restrict__ A, long lda, int m, int mn, int nb,
                    const int* __restrict__ lab, T* __restrict__ tmp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s_col = reinterpret_cast<T*>(smem_raw);
  const int nblk = (mn + nb - 1) / nb;
  const int ncols = (nblk - 1) * nb;  // the last block column has no later panel
  const int bd = blockDim.x, tid = threadIdx.x;
  T* t = tmp + (long)blockIdx.x * m;
  for (int c = blockIdx.x; c < ncols; c += gridDim.x) {
    const int b = c / nb, base = (b + 1) * nb;
    if (base >= m) continue;
    const int* lb = lab + (long)b * m;
    T* col = A + (long)c * lda;
    if (STAGE) {
#pragma unroll 4
      for (int r = base + tid; r < m; r += bd) s_col[r - base] = col[r];
      __syncthreads();
#pragma unroll 4
      for (int r = base + tid; r < m; r += bd) col[r] = s_col[lb[r] - base];
    } else {
      for (int r = base + tid; r < m; r += bd) t[r] = col[lb[r]];
      __syncthreads();
      for (int r = base + tid; r < m; r += bd) col[r] = t[r];
    }
    __syncthreads();
  }
}

int defer_gather_grid(int num_sms) { return 2 * num_sms; }

// Parallel form of the same labels.  With Q_b the replay from step base_b to
// the end applied to the identity, Q_b[i] = S_b[Q_{b+1}[i]], where S_b is the
// replay of block b+1's own steps [base_b, base_b + nb) alone (the identity
// outside at most 2 nb positions).  defer_maps_kernel makes every S_b at once
// (one CTA a block, nb serial steps each) as (position, value) pairs;
// defer_compose_kernel then walks the blocks from the last one back, one
// parallel gather a block.
__global__ void defer_maps_kernel(const int* __restrict__ ipiv, int m, int mn, int nb,
                                  int* __restrict__ pairs, int* __restrict__ counts) {
  extern __shared__ int sl[];  // positions base .. m
  __shared__ int s_p[kDeferChunk];
  __shared__ int s_cnt;
  const int b = blockIdx.x, base = (b + 1) * nb;
  const int rows = m - base;
  for (int i = threadIdx.x; i < rows; i += blockDim.x) sl[i] = base + i;
  if (threadIdx.x == 0) s_cnt = 0;
  __syncthreads();
  const int t_end = min(base + nb, mn);
  for (int t0 = base; t0 < t_end; t0 += kDeferChunk) {
    const int nc = min(kDeferChunk, t_end - t0);
    for (int i = threadIdx.x; i < nc; i += blockDim.x) s_p[i] = ipiv[t0 + i];
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int i = 0; i < nc; ++i) {
        const int t = t0 + i, p = s_p[i];  // p >= t >= base
        if (p != t) {
          const int a = sl[t - base];
          sl[t - base] = sl[p - base];
          sl[p - base] = a;
        }
      }
    }
    __syncthreads();
  }
  int* pos = pairs + (long)b * 4 * nb;
  int* val = pos + 2 * nb;
  for (int i = threadIdx.x; i < rows; i += blockDim.x)
    if (sl[i] != base + i) {
      const int k = atomicAdd(&s_cnt, 1);  // at most 2 nb moved positions
      pos[k] = base + i;
      val[k] = sl[i];
    }
  __syncthreads();
  if (threadIdx.x == 0) counts[b] = s_cnt;
}

__global__ void __launch_bounds__(1024)
defer_compose_kernel(int m, int mn, int nb, const int* __restrict__ pairs,
                     const int* __restrict__ counts, int* __restrict__ map, int* __restrict__ lab) {
  extern __shared__ int cur[];  // Q_{b+1}, the identity to start with
  const int nblk = (mn + nb - 1) / nb;
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    cur[i] = i;
    map[i] = i;
  }
  __syncthreads();
  for (int b = nblk - 2; b >= 0; --b) {
    const int base = (b + 1) * nb, cnt = counts[b];
    const int* pos = pairs + (long)b * 4 * nb;
    const int* val = pos + 2 * nb;
    for (int e = threadIdx.x; e < cnt; e += blockDim.x) map[pos[e]] = val[e];
    __syncthreads();
    int* lb = lab + (long)b * m;
#pragma unroll 4
    for (int i = base + threadIdx.x; i < m; i += blockDim.x) {
      const int v = map[cur[i]];
      cur[i] = v;
      lb[i] = v;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < cnt; e += blockDim.x) map[pos[e]] = pos[e];
    __syncthreads();
  }
}

size_t defer_labels_work_ints(int m, int mn, int nb) {
  const size_t nblk = (size_t)(std::max(mn, 1) + nb - 1) / std::max(nb, 1);
  return nblk * 4 * (size_t)nb + nblk + (size_t)m;
}

cudaError_t launch_defer_labels(const int* ipiv, int m, int mn, int nb, int* lab, int* work,
                                cudaStream_t stream) {
  const int nblk = (mn + nb - 1) / nb;
  if (nblk <= 1) return cudaSuccess;
  const size_t smem = (size_t)m * sizeof(int);
  const bool use_smem = smem <= 200 * 1024;
  if (use_smem && work) {
    int* pairs = work;
    int* counts = pairs + (size_t)nblk * 4 * nb;
    int* map = counts + nblk;
    const size_t msm = (size_t)std::max(m - nb, 1) * sizeof(int);
    if (msm + kDeferChunk * sizeof(int) > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(defer_maps_kernel,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)msm);
      if (e != cudaSuccess) return e;
    }
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(defer_compose_kernel,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    defer_maps_kernel<<<nblk - 1, 256, msm, stream>>>(ipiv, m, mn, nb, pairs, counts);
    defer_compose_kernel<<<1, 1024, smem, stream>>>(m, mn, nb, pairs, counts, map, lab);
    return cudaGetLastError();
  }
  // (the kernel's static pivot chunk counts against the same 48 KB default)
  if (use_smem && smem + kDeferChunk * sizeof(int) > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(defer_labels_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  defer_labels_kernel<<<nblk - 1, 256, use_smem ? smem : 0, stream>>>(ipiv, m, mn, nb, lab,
                                                                      use_smem ? 1 : 0);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_defer_gather(T* A, long lda, int m, int mn, int nb, const int* lab, T* tmp,
                                int grid, cudaStream_t stream) {
  const int nblk = (mn + nb - 1) / nb;
  if (nblk <= 1) return cudaSuccess;
  // rows nb .. m of a column (block column 0's share, the largest)
  const size_t smem = (size_t)std::max(m - nb, 0) * sizeof(T);
  if (smem <= 200 * 1024) {
    auto kern = defer_gather_kernel<T, true>;
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem);
      if (e != cudaSuccess) return e;
    }
    // one CTA an SM while a column takes over ~100 KB, else two
    const int per_sm = smem > 100 * 1024 ? 1 : 2;
    kern<<<grid / 2 * per_sm, 1024, smem, stream>>>(A, lda, m, mn, nb, lab, tmp);
    return cudaGetLastError();
  }
  defer_gather_kernel<T, false><<<grid, 256, 0, stream>>>(A, lda, m, mn, nb, lab, tmp);
  return cudaGetLastError();
}

template cudaError_t launch_defer_gather<double>(double*, long, int, int, int, const int*, double*,
                                                 int, cudaStream_t);
template cudaError_t launch_defer_gather<float>(float*, long, int, int, int, const int*, float*,
                                                int, cudaStream_t);

// Explicit permutation vector of a whole swap sequence (one thread; the
// labels live in shared memory when they fit).
__global__ void explicit_perm_kernel(const int* __restrict__ ipiv, int nswaps, int n,
                                     int* __restrict__ perm, int use_smem) {
  extern __shared__ int s_perm[];
  int* lab = use_smem ? s_perm : perm;
  for (int i = threadIdx.x; i < n; i += blockDim.x) lab[i] = i;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 0; i < nswaps; ++i) {
      const int d = ipiv[i];
      if (d != i) {
        const int t = lab[i];
        lab[i] = lab[d];
        lab[d] = t;
      }
    }
  }
  __syncthreads();
  if (use_smem)
    for (int i = threadIdx.x; i < n; i += blockDim.x) perm[i] = s_perm[i];
}

cudaError_t launch_explicit_perm(const int* ipiv, int nswaps, int n, int* perm,
                                 cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  const size_t smem = (size_t)n * sizeof(int);
  const int use_smem = smem <= 200 * 1024;
  if (use_smem && smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(explicit_perm_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         200 * 1024);
    if (e != cudaSuccess) return e;
  }
  explicit_perm_kernel<<<1, 1024, use_smem ? smem : 0, stream>>>(ipiv, nswaps, n, perm,
                                                                use_smem);
  return cudaGetLastError();
}

template <typename T>
__global__ void permute_rows_kernel(const T* __restrict__ X, long ldx, T* __restrict__ Y,
                                    long ldy, int n, int ncols,
                                    const int* __restrict__ perm, int inverse) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int pi = perm[i];
  for (int c = blockIdx.y; c < ncols; c += gridDim.y) {
    if (!inverse)
      Y[i + (long)c * ldy] = X[pi + (long)c * ldx];
    else
      Y[pi + (long)c * ldy] = X[i + (long)c * ldx];
  }
}

template <typename T>
cudaError_t launch_permute_rows(const T* X, long ldx, T* Y, long ldy, int n, int ncols,
                                const int* perm, bool inverse, cudaStream_t stream) {
  if (n <= 0 || ncols <= 0) return cudaSuccess;
  dim3 grid(ceil_div(n, 256), grid_y(ncols));
  permute_rows_kernel<T><<<grid, 256, 0, stream>>>(X, ldx, Y, ldy, n, ncols, perm,
                                                   inverse ? 1 : 0);
  return cudaGetLastError();
}
template cudaError_t launch_permute_rows<double>(const double*, long, double*, long, int,
                                                 int, const int*, bool, cudaStream_t);
template cudaError_t launch_permute_rows<float>(const float*, long, float*, long, int, int,
                                                const int*, bool, cudaStream_t);

// ---------------------------------------------------------------------------
// K4: triangular solve on one diagonal block, op(A11) X = B, nb <= NB
// ---------------------------------------------------------------------------
// op(A11) goes to shared memory once per CTA.  B is processed 32 columns at a
// time: staged through shared memory (coalesced in either storage order),
// then one warp per column keeps the column in registers (row lane + 32 t in
// x[t]) and substitutes with the pivot broadcast by a warp shuffle.
constexpr int kTrsmThreads = 256;
constexpr int kTrsmCols = 32;

template <typename T, int NB>
__global__ void __launch_bounds__(kTrsmThreads)
trsm_block_kernel(const T* __restrict__ A, long lda, T* __restrict__ Bm, long ldb, int nb,
                  int ncols, int lower, int unit, int trans_a, int trans_b, int bulk,
                  DevStatus* st) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t s_mbar;
  T* sA = reinterpret_cast<T*>(smem_raw);  // op(A)(i, j) at sA[i + j * NB]
  T* sB = sA + NB * NB;                     // B(i, c) at sB[i + c * (NB + 1)]
  constexpr int LDS = NB + 1;
  const int tid = threadIdx.x;
  pdl_launch_dependents();
  if (bulk) {
    // (caller: A, lda and nb rows of T in 16-byte units, A11 not
    // transposed) each of the nb columns' first nb rows in one bulk copy
    // by the TMA engine: one round trip instead of a loop of loads
    if (tid == 0) {
      tc::mbar_init(&s_mbar, 1);
      tc::fence_mbar_init();
      tc::mbar_arrive_expect_tx(&s_mbar, (uint32_t)(nb * nb * sizeof(T)));
    }
    __syncthreads();
    for (int j = tid; j < nb; j += blockDim.x)
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
          "[%3];" ::"r"((unsigned)__cvta_generic_to_shared(sA + j * NB)),
          "l"(A + (long)j * lda), "r"((uint32_t)(nb * sizeof(T))), "r"(tc::smem_u32(&s_mbar))
          : "memory");
    for (int idx = tid; idx < NB * NB; idx += blockDim.x) {
      const int i = idx % NB, j = idx / NB;
      if (i >= nb || j >= nb) sA[idx] = (i == j) ? T(1) : T(0);
    }
    tc::mbar_wait(&s_mbar, 0, st, 42);
  } else {
    for (int idx = tid; idx < NB * NB; idx += blockDim.x) {
      const int i = idx % NB, j = idx / NB;
      T v;
      if (i < nb && j < nb)
        v = trans_a ? A[j + (long)i * lda] : A[i + (long)j * lda];
      else
        v = (i == j) ? T(1) : T(0);
      sA[idx] = v;
    }
  }
  const int lane = tid & 31, warp = tid >> 5;
  constexpr int NT = NB / 32;
  for (int c0 = blockIdx.x * kTrsmCols; c0 < ncols; c0 += gridDim.x * kTrsmCols) {
    const int cw = min(kTrsmCols, ncols - c0);
    // B not transposed: each lane loads its rows of its columns straight into
    // registers (coalesced, all in flight at once); transposed: through
    // shared memory
    if (trans_b) {
      __syncthreads();
      for (int idx = tid; idx < NB * kTrsmCols; idx += blockDim.x) {
        const int c = idx % kTrsmCols, i = idx / kTrsmCols;
        sB[i + c * LDS] = (i < nb && c < cw) ? Bm[(c0 + c) + (long)i * ldb] : T(0);
      }
    }
    __syncthreads();
    // warp w solves columns w, w + 8, w + 16, w + 24 of the chunk together:
    // each column's operations and their order are those of a column solved
    // alone, but the four dependency chains (shuffle, FMA) interleave
    {
      constexpr int kW = kTrsmThreads / 32;
      constexpr int CPW = kTrsmCols / kW;
      static_assert(CPW * kW == kTrsmCols, "columns per warp");
      T x[CPW][NT];
      bool on[CPW];
#pragma unroll
      for (int q = 0; q < CPW; ++q) {
        const int c = warp + kW * q;
        on[q] = c < cw;
#pragma unroll
        for (int t = 0; t < NT; ++t) {
          const int i = lane + 32 * t;
          x[q][t] = !on[q] ? T(0)
                    : trans_b ? sB[i + c * LDS]
                              : (i < nb ? Bm[i + (long)(c0 + c) * ldb] : T(0));
        }
      }
      if (lower) {
#pragma unroll
        for (int t = 0; t < NT; ++t) {
#pragma unroll 8
          for (int jj = 0; jj < 32; ++jj) {
            const int j = 32 * t + jj;
            if (!unit && lane == jj) {
              const T d = sA[j + j * NB];
#pragma unroll
              for (int q = 0; q < CPW; ++q) x[q][t] = x[q][t] / d;
            }
            T xj[CPW];
#pragma unroll
            for (int q = 0; q < CPW; ++q) xj[q] = __shfl_sync(0xffffffffu, x[q][t], jj);
#pragma unroll
            for (int tt = t; tt < NT; ++tt) {
              const int i = lane + 32 * tt;
              if (i > j) {
                const T a = sA[i + j * NB];
#pragma unroll
                for (int q = 0; q < CPW; ++q) x[q][tt] = fma(-a, xj[q], x[q][tt]);
              }
            }
          }
        }
      } else {
#pragma unroll
        for (int t = NT - 1; t >= 0; --t) {
#pragma unroll 8
          for (int jj = 31; jj >= 0; --jj) {
            const int j = 32 * t + jj;
            if (!unit && lane == jj) {
              const T d = sA[j + j * NB];
#pragma unroll
              for (int q = 0; q < CPW; ++q) x[q][t] = x[q][t] / d;
            }
            T xj[CPW];
#pragma unroll
            for (int q = 0; q < CPW; ++q) xj[q] = __shfl_sync(0xffffffffu, x[q][t], jj);
#pragma unroll
            for (int tt = 0; tt <= t; ++tt) {
              const int i = lane + 32 * tt;
              if (i < j) {
                const T a = sA[i + j * NB];
#pragma unroll
                for (int q = 0; q < CPW; ++q) x[q][tt] = fma(-a, xj[q], x[q][tt]);
              }
            }
          }
        }
      }
#pragma unroll
      for (int q = 0; q < CPW; ++q)
        if (on[q])
#pragma unroll
          for (int t = 0; t < NT; ++t) {
            const int i = lane + 32 * t;
            if (trans_b)
              sB[i + (warp + kW * q) * LDS] = x[q][t];
            else if (i < nb)
              Bm[i + (long)(c0 + warp + kW * q) * ldb] = x[q][t];
          }
    }
    if (trans_b) {
      __syncthreads();
      for (int idx = tid; idx < NB * kTrsmCols; idx += blockDim.x) {
        const int c = idx % kTrsmCols, i = idx / kTrsmCols;
        if (i < nb && c < cw) Bm[(c0 + c) + (long)i * ldb] = sB[i + c * LDS];
      }
    }
  }
}

template <typename T, int NB>
static cudaError_t trsm_block_nb(const T* A11, long lda, T* Bm, long ldb, int nb, int ncols,
                                 bool lower, bool unit, bool trans_a, bool trans_b,
                                 cudaStream_t stream, DevStatus* st) {
  const size_t smem = ((size_t)NB * NB + (size_t)(NB + 1) * kTrsmCols) * sizeof(T);
  auto kern = trsm_block_kernel<T, NB>;
  if (smem + 64 > 48 * 1024) {  // (with the kernel's static mbarrier)
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
  }
  int blocks = ceil_div(ncols, kTrsmCols);
  if (blocks > 1024) blocks = 1024;
  const int bulk = !trans_a && st != nullptr && ((uintptr_t)A11 % 16) == 0 &&
                   ((size_t)lda * sizeof(T)) % 16 == 0 && ((size_t)nb * sizeof(T)) % 16 == 0;
  kern<<<blocks, kTrsmThreads, smem, stream>>>(A11, lda, Bm, ldb, nb, ncols, lower, unit,
                                                trans_a, trans_b, bulk, st);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_trsm_block(const T* A11, long lda, T* Bm, long ldb, int nb, int ncols,
                              bool lower, bool unit, bool trans_a, bool trans_b,
                              cudaStream_t stream, DevStatus* st) {
  if (nb <= 0 || ncols <= 0) return cudaSuccess;
  if (nb <= 32)
    return trsm_block_nb<T, 32>(A11, lda, Bm, ldb, nb, ncols, lower, unit, trans_a, trans_b,
                                stream, st);
  if (nb <= 64)
    return trsm_block_nb<T, 64>(A11, lda, Bm, ldb, nb, ncols, lower, unit, trans_a, trans_b,
                                stream, st);
  if (nb <= 128)
    return trsm_block_nb<T, 128>(A11, lda, Bm, ldb, nb, ncols, lower, unit, trans_a,
                                 trans_b, stream, st);
  return cudaErrorInvalidValue;
}
template cudaError_t launch_trsm_block<double>(const double*, long, double*, long, int, int,
                                               bool, bool, bool, bool, cudaStream_t,
                                               DevStatus*);
template cudaError_t launch_trsm_block<float>(const float*, long, float*, long, int, int,
                                              bool, bool, bool, bool, cudaStream_t, DevStatus*);

// out (n x n, leading dimension ldo) := the strictly lower triangle of A
// (zeros on and above the diagonal).
template <typename T>
__global__ void copy_strict_lower_kernel(const T* __restrict__ A, long lda, int n,
                                         T* __restrict__ out, long ldo) {
  const int j = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i + (long)j * ldo] = i > j ? A[i + (long)j * lda] : T(0);
}

template <typename T>
cudaError_t launch_copy_strict_lower(const T* A, long lda, int n, T* out, long ldo,
                                     cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  copy_strict_lower_kernel<T><<<dim3(ceil_div(n, 256), n), 256, 0, stream>>>(A, lda, n, out, ldo);
  return cudaGetLastError();
}
template cudaError_t launch_copy_strict_lower<double>(const double*, long, int, double*, long,
                                                      cudaStream_t);
template cudaError_t launch_copy_strict_lower<float>(const float*, long, int, float*, long,
                                                     cudaStream_t);

// ---------------------------------------------------------------------------
// K5 (FP64 and FP32 SIMT): C = alpha op(A) op(B) + beta C
// ---------------------------------------------------------------------------
// 64 x 64 tile per CTA, 256 threads, 4 x 4 outputs per thread (rows tx+16i,
// columns ty+16j: conflict-free shared-memory reads), K in steps of 16 with
// register prefetch of the next step.
constexpr int kGBM = 64, kGBN = 64, kGBK = 16;

template <typename T, bool TA, bool TB>
__global__ void __launch_bounds__(256)
gemm_simt_kernel(int m, int n, int k, T alpha, const T* __restrict__ A, long lda,
                 const T* __restrict__ Bm, long ldb, T beta, T* __restrict__ C, long ldc,
                 int uplo) {
  __shared__ T sA[kGBK][kGBM + 1];
  __shared__ T sB[kGBK][kGBN + 1];
  pdl_launch_dependents();  // a leaf panel after it may be scheduled now
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int row0 = blockIdx.x * kGBM, col0 = blockIdx.y * kGBN;
  if (uplo == 1 && col0 > row0 + kGBM - 1) return;  // tile strictly above diagonal
  if (uplo == 2 && row0 > col0 + kGBN - 1) return;  // tile strictly below diagonal
  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = T(0);

  T ra[4], rb[4];
  auto load = [&](int k0) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int i, kk;
      if (!TA) { i = tid % kGBM; kk = tid / kGBM + 4 * q; }
      else { kk = tid % kGBK; i = tid / kGBK + 16 * q; }
      const int gi = row0 + i, gk = k0 + kk;
      ra[q] = (gi < m && gk < k) ? (TA ? A[gk + (long)gi * lda] : A[gi + (long)gk * lda])
                                 : T(0);
      int j, kb;
      if (!TB) { kb = tid % kGBK; j = tid / kGBK + 16 * q; }
      else { j = tid % kGBN; kb = tid / kGBN + 4 * q; }
      const int gj = col0 + j, gkb = k0 + kb;
      rb[q] = (gj < n && gkb < k) ? (TB ? Bm[gj + (long)gkb * ldb] : Bm[gkb + (long)gj * ldb])
                                  : T(0);
    }
  };
  auto store = [&]() {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int i, kk;
      if (!TA) { i = tid % kGBM; kk = tid / kGBM + 4 * q; }
      else { kk = tid % kGBK; i = tid / kGBK + 16 * q; }
      sA[kk][i] = ra[q];
      int j, kb;
      if (!TB) { kb = tid % kGBK; j = tid / kGBK + 16 * q; }
      else { j = tid % kGBN; kb = tid / kGBN + 4 * q; }
      sB[kb][j] = rb[q];
    }
  };
  load(0);
  for (int k0 = 0; k0 < k; k0 += kGBK) {
    __syncthreads();
    store();
    __syncthreads();
    if (k0 + kGBK < k) load(k0 + kGBK);
#pragma unroll
    for (int kk = 0; kk < kGBK; ++kk) {
      T a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = sA[kk][tx + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = sB[kk][ty + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int gj = col0 + ty + 16 * j;
    if (gj >= n) continue;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int gi = row0 + tx + 16 * i;
      if (gi >= m) continue;
      if (uplo == 1 && gi < gj) continue;
      if (uplo == 2 && gi > gj) continue;
      T* cp = C + gi + (long)gj * ldc;
      *cp = (beta == T(0)) ? alpha * acc[i][j] : fma(alpha, acc[i][j], beta * *cp);
    }
  }
}

template <typename T>
cudaError_t launch_gemm_simt(bool ta, bool tb, int m, int n, int k, T alpha, const T* A,
                             long lda, const T* Bm, long ldb, T beta, T* C, long ldc,
                             int uplo, cudaStream_t stream) {
  if (m <= 0 || n <= 0) return cudaSuccess;
  dim3 grid(ceil_div(m, kGBM), ceil_div(n, kGBN));
  if (ta && tb)
    gemm_simt_kernel<T, true, true><<<grid, 256, 0, stream>>>(m, n, k, alpha, A, lda, Bm,
                                                               ldb, beta, C, ldc, uplo);
  else if (ta)
    gemm_simt_kernel<T, true, false><<<grid, 256, 0, stream>>>(m, n, k, alpha, A, lda, Bm,
                                                                ldb, beta, C, ldc, uplo);
  else if (tb)
    gemm_simt_kernel<T, false, true><<<grid, 256, 0, stream>>>(m, n, k, alpha, A, lda, Bm,
                                                                ldb, beta, C, ldc, uplo);
  else
    gemm_simt_kernel<T, false, false><<<grid, 256, 0, stream>>>(m, n, k, alpha, A, lda, Bm,
                                                                 ldb, beta, C, ldc, uplo);
  return cudaGetLastError();
}
template cudaError_t launch_gemm_simt<double>(bool, bool, int, int, int, double,
                                              const double*, long, const double*, long,
                                              double, double*, long, int, cudaStream_t);
template cudaError_t launch_gemm_simt<float>(bool, bool, int, int, int, float, const float*,
                                             long, const float*, long, float, float*, long,
                                             int, cudaStream_t);

// ---------------------------------------------------------------------------
// Tall-skinny update for the blocked solves: C[m x q] -= op(A)[m x K] X[K x q]
// ---------------------------------------------------------------------------
constexpr int kTallMaxK = 256, kTallMaxQ = 16;

template <typename T>
__global__ void __launch_bounds__(256)
gemm_tall_sub_kernel(int ta, int m, int q, int K, const T* __restrict__ A, long lda,
                     const T* __restrict__ X, long ldx, T* __restrict__ C, long ldc) {
  __shared__ T sX[kTallMaxK * kTallMaxQ];
  for (int idx = threadIdx.x; idx < K * q; idx += blockDim.x) {
    const int kk = idx % K, c = idx / K;
    sX[kk + c * K] = X[kk + (long)c * ldx];
  }
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  T acc[kTallMaxQ];
#pragma unroll
  for (int c = 0; c < kTallMaxQ; ++c) acc[c] = T(0);
  for (int kk = 0; kk < K; ++kk) {
    const T a = ta ? A[kk + (long)i * lda] : A[i + (long)kk * lda];
#pragma unroll
    for (int c = 0; c < kTallMaxQ; ++c)
      if (c < q) acc[c] = fma(a, sX[kk + c * K], acc[c]);
  }
#pragma unroll
  for (int c = 0; c < kTallMaxQ; ++c)
    if (c < q) C[i + (long)c * ldc] -= acc[c];
}

template <typename T>
cudaError_t launch_gemm_tall_sub(bool ta, int m, int q, int K, const T* A, long lda,
                                 const T* X, long ldx, T* C, long ldc,
                                 cudaStream_t stream) {
  if (m <= 0 || q <= 0 || K <= 0) return cudaSuccess;
  if (K > kTallMaxK || q > kTallMaxQ) return cudaErrorInvalidValue;
  gemm_tall_sub_kernel<T><<<ceil_div(m, 256), 256, 0, stream>>>(ta ? 1 : 0, m, q, K, A, lda,
                                                                X, ldx, C, ldc);
  return cudaGetLastError();
}
template cudaError_t launch_gemm_tall_sub<double>(bool, int, int, int, const double*, long,
                                                  const double*, long, double*, long,
                                                  cudaStream_t);
template cudaError_t launch_gemm_tall_sub<float>(bool, int, int, int, const float*, long,
                                                 const float*, long, float*, long,
                                                 cudaStream_t);

// ---------------------------------------------------------------------------
// K6: Cholesky diagonal block (LowerVariant3Unblocked / UpperVariant3Unblocked)
// ---------------------------------------------------------------------------
// The block (lower triangle, or the transpose of the upper triangle) sits in
// shared memory; per column: sqrt of the pivot, scaling by its reciprocal,
// rank-1 update of the trailing lower triangle.  Only the referenced
// triangle is written back.
template <typename T>
__global__ void __launch_bounds__(256)
potf2_block_kernel(T* __restrict__ A, long lda, int nb, int upper, int info_base,
                   DevStatus* st) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);  // L(i, j) at s[i + j * nb], i >= j
  __shared__ int s_bad;
  const int tid = threadIdx.x;
  for (int idx = tid; idx < nb * nb; idx += blockDim.x) {
    const int i = idx % nb, j = idx / nb;
    if (i >= j) s[idx] = upper ? A[j + (long)i * lda] : A[i + (long)j * lda];
  }
  if (tid == 0) s_bad = 0;
  __syncthreads();
  int done = nb;
  for (int j = 0; j < nb; ++j) {
    T alpha = s[j + j * nb];
    if (!(alpha > T(0)) && !(alpha != alpha)) {  // alpha <= 0 (NaN passes, as in El)
      if (tid == 0) {
        atomicCAS(&st->info, 0, info_base + j + 1);
        s_bad = 1;
      }
      done = j;
      break;
    }
    alpha = sqrt(alpha);
    const T inv = T(1) / alpha;
    __syncthreads();
    if (tid == 0) s[j + j * nb] = alpha;
    for (int i = j + 1 + tid; i < nb; i += blockDim.x) s[i + j * nb] *= inv;
    __syncthreads();
    const int rest = nb - (j + 1);
    for (int idx = tid; idx < rest * rest; idx += blockDim.x) {
      const int ii = idx % rest, cc = idx / rest;
      if (ii >= cc) {
        const int i = j + 1 + ii, c = j + 1 + cc;
        s[i + c * nb] = fma(-s[i + j * nb], s[c + j * nb], s[i + c * nb]);
      }
    }
    __syncthreads();
  }
  (void)done;
  __syncthreads();
  for (int idx = tid; idx < nb * nb; idx += blockDim.x) {
    const int i = idx % nb, j = idx / nb;
    if (i >= j) {
      if (upper)
        A[j + (long)i * lda] = s[idx];
      else
        A[i + (long)j * lda] = s[idx];
    }
  }
}

template <typename T>
cudaError_t launch_potf2_block(T* A, long lda, int nb, bool upper, int info_base,
                               DevStatus* st, cudaStream_t stream) {
  if (nb <= 0) return cudaSuccess;
  if (nb > 128) return cudaErrorInvalidValue;
  const size_t smem = (size_t)nb * nb * sizeof(T);
  auto kern = potf2_block_kernel<T>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
  }
  kern<<<1, 256, smem, stream>>>(A, lda, nb, upper ? 1 : 0, info_base, st);
  return cudaGetLastError();
}
template cudaError_t launch_potf2_block<double>(double*, long, int, bool, int, DevStatus*,
                                                cudaStream_t);
template cudaError_t launch_potf2_block<float>(float*, long, int, bool, int, DevStatus*,
                                               cudaStream_t);

// ---------------------------------------------------------------------------
// K7: FP64 residual R = B - A X, deterministic (fixed-order) reduction
// ---------------------------------------------------------------------------
constexpr int kResChunk = 4096, kResSub = 256, kResMaxQ = 16;

__global__ void __launch_bounds__(256)
residual_partial_kernel(int n, int q, const double* __restrict__ A, long lda,
                        const double* __restrict__ X, long ldx,
                        double* __restrict__ partial) {
  __shared__ double sX[kResSub * kResMaxQ];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int chunk = blockIdx.y;
  const int j0 = chunk * kResChunk, j1 = min(j0 + kResChunk, n);
  double acc[kResMaxQ];
#pragma unroll
  for (int c = 0; c < kResMaxQ; ++c) acc[c] = 0.0;
  for (int js = j0; js < j1; js += kResSub) {
    const int jn = min(kResSub, j1 - js);
    __syncthreads();
    for (int idx = threadIdx.x; idx < jn * q; idx += blockDim.x) {
      const int jj = idx % jn, c = idx / jn;
      sX[jj * kResMaxQ + c] = X[(js + jj) + (long)c * ldx];
    }
    __syncthreads();
    if (i < n) {
      const double* ap = A + i + (long)js * lda;
      int jj = 0;
      for (; jj + 4 <= jn; jj += 4) {
        const double a0 = ap[(long)(jj + 0) * lda];
        const double a1 = ap[(long)(jj + 1) * lda];
        const double a2 = ap[(long)(jj + 2) * lda];
        const double a3 = ap[(long)(jj + 3) * lda];
#pragma unroll
        for (int c = 0; c < kResMaxQ; ++c)
          if (c < q) {
            acc[c] = fma(a0, sX[(jj + 0) * kResMaxQ + c], acc[c]);
            acc[c] = fma(a1, sX[(jj + 1) * kResMaxQ + c], acc[c]);
            acc[c] = fma(a2, sX[(jj + 2) * kResMaxQ + c], acc[c]);
            acc[c] = fma(a3, sX[(jj + 3) * kResMaxQ + c], acc[c]);
          }
      }
      for (; jj < jn; ++jj) {
        const double a0 = ap[(long)jj * lda];
#pragma unroll
        for (int c = 0; c < kResMaxQ; ++c)
          if (c < q) acc[c] = fma(a0, sX[jj * kResMaxQ + c], acc[c]);
      }
    }
  }
  if (i < n)
#pragma unroll
    for (int c = 0; c < kResMaxQ; ++c)
      if (c < q) partial[((long)chunk * q + c) * n + i] = acc[c];
}

__global__ void residual_finish_kernel(int n, int q, int nchunks,
                                       const double* __restrict__ partial,
                                       const double* __restrict__ B, long ldb,
                                       double* __restrict__ R, long ldr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (i >= n) return;
  double s = 0.0;
  for (int ch = 0; ch < nchunks; ++ch) s += partial[((long)ch * q + c) * n + i];
  R[i + (long)c * ldr] = B ? B[i + (long)c * ldb] - s : s;  // B == nullptr: R = A X
}

cudaError_t launch_residual_f64(int n, int q, const double* A, long lda, const double* X,
                                long ldx, const double* B, long ldb, double* R, long ldr,
                                double* partial, cudaStream_t stream) {
  if (n <= 0 || q <= 0) return cudaSuccess;
  if (q > kResMaxQ) return cudaErrorInvalidValue;
  const int nchunks = ceil_div(n, kResChunk);
  residual_partial_kernel<<<dim3(ceil_div(n, 256), nchunks), 256, 0, stream>>>(
      n, q, A, lda, X, ldx, partial);
  residual_finish_kernel<<<dim3(ceil_div(n, 256), q), 256, 0, stream>>>(n, q, nchunks,
                                                                        partial, B, ldb, R,
                                                                        ldr);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Norms for the backward error (deterministic)
// ---------------------------------------------------------------------------
constexpr int kSumsqChunks = 64;

template <typename T>
__global__ void __launch_bounds__(256)
col_sumsq_partial_kernel(const T* __restrict__ A, long lda, int m, int ncols,
                         double* __restrict__ partial) {
  __shared__ double s[256];
  const int c = blockIdx.x, ch = blockIdx.y;
  const int rows_per = ceil_div(m, kSumsqChunks);
  const int r0 = ch * rows_per, r1 = min(r0 + rows_per, m);
  double acc = 0.0;
  for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    const double v = (double)A[r + (long)c * lda];
    acc = fma(v, v, acc);
  }
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[(long)c * kSumsqChunks + ch] = s[0];
}

// Per-column sums (one warp per column, fixed shuffle order), then the total
// over columns by the last block to finish (fixed order, deterministic).
__global__ void col_sumsq_finish_kernel(int ncols, const double* __restrict__ partial,
                                        double* __restrict__ out, unsigned* __restrict__ done) {
  __shared__ bool last;
  const int lane = threadIdx.x & 31;
  const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (c < ncols) {
    double s = partial[(long)c * kSumsqChunks + lane] + partial[(long)c * kSumsqChunks + 32 + lane];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) out[c] = s;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(done, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  __shared__ double red[256];
  double t = 0.0;
  const int per = (ncols + blockDim.x - 1) / blockDim.x;
  for (int i = 0; i < per; ++i) {
    const int cc = threadIdx.x * per + i;
    if (cc < ncols) t += __ldcg(out + cc);
  }
  red[threadIdx.x] = t;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[ncols] = red[0];
    *done = 0;  // ready for the next call
  }
}

template <typename T>
cudaError_t launch_col_sumsq(const T* A, long lda, int m, int ncols, double* out,
                             double* partial, cudaStream_t stream) {
  if (ncols <= 0) return cudaSuccess;
  if (m <= 0) return cudaMemsetAsync(out, 0, sizeof(double) * (ncols + 1), stream);
  col_sumsq_partial_kernel<T><<<dim3(ncols, kSumsqChunks), 256, 0, stream>>>(A, lda, m,
                                                                             ncols, partial);
  // the completion counter lives right after the partial sums
  unsigned* done = reinterpret_cast<unsigned*>(partial + (long)kSumsqChunks * (ncols + 1));
  cudaError_t e = cudaMemsetAsync(done, 0, sizeof(unsigned), stream);
  if (e != cudaSuccess) return e;
  col_sumsq_finish_kernel<<<(ncols + 7) / 8, 256, 0, stream>>>(ncols, partial, out, done);
  return cudaGetLastError();
}
template cudaError_t launch_col_sumsq<double>(const double*, long, int, int, double*,
                                              double*, cudaStream_t);
template cudaError_t launch_col_sumsq<float>(const float*, long, int, int, double*, double*,
                                             cudaStream_t);

// ---------------------------------------------------------------------------
// FP64 FMA-rate probe (the FP64 roofline denominator)
// ---------------------------------------------------------------------------
__global__ void fp64_fma_probe_kernel(double* out, int iters) {
  double a0 = threadIdx.x * 1e-9, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
  double a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
  const double m = 0.999999, c = 1e-7;
  for (int i = 0; i < iters; ++i) {
    a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
    a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
  }
  const double s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == 12345.678) out[0] = s;  // keeps the chains live
}

cudaError_t launch_fp64_fma_probe(double* out, int blocks, int threads, int iters,
                                  cudaStream_t stream) {
  fp64_fma_probe_kernel<<<blocks, threads, 0, stream>>>(out, iters);
  return cudaGetLastError();
}

}  // namespace elgb
