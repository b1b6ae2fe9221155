// Host drivers of the GB300 dense factor-and-solve path and the device-level
// C ABI declared in include/elgb300.h.  The drivers reproduce the blocking
// and the order of operations of the reference's sequential path (cited per
// routine) on top of the kernels in lu_kernels.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <limits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/elgb300.h"
#include "driver.h"
#include "kernels.h"
#include "tc_gemm.h"

namespace elgb {

static int g_blocksize = 128;  // El's default blocksize (src/core/environment.cpp:183)

int to_el_error(cudaError_t e) { return e == cudaSuccess ? kElSuccess : kElRuntimeError; }

cudaEvent_t Context::next_event() {
  if (ev_used == ev_pool.size()) {
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    ev_pool.push_back(e);
  }
  return ev_pool[ev_used++];
}

int Context::prof_begin(cudaStream_t st, int tag) {
  if (!prof_wants(tag)) return -1;
  cudaEvent_t a = next_event();
  if (!a) return -1;
  cudaEventRecord(a, st);
  prof.push_back({a, nullptr, 0, 0, -1});
  return (int)prof.size() - 1;
}

void Context::prof_end(int idx, cudaStream_t st, int tag, double flops, double bytes) {
  if (idx < 0 || !prof_on) return;
  cudaEvent_t b = next_event();
  if (!b) return;
  cudaEventRecord(b, st);
  prof[idx].b = b;
  prof[idx].tag = tag;
  prof[idx].flops = flops;
  prof[idx].bytes = bytes;
  prof[idx].side = st == side_stream && side_stream != nullptr;
  prof[idx].lane = stream_lane(st);
}

Context::~Context() {
  for (cudaEvent_t e : ev_pool) cudaEventDestroy(e);
  if (ev_fork) cudaEventDestroy(ev_fork);
  if (ev_join) cudaEventDestroy(ev_join);
  if (ev_iter) cudaEventDestroy(ev_iter);
  if (ev_swapped) cudaEventDestroy(ev_swapped);
  if (side_stream) cudaStreamDestroy(side_stream);
  if (swap_stream) cudaStreamDestroy(swap_stream);
  if (arena) cudaFree(arena);
  if (arena2) cudaFree(arena2);
  if (trace_buf) cudaFree(trace_buf);
  if (status) cudaFree(status);
  if (h_status) cudaFreeHost(h_status);
  if (own_stream) cudaStreamDestroy(own_stream);
}

cudaError_t Context::ensure(size_t bytes) {
  if (bytes <= arena_bytes) return cudaSuccess;
  cudaError_t e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return e;
  if (arena) cudaFree(arena);
  arena = nullptr;
  arena_bytes = 0;
  // sized exactly: the largest users (an n = 32768 FP32 copy, the refinement
  // vectors) hold gigabytes, and slack would come out of the caller's HBM
  e = cudaMalloc(&arena, bytes);
  if (e != cudaSuccess) return e;
  arena_bytes = bytes;
  return cudaSuccess;
}

cudaError_t Context::ensure2(size_t bytes) {
  if (bytes <= arena2_bytes) return cudaSuccess;
  cudaError_t e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return e;
  if (arena2) cudaFree(arena2);
  arena2 = nullptr;
  arena2_bytes = 0;
  e = cudaMalloc(&arena2, bytes);
  if (e != cudaSuccess) return e;
  arena2_bytes = bytes;
  return cudaSuccess;
}

cudaError_t Context::begin_call() {
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return e;
  return cudaMemsetAsync(status, 0, sizeof(DevStatus), stream);
}

// Bump allocator over the context arena, reset per call.
struct Carver {
  char* base;
  size_t off = 0, cap;
  explicit Carver(Context* c) : base(static_cast<char*>(c->arena)), cap(c->arena_bytes) {}
  template <typename T>
  T* take(size_t count) {
    off = (off + 255) & ~size_t(255);
    T* p = reinterpret_cast<T*>(base + off);
    off += count * sizeof(T);
    return off <= cap ? p : nullptr;
  }
};

static size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

template <typename T>
static size_t panel_scratch_bytes(int maxG) {
  return align256(2 * (size_t)maxG * sizeof(PanelSlot<T>)) +
         align256(calu_scratch_ints(maxG) * sizeof(int));
}
template <typename T>
static PanelScratch<T> carve_panel(Carver& cv, int maxG) {
  PanelScratch<T> s;
  s.slots = cv.take<PanelSlot<T>>(2 * (size_t)maxG);
  s.maxG = maxG;
  s.cand = cv.take<int>(calu_scratch_ints(maxG));
  return s;
}

#define ELGB_CHECK(expr, nk)                   \
  do {                                          \
    cudaError_t e_ = (expr);                    \
    if (e_ != cudaSuccess) return e_;           \
    ctx->launches += (nk);                      \
  } while (0)

// ---------------------------------------------------------------------------
// LU with partial pivoting
// ---------------------------------------------------------------------------
// How the float path's contractions run: SIMT FP32 FMA (tc_kind < 0) or on
// the tensor cores (tc_gemm.cu) with `ws` holding the packed operands.
struct GemmCfg {
  int tc_kind = -1;     // panel-internal and TRSM GEMMs
  int trail_kind = -1;  // the trailing-matrix update (>= 0: overrides tc_kind)
  void* ws = nullptr;
  // the trailing updates' own workspace: a block's three updates (its next
  // block column, the columns beside the panel, the rest) share one L21, so
  // its packed words are made once (what ws_trail holds: trail_a ...)
  void* ws_trail = nullptr;
  mutable const float* trail_a = nullptr;
  mutable long trail_lda = 0;
  mutable int trail_m = 0, trail_k = 0, trail_kind_packed = -1;
};

// One stream of the factorization with the scratch only it touches, so two
// lanes (the trailing update and the look-ahead panel) can run concurrently.
struct LuLane {
  cudaStream_t st = nullptr;
  int* pairs = nullptr;  // 4 * cap ints
  int* pair_count = nullptr;
  GemmCfg gemm;
  // SMs the lane's tensor-core updates may hold (TcGridMode): while the
  // look-ahead panel runs, the trailing update leaves a GPC free for it and
  // the panel's own updates stay small
  int grid_mode = kGridFull;
};

#define LANE_CHECK(expr, nk)                   \
  do {                                          \
    cudaError_t e_ = (expr);                    \
    if (e_ != cudaSuccess) return e_;           \
    ctx->launches += (nk);                      \
  } while (0)

static cudaError_t gemm_sub(Context* ctx, const LuLane& L, int m, int n, int k, const double* A,
                            long lda, const double* B, long ldb, double* C, long ldc,
                            bool trailing = false) {
  (void)trailing;
  const int pi = ctx->prof_begin(L.st, ELGB_PROF_GEMM_SIMT);
  LANE_CHECK(launch_gemm_simt<double>(false, false, m, n, k, -1.0, A, lda, B, ldb, 1.0, C, ldc,
                                      0, L.st), 1);
  ctx->prof_end(pi, L.st, ELGB_PROF_GEMM_SIMT, 2.0 * m * n * (double)k, 24.0 * m * n);
  return cudaSuccess;
}

static cudaError_t gemm_sub(Context* ctx, const LuLane& L, int m, int n, int k, const float* A,
                            long lda, const float* B, long ldb, float* C, long ldc,
                            bool trailing = false) {
  const GemmCfg& g = L.gemm;
  const int kind = (trailing && g.trail_kind >= 0) ? g.trail_kind : g.tc_kind;
  // the look-ahead stream's narrow updates (its recursion's m x n x n) go to
  // the CUDA cores below ctx->opt_side_tc_min_n columns: the tensor-core
  // path's fixed cost (two packing launches and the persistent kernel's
  // set-up) exceeds their work
  const int min_n = (L.st == ctx->side_stream && ctx->side_stream) ? ctx->opt_side_tc_min_n : 64;
  if (kind >= 0 && m >= 64 && n >= min_n && k >= 16) {
    int nl = 0;
    cudaEvent_t a = nullptr, b = nullptr;
    if (ctx->prof_wants(ELGB_PROF_TC_GEMM)) {
      a = ctx->next_event();
      b = ctx->next_event();
    }
    void* ws = g.ws;
    bool a_packed = false;
    const bool reuse = trailing && g.ws_trail && kind != kTcFP8;
    if (reuse) {
      ws = g.ws_trail;
      a_packed = g.trail_a == A && g.trail_lda == lda && g.trail_m == m && g.trail_k == k &&
                 g.trail_kind_packed == kind;
    }
    cudaError_t e = launch_tc_gemm_sub(kind, m, n, k, A, lda, B, ldb, C, ldc, ws, ctx->status,
                                       L.st, &nl, a, b, L.grid_mode, a_packed);
    if (reuse) {
      g.trail_a = e == cudaSuccess ? A : nullptr;
      g.trail_lda = lda;
      g.trail_m = m;
      g.trail_k = k;
      g.trail_kind_packed = kind;
    }
    ctx->launches += nl;
    if (a && b) {
      const double esz = kind == kTcBF16 ? 2.0 : kind == kTcFP8 ? 1.0 : 4.0;
      const double copies = kind == kTcTF32x3 ? 2.0 : 1.0;
      ctx->prof.push_back({a, b, 2.0 * m * n * (double)k,
                           8.0 * m * n + copies * esz * (double)k * (m + n), ELGB_PROF_TC_GEMM,
                           L.st == ctx->side_stream && ctx->side_stream != nullptr,
                           ctx->stream_lane(L.st)});
    }
    return e;
  }
  const int pi = ctx->prof_begin(L.st, ELGB_PROF_GEMM_SIMT);
  LANE_CHECK(launch_gemm_simt<float>(false, false, m, n, k, -1.f, A, lda, B, ldb, 1.f, C, ldc,
                                     0, L.st), 1);
  ctx->prof_end(pi, L.st, ELGB_PROF_GEMM_SIMT, 2.0 * m * n * (double)k, 12.0 * m * n);
  return cudaSuccess;
}

template <typename T>
struct LuState {
  Context* ctx;
  T* A;
  long lda;
  int m, n;
  int* ipiv;           // absolute swap destinations, device
  PanelScratch<T> ps;  // used by whichever lane factors panels
  int panel_ctas;      // CTAs of a panel launch (fewer when it overlaps the update)
  int panel_epoch;     // panel columns published so far (slot epochs)
  LuLane main, side;   // side.st == nullptr: no look-ahead
  LuLane swp;          // interchanges of the trailing update's second part
  T* Bc;               // companion block receiving the same row operations
  long ldbc;           // (RowEchelon's B, src/lapack_like/solve/Linear.cpp:62-71)
  int nbc;
  bool nopiv;          // El::LU(A): no pivot search, no interchanges
  int* dlab;           // deferred left interchanges: labels per block column,
  int* dwork;          //   the labels' scratch
  T* dtmp;             //   and the gather's scratch
  bool tournament;     // FP32 leaf panels by tournament pivoting
  unsigned long long* trace;  // leaf-panel timestamps (4 per column), or null
  int trace_cols;
  int trail_grid;      // TcGridMode of the trailing update beside the look-ahead panel
  bool trail_split;    // the trailing update's columns past the look-ahead panel's
                       // expected end wait for it and take every SM
  double trail_split_scale;  // margin on that expected end
  bool inv_trsm;       // U12 = A12 - N A12 with N = I - L11^{-1} (tensor cores)
  T* ninv;             // N of block ninv_k (nb x nb, leading dimension nb)
  int ninv_ld, ninv_k;
};

// Blocked TRSM, left / lower / unit: B := L11^{-1} B with L11 nb x nb (any
// nb): 128-row diagonal solves plus GEMM updates of the rows below.
template <typename T>
static cudaError_t trsm_llnu(Context* ctx, const LuLane& L, const T* Lm, long ldl, int nb,
                             T* Bm, long ldb, int ncols) {
  if (ncols <= 0) return cudaSuccess;
  for (int i0 = 0; i0 < nb; i0 += 128) {
    const int ib = std::min(128, nb - i0);
    const int pi = ctx->prof_begin(L.st, ELGB_PROF_TRSM);
    LANE_CHECK(launch_trsm_block<T>(Lm + i0 + (long)i0 * ldl, ldl, Bm + i0, ldb, ib, ncols,
                                    true, true, false, false, L.st, ctx->status), 1);
    ctx->prof_end(pi, L.st, ELGB_PROF_TRSM, (double)ib * ib * ncols,
                  2.0 * sizeof(T) * ib * (double)ncols);
    const int rest = nb - i0 - ib;
    if (rest > 0) {
      cudaError_t e = gemm_sub(ctx, L, rest, ncols, ib, Lm + (i0 + ib) + (long)i0 * ldl, ldl,
                               Bm + i0, ldb, Bm + i0 + ib, ldb);
      if (e != cudaSuccess) return e;
    }
  }
  return cudaSuccess;
}

// Row interchanges of the swaps ipiv[c0 .. c0+w) (rows c0.. of A) applied to
// the column ranges [a0, a1) and [b0, b1) of A and, if requested, to the
// companion block.
template <typename T>
static cudaError_t apply_swaps(LuState<T>& s, const LuLane& L, int c0, int w, int a0, int a1,
                               int b0, int b1, bool companion) {
  Context* ctx = s.ctx;
  if (s.nopiv) return cudaSuccess;  // every interchange is the identity
  const int pi = ctx->prof_begin(L.st, ELGB_PROF_SWAP);
  LANE_CHECK(launch_build_swap_pairs(s.ipiv + c0, c0, w, L.pairs, L.pair_count, L.st), 1);
  if ((a1 > a0) || (b1 > b0))
    LANE_CHECK(launch_apply_swap_pairs<T>(s.A, s.lda, a0, a1, b0, b1, L.pairs, L.pair_count, w,
                                          L.st), 1);
  ctx->prof_end(pi, L.st, ELGB_PROF_SWAP, 0.0,
                4.0 * sizeof(T) * w * (double)(std::max(a1 - a0, 0) + std::max(b1 - b0, 0)));
  if (companion && s.Bc && s.nbc > 0)
    LANE_CHECK(launch_apply_swap_pairs<T>(s.Bc, s.ldbc, 0, s.nbc, 0, 0, L.pairs, L.pair_count,
                                          w, L.st), 1);
  return cudaSuccess;
}

// Recursive panel factorization of columns [c0, c0 + w), rows [c0, m), of
// the block panel [b0, b1): left half, TRSM / GEMM onto the right half,
// right half.  Leaves of <= 32 columns (16 on panels taller than 16384
// rows, see leaf_width) go to the getf2 kernels, and each
// leaf's row interchanges go at once onto every other column of the block
// (by the leaf kernel itself where it can, else one swap launch): the same
// row moves, in the same order per column, as swapping each half's
// interchanges onto its sibling after it -- no operation reads those
// columns in between -- with one launch per leaf instead of two per node.
// Leaf width of the block starting at column b0: 16 where the FP32 panel is
// taller than 16384 rows (up to 32768), so that its rows still fit in the
// registers of one 16-CTA cluster (16 columns, 4 rows a thread); else 32.
template <typename T>
static int leaf_width(const LuState<T>& s, int b0) {
  if constexpr (sizeof(T) == 4) {
    if (g_panel_regs == 2 && g_panel_cluster == 16 && !s.nopiv && !s.tournament &&
        s.m - b0 > 16384 && s.m - b0 <= 32768)
      return 16;
  }
  return 32;
}

// Whether gemm_sub runs this m x n x k update on the CUDA cores (the path
// whose arithmetic the fused node update of the register leaf kernel copies).
static bool gemm_sub_is_simt(const Context* ctx, const LuLane& L, int m, int n, int k) {
  const int kind = L.gemm.tc_kind;
  const int min_n = (L.st == ctx->side_stream && ctx->side_stream) ? ctx->opt_side_tc_min_n : 64;
  return !(kind >= 0 && m >= 64 && n >= min_n && k >= 16);
}

// One leaf panel, columns [c0, c0 + w) of the block [b0, b1), its
// interchanges onto the block's other columns; sib_w > 0: the leaf is the
// left child of a node whose right child has sib_w columns, and *node_done
// tells whether the leaf kernel also applied that node's TRSM and update.
template <typename T>
static cudaError_t panel_leaf(LuState<T>& s, const LuLane& L, int c0, int w, int b0, int b1,
                              int sib_w, bool* node_done) {
  Context* ctx = s.ctx;
  if (node_done) *node_done = false;
  const int pi = ctx->prof_begin(L.st, ELGB_PROF_PANEL);
  bool done = false, swapped = false;
  if constexpr (sizeof(T) == 4) {
    if (s.tournament && !s.nopiv) {
      int nl = 0;
      const cudaError_t e = launch_calu_panel(
          reinterpret_cast<float*>(s.A) + c0 + (long)c0 * s.lda, s.lda, s.m - c0, w,
          s.ipiv + c0, c0, c0, s.ps.cand, s.ps.maxG, ctx->status, s.panel_ctas, L.st, &nl);
      ctx->launches += nl;
      if (e == cudaSuccess) done = true;
      else if (e != cudaErrorNotSupported) return e;
    }
  }
  if (!done) {
    PanelScratch<T> ps = s.ps;
    ps.trace = (s.trace && c0 + w <= s.trace_cols) ? s.trace + 4 * (long)c0 : nullptr;
    LANE_CHECK(launch_getf2_panel<T>(s.A + c0 + (long)c0 * s.lda, s.lda, s.m - c0, w,
                                     s.ipiv + c0, c0, c0, s.panel_epoch, ps, ctx->status,
                                     s.panel_ctas, L.st, s.nopiv, b0 - c0, b1 - c0, &swapped,
                                     sib_w, node_done),
               1);
    s.panel_epoch += w;
  }
  ctx->prof_end(pi, L.st, ELGB_PROF_PANEL, (double)(s.m - c0) * w * w,
                2.0 * sizeof(T) * (s.m - c0) * (double)w);
  if (!swapped && (b0 < c0 || c0 + w < b1)) {
    cudaError_t e = apply_swaps(s, L, c0, w, b0, c0, c0 + w, b1, false);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <typename T>
static cudaError_t panel_rec(LuState<T>& s, const LuLane& L, int c0, int w, int b0, int b1) {
  Context* ctx = s.ctx;
  const int lw = leaf_width(s, b0);
  if (w <= lw) return panel_leaf(s, L, c0, w, b0, b1, 0, nullptr);
  int w1 = (w / 2 + lw - 1) / lw * lw;
  if (w1 >= w) w1 = w - lw;
  const int w2 = w - w1;
  // a node of two leaves: the left leaf's kernel may apply the node's TRSM
  // and update itself (when the update would run on the CUDA cores, whose
  // arithmetic it copies)
  const bool two_leaves = w1 <= lw && w2 <= lw && ctx->opt_panel_node;
  bool node_done = false;
  cudaError_t e =
      two_leaves ? panel_leaf(s, L, c0, w1, b0, b1,
                              gemm_sub_is_simt(ctx, L, s.m - c0 - w1, w2, w1) ? w2 : 0,
                              &node_done)
                 : panel_rec(s, L, c0, w1, b0, b1);
  if (e != cudaSuccess) return e;
  if (!node_done) {
    T* A11 = s.A + c0 + (long)c0 * s.lda;
    T* A12 = s.A + c0 + (long)(c0 + w1) * s.lda;
    T* A21 = s.A + (c0 + w1) + (long)c0 * s.lda;
    T* A22 = s.A + (c0 + w1) + (long)(c0 + w1) * s.lda;
    e = trsm_llnu<T>(ctx, L, A11, s.lda, w1, A12, s.lda, w2);
    if (e != cudaSuccess) return e;
    e = gemm_sub(ctx, L, s.m - c0 - w1, w2, w1, A21, s.lda, A12, s.lda, A22, s.lda);
    if (e != cudaSuccess) return e;
  }
  return panel_rec(s, L, c0 + w1, w2, b0, b1);
}

// Trailing update of block k (columns [c_begin, c_end) of the right part):
// Trsm(LEFT, LOWER, NORMAL, UNIT) on A12 then Gemm(-1) on A22.
// U12 := L11^{-1} U12 for block k (jb x ncols at B): one tensor-core product
// U12 - N U12 with N = I - L11^{-1} where gemm_sub takes the tensor cores for
// it (it packs B before C is written, so B may be C), else the blocked
// substitution.  N is strictly lower: L11 N = L11 - I, solved once per block.
template <typename T>
static cudaError_t trsm_block_rows(LuState<T>& s, const LuLane& L, int k, int jb, T* B, long ldb,
                                   int ncols) {
  Context* ctx = s.ctx;
  T* A11 = s.A + k + (long)k * s.lda;
  if (s.inv_trsm && L.gemm.tc_kind >= 0 && jb >= 64 && ncols >= 64) {
    if (s.ninv_k != k) {
      LANE_CHECK(launch_copy_strict_lower<T>(A11, s.lda, jb, s.ninv, s.ninv_ld, L.st), 1);
      cudaError_t e = trsm_llnu<T>(ctx, L, A11, s.lda, jb, s.ninv, s.ninv_ld, jb);
      if (e != cudaSuccess) return e;
      s.ninv_k = k;
    }
    return gemm_sub(ctx, L, jb, ncols, jb, s.ninv, s.ninv_ld, B, ldb, B, ldb);
  }
  return trsm_llnu<T>(ctx, L, A11, s.lda, jb, B, ldb, ncols);
}

template <typename T>
static cudaError_t update_cols(LuState<T>& s, const LuLane& L, int k, int jb, int c_begin,
                               int c_end) {
  if (c_end <= c_begin) return cudaSuccess;
  Context* ctx = s.ctx;
  const int m2 = s.m - k - jb;
  cudaError_t e = trsm_block_rows<T>(s, L, k, jb, s.A + k + (long)c_begin * s.lda, s.lda,
                                     c_end - c_begin);
  if (e != cudaSuccess) return e;
  if (m2 > 0)
    e = gemm_sub(ctx, L, m2, c_end - c_begin, jb, s.A + (k + jb) + (long)k * s.lda, s.lda,
                 s.A + k + (long)c_begin * s.lda, s.lda,
                 s.A + (k + jb) + (long)c_begin * s.lda, s.lda, true);
  return e;
}

template <typename T>
static cudaError_t update_companion(LuState<T>& s, const LuLane& L, int k, int jb) {
  if (!s.Bc || s.nbc <= 0) return cudaSuccess;
  Context* ctx = s.ctx;
  const int m2 = s.m - k - jb;
  cudaError_t e = trsm_block_rows<T>(s, L, k, jb, s.Bc + k, s.ldbc, s.nbc);
  if (e != cudaSuccess || m2 <= 0) return e;
  return gemm_sub(ctx, L, m2, s.nbc, jb, s.A + (k + jb) + (long)k * s.lda, s.lda, s.Bc + k,
                  s.ldbc, s.Bc + k + jb, s.ldbc);
}

// El::LU(A, P) (src/lapack_like/factor/LU.cpp:104-138), right-looking over
// blocks of nb columns: panel, PB.PermuteRows on the left and right blocks,
// Trsm(LEFT, LOWER, NORMAL, UNIT) on A12, Gemm(-1) on A22.
//
// With a side lane the schedule has a look-ahead of one panel: after block
// k's swaps, the block column of panel k+1 is updated first, panel k+1 is
// factored on the side stream while the main stream updates the remaining
// columns, and the two meet before block k+1's swaps.  Every element sees the
// same operations in the same order as without look-ahead.
template <typename T>
static cudaError_t getrf_run(LuState<T>& s, int nb) {
  Context* ctx = s.ctx;
  const int minDim = std::min(s.m, s.n);
  const bool la = s.side.st != nullptr;
  cudaError_t e = cudaSuccess;
  if (minDim == 0) return e;
  e = panel_rec(s, s.main, 0, std::min(nb, minDim), 0, std::min(nb, minDim));
  if (e != cudaSuccess) return e;
  for (int k = 0; k < minDim; k += nb) {
    const int jb = std::min(nb, minDim - k);
    const int kn = k + jb;
    const int jb2 = std::min(nb, std::max(minDim - kn, 0));
    // interchanges right of the panel (left of it, earlier L columns, are
    // deferred to the end); with look-ahead the next panel's block column
    // goes first, so only its share of the swap sits on the critical path
    const bool split = la && jb2 > 0;
    // beside the look-ahead panel the trailing update leaves SMs to it; with
    // trail_split, only the columns it is expected to take while the panel
    // runs, and the rest after the panel on every SM
    int c_mid = s.n;
    if (split && s.trail_split && s.n > kn + jb2) {
      // the panel of jb2 columns on m - kn rows: ~1.5 us per pivot step up
      // to 16384 rows (registers, push exchange), ~2.6 us above, plus ~1 ms
      // of recursion kernels; the update at ~180 TF/s beside it (TF32x3 on
      // all GPCs but one), rounded up to whole 256-column tiles
      const double side_s =
          (jb2 * ((s.m - kn) <= 16384 ? 1.5e-6 : 2.6e-6) + 1.0e-3) * s.trail_split_scale;
      const double cols = side_s * 180e12 / (2.0 * (double)(s.m - kn) * jb);
      const long c = (long)kn + jb2 + ((long)std::ceil(cols / 256.0)) * 256;
      if (c < s.n) c_mid = (int)c;
    }
    // the interchanges of the second part's columns [c_mid, n) on the swap
    // stream, beside everything up to that part (nothing else touches those
    // columns in between; the stream starts after the previous block's
    // update of them)
    const bool swap_apart = c_mid < s.n && s.swp.st != nullptr;
    if (swap_apart) {
      e = cudaEventRecord(ctx->ev_iter, s.main.st);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(s.swp.st, ctx->ev_iter, 0);
      if (e == cudaSuccess) e = apply_swaps(s, s.swp, k, jb, c_mid, s.n, 0, 0, false);
      if (e == cudaSuccess) e = cudaEventRecord(ctx->ev_swapped, s.swp.st);
      if (e != cudaSuccess) return e;
    }
    // interchanges right of the panel (left of it, earlier L columns, are
    // deferred to the end); with look-ahead the next panel's block column
    // goes first, so only its share of the swap sits on the critical path
    e = split ? apply_swaps(s, s.main, k, jb, kn, kn + jb2, 0, 0, false)
              : apply_swaps(s, s.main, k, jb, 0, 0, kn, s.n, true);
    if (e != cudaSuccess) return e;
    if (jb2 > 0) {
      // the next panel's block column first
      e = update_cols(s, s.main, k, jb, kn, kn + jb2);
      if (e != cudaSuccess) return e;
      if (la) {
        e = cudaEventRecord(ctx->ev_fork, s.main.st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s.side.st, ctx->ev_fork, 0);
        if (e == cudaSuccess) e = panel_rec(s, s.side, kn, jb2, kn, kn + jb2);
        if (e == cudaSuccess) e = cudaEventRecord(ctx->ev_join, s.side.st);
        if (e != cudaSuccess) return e;
      }
    }
    if (split) {
      e = apply_swaps(s, s.main, k, jb, kn + jb2, swap_apart ? c_mid : s.n, 0, 0, true);
      if (e != cudaSuccess) return e;
    }
    if (split) s.main.grid_mode = s.trail_grid;
    e = update_cols(s, s.main, k, jb, kn + jb2, c_mid);
    s.main.grid_mode = kGridFull;
    if (e != cudaSuccess) return e;
    if (jb2 > 0) {
      if (la)
        e = cudaStreamWaitEvent(s.main.st, ctx->ev_join, 0);
      else
        e = panel_rec(s, s.main, kn, jb2, kn, kn + jb2);
      if (e != cudaSuccess) return e;
    }
    if (c_mid < s.n) {
      if (swap_apart) e = cudaStreamWaitEvent(s.main.st, ctx->ev_swapped, 0);
      if (e == cudaSuccess) e = update_cols(s, s.main, k, jb, c_mid, s.n);
      if (e != cudaSuccess) return e;
    }
    e = update_companion(s, s.main, k, jb);
    if (e != cudaSuccess) return e;
  }
  if (s.nopiv) return cudaSuccess;
  // every block column of L takes the later panels' interchanges at once
  int pi = ctx->prof_begin(s.main.st, ELGB_PROF_SWAP);
  LANE_CHECK(launch_defer_labels(s.ipiv, s.m, minDim, nb, s.dlab, s.dwork, s.main.st), 2);
  ctx->prof_end(pi, s.main.st, ELGB_PROF_SWAP, 0.0, 0.0);
  pi = ctx->prof_begin(s.main.st, ELGB_PROF_SWAP);
  LANE_CHECK(launch_defer_gather<T>(s.A, s.lda, s.m, minDim, nb, s.dlab, s.dtmp,
                                    defer_gather_grid(ctx->num_sms), s.main.st), 1);
  ctx->prof_end(pi, s.main.st, ELGB_PROF_SWAP, 0.0,
                8.0 * sizeof(T) * 0.5 * (double)s.m * minDim);
  return cudaSuccess;
}

template <typename T>
static size_t getrf_scratch_bytes(const Context* ctx, int nb, int m, int n) {
  const int cap = std::max(nb, 32);
  const size_t nblk = (size_t)(std::min(m, n) + nb - 1) / std::max(nb, 1);
  return panel_scratch_bytes<T>(ctx->num_sms) + 3 * align256(4 * (size_t)cap * sizeof(int)) +
         3 * align256(sizeof(int)) + align256(nblk * (size_t)m * sizeof(int)) +
         align256(defer_labels_work_ints(m, std::min(m, n), nb) * sizeof(int)) +
         align256((size_t)nb * nb * sizeof(T)) +
         align256((size_t)defer_gather_grid(ctx->num_sms) * m * sizeof(T));
}

template <typename T>
static cudaError_t setup_lu_state(Context* ctx, LuState<T>& s, Carver& cv, int nb, int m, int n) {
  const int cap = std::max(nb, 32);
  const size_t nblk = (size_t)(std::min(m, n) + nb - 1) / std::max(nb, 1);
  s.dlab = cv.take<int>(nblk * (size_t)m);
  s.dwork = cv.take<int>(defer_labels_work_ints(m, std::min(m, n), nb));
  s.ninv = cv.take<T>((size_t)nb * nb);
  s.ninv_ld = nb;
  s.ninv_k = -1;
  s.dtmp = cv.take<T>((size_t)defer_gather_grid(ctx->num_sms) * m);
  if (!s.dtmp) return cudaErrorMemoryAllocation;
  s.ctx = ctx;
  s.ps = carve_panel<T>(cv, ctx->num_sms);
  s.panel_ctas = ctx->num_sms;
  s.panel_epoch = 0;
  if (!s.ps.slots) return cudaErrorMemoryAllocation;
  cudaError_t e = cudaMemsetAsync(s.ps.slots, 0, 2 * (size_t)ctx->num_sms * sizeof(PanelSlot<T>),
                                  ctx->stream);
  if (e != cudaSuccess) return e;
  s.main.st = ctx->stream;
  s.main.pairs = cv.take<int>(4 * (size_t)cap);
  s.main.pair_count = cv.take<int>(1);
  s.side.pairs = cv.take<int>(4 * (size_t)cap);
  s.side.pair_count = cv.take<int>(1);
  s.swp.pairs = cv.take<int>(4 * (size_t)cap);
  s.swp.pair_count = cv.take<int>(1);
  if (!s.swp.pair_count) return cudaErrorMemoryAllocation;
  return cudaSuccess;
}

// Look-ahead pays once the trailing update is large enough to hide a panel.
static bool use_lookahead(int m, int n, int nb) { return std::min(m, n) >= 4 * nb && n >= 2048; }

template <typename T>
cudaError_t getrf(Context* ctx, int m, int n, T* A, long lda, int* ipiv, int nb, int tc_kind,
                  bool tournament, bool nopiv) {
  if (nb <= 0) nb = g_blocksize;
  cudaError_t e = ctx->begin_call();
  if (e != cudaSuccess) return e;
  if (m == 0 || n == 0) return cudaSuccess;
  const bool tc = sizeof(T) == 4 && tc_kind >= 0;
  // FP8 serves the trailing update only; the panel's and the TRSM's
  // contractions keep TF32x3 (their operands are the pivoted panel itself)
  const int inner_kind = tc_kind == kTcFP8 ? kTcTF32x3 : tc_kind;
  const bool la = use_lookahead(m, n, nb) && ctx->side_stream && ctx->opt_lookahead;
  const size_t tcb =
      tc ? std::max(tc_gemm_workspace_bytes(tc_kind, m, std::max(n, nb), nb),
                    tc_gemm_workspace_bytes(inner_kind, m, std::max(n, nb), nb))
         : 0;
  const size_t tcs = (tc && la) ? tc_gemm_workspace_bytes(inner_kind, m, nb, nb) : 0;
  e = ctx->ensure(getrf_scratch_bytes<T>(ctx, nb, m, n) + 2 * align256(tcb) + align256(tcs));
  if (e != cudaSuccess) return e;
  Carver cv(ctx);
  LuState<T> s{};
  e = setup_lu_state(ctx, s, cv, nb, m, n);
  if (e != cudaSuccess) return e;
  if (tc) {
    s.main.gemm.tc_kind = inner_kind;
    s.main.gemm.trail_kind = tc_kind;
    s.main.gemm.ws = cv.take<char>(tcb);
    s.main.gemm.ws_trail = cv.take<char>(tcb);
    if (!s.main.gemm.ws_trail) return cudaErrorMemoryAllocation;
  }
  // ELGB_OPT_TRAIL_GRID: 0 every SM (persistent), 1 all GPCs but one, 2
  // (default) the same with the look-ahead stream's updates one CTA per tile,
  // 3 one CTA per tile for both streams.  Measured at n = 32768 (LU ms):
  // 379, 329, 325, 361.
  s.trail_grid = ctx->opt_trail_grid == 0   ? kGridFull
                 : ctx->opt_trail_grid == 3 ? kGridTiles
                                            : kGridSpareGpc;
  s.trail_split = tc && ctx->opt_trail_split && s.trail_grid == kGridSpareGpc;
  s.trail_split_scale = ctx->opt_trail_split > 1 ? ctx->opt_trail_split / 100.0 : 1.1;
  s.inv_trsm = tc && ctx->opt_inv_trsm && s.ninv;
  if (la && ctx->opt_swap_stream) s.swp.st = ctx->swap_stream;
  if (la) {
    s.side.st = ctx->side_stream;
    s.side.grid_mode = ctx->opt_trail_grid >= 2 ? kGridTiles : kGridSmall;
    s.side.gemm.tc_kind = tc ? inner_kind : -1;
    if (tc) {
      s.side.gemm.ws = cv.take<char>(tcs);
      if (!s.side.gemm.ws) return cudaErrorMemoryAllocation;
    }
  }
  if (ctx->opt_panel_ctas > 0) s.panel_ctas = std::min(ctx->opt_panel_ctas, ctx->num_sms);
  s.tournament = tournament && sizeof(T) == 4;
  s.nopiv = nopiv;
  s.trace = ctx->trace_buf;
  s.trace_cols = ctx->trace_cols;
  s.A = A;
  s.lda = lda;
  s.m = m;
  s.n = n;
  s.ipiv = ipiv;
  return getrf_run(s, nb);
}

// ---------------------------------------------------------------------------
// Triangular solves with a few right-hand sides (blocked, 128-row blocks)
// ---------------------------------------------------------------------------
// Solves op(A) X = W in place for W n x q (q <= 16), where op(A) is the
// lower (unit or not) or upper triangle of A, optionally transposed.
template <typename T>
static cudaError_t trsv_blocked(Context* ctx, bool lower_of_A, bool trans, bool unit, int n,
                                const T* A, long lda, T* W, long ldw, int q) {
  constexpr int bs = 128;
  // op(A) is lower when (lower_of_A && !trans) || (!lower_of_A && trans).
  const bool op_lower = lower_of_A != trans;
  const int nblk = (n + bs - 1) / bs;
  for (int b = 0; b < nblk; ++b) {
    const int bi = op_lower ? b : nblk - 1 - b;
    const int i0 = bi * bs, ib = std::min(bs, n - i0);
    const T* Aii = A + i0 + (long)i0 * lda;
    ELGB_CHECK(launch_trsm_block<T>(Aii, lda, W + i0, ldw, ib, q, op_lower, unit, trans,
                                    false, ctx->stream), 1);
    if (op_lower) {
      const int r0 = i0 + ib, rm = n - r0;
      if (rm > 0) {
        // rows below: op(A)(r0.., i0..i0+ib)
        const T* Ab = trans ? A + i0 + (long)r0 * lda : A + r0 + (long)i0 * lda;
        ELGB_CHECK(launch_gemm_tall_sub<T>(trans, rm, q, ib, Ab, lda, W + i0, ldw, W + r0, ldw,
                                           ctx->stream), 1);
      }
    } else {
      if (i0 > 0) {
        // rows above: op(A)(0..i0, i0..i0+ib)
        const T* Ab = trans ? A + i0 : A + (long)i0 * lda;
        ELGB_CHECK(launch_gemm_tall_sub<T>(trans, i0, q, ib, Ab, lda, W + i0, ldw, W, ldw,
                                           ctx->stream), 1);
      }
    }
  }
  return cudaSuccess;
}

template <typename T>
static cudaError_t trsv_any(Context* ctx, bool lower_of_A, bool trans, bool unit, int n,
                            const T* A, long lda, T* W, long ldw, int nrhs) {
  for (int c = 0; c < nrhs; c += 16) {
    cudaError_t e = trsv_blocked<T>(ctx, lower_of_A, trans, unit, n, A, lda,
                                    W + (long)c * ldw, ldw, std::min(16, nrhs - c));
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// op(A) X = W for many right-hand sides, A's lower (unit) or upper
// (non-unit) triangle: 128-row blocks, each a triangular block solve
// (trsm_block_kernel) followed by one GEMM update of the rows still to be
// solved -- level-3 work, where the 16-column TRSV passes of trsv_any would
// re-read A once per 16 columns with ~100 launches each.  The GEMMs run on
// the CUDA cores (FP64 DFMA / FP32 FFMA), as the reference's dtrsm does.
template <typename T>
static cudaError_t trsm_many(Context* ctx, bool lower, bool unit, int n, const T* A, long lda,
                             T* W, long ldw, int nrhs) {
  LuLane L;
  L.st = ctx->stream;
  if (lower) {
    for (int i0 = 0; i0 < n; i0 += 128) {
      const int ib = std::min(128, n - i0);
      ELGB_CHECK(launch_trsm_block<T>(A + i0 + (long)i0 * lda, lda, W + i0, ldw, ib, nrhs, true,
                                      unit, false, false, ctx->stream),
                 1);
      const int rest = n - i0 - ib;
      if (rest > 0) {
        cudaError_t e = gemm_sub(ctx, L, rest, nrhs, ib, A + (i0 + ib) + (long)i0 * lda, lda,
                                 W + i0, ldw, W + i0 + ib, ldw);
        if (e != cudaSuccess) return e;
      }
    }
  } else {
    for (int i0 = ((n - 1) / 128) * 128; i0 >= 0; i0 -= 128) {
      const int ib = std::min(128, n - i0);
      ELGB_CHECK(launch_trsm_block<T>(A + i0 + (long)i0 * lda, lda, W + i0, ldw, ib, nrhs, false,
                                      unit, false, false, ctx->stream),
                 1);
      if (i0 > 0) {
        cudaError_t e = gemm_sub(ctx, L, i0, nrhs, ib, A + (long)i0 * lda, lda, W + i0, ldw, W,
                                 ldw);
        if (e != cudaSuccess) return e;
      }
    }
  }
  return cudaSuccess;
}

// lu::SolveAfter (src/lapack_like/factor/LU/SolveAfter.hpp:66-92).
template <typename T>
cudaError_t getrs(Context* ctx, int orient, int n, const T* A, long lda, const int* ipiv,
                  int nrhs, T* B, long ldb, const int* perm_in) {
  cudaError_t e = ctx->begin_call();
  if (e != cudaSuccess) return e;
  if (n == 0 || nrhs == 0) return cudaSuccess;
  e = ctx->ensure(align256((size_t)n * sizeof(int)) + align256((size_t)n * nrhs * sizeof(T)));
  if (e != cudaSuccess) return e;
  Carver cv(ctx);
  int* perm = cv.take<int>(n);
  T* W = cv.take<T>((size_t)n * nrhs);
  if (!perm || !W) return cudaErrorMemoryAllocation;
  if (perm_in) {
    perm = const_cast<int*>(perm_in);
  } else {
    ELGB_CHECK(launch_explicit_perm(ipiv, n, n, perm, ctx->stream), 1);
  }
  if (orient == 0) {
    ELGB_CHECK(launch_permute_rows<T>(B, ldb, W, n, n, nrhs, perm, false, ctx->stream), 1);
    if (nrhs > 64) {  // many right-hand sides (e.g. El::Inverse's identity)
      e = trsm_many<T>(ctx, true, true, n, A, lda, W, n, nrhs);
      if (e != cudaSuccess) return e;
      e = trsm_many<T>(ctx, false, false, n, A, lda, W, n, nrhs);
      if (e != cudaSuccess) return e;
    } else {
      e = trsv_any<T>(ctx, true, false, true, n, A, lda, W, n, nrhs);
      if (e != cudaSuccess) return e;
      e = trsv_any<T>(ctx, false, false, false, n, A, lda, W, n, nrhs);
      if (e != cudaSuccess) return e;
    }
    e = cudaMemcpy2DAsync(B, ldb * sizeof(T), W, (size_t)n * sizeof(T), (size_t)n * sizeof(T),
                          nrhs, cudaMemcpyDeviceToDevice, ctx->stream);
    if (e != cudaSuccess) return e;
  } else {
    e = cudaMemcpy2DAsync(W, (size_t)n * sizeof(T), B, ldb * sizeof(T), (size_t)n * sizeof(T),
                          nrhs, cudaMemcpyDeviceToDevice, ctx->stream);
    if (e != cudaSuccess) return e;
    e = trsv_any<T>(ctx, false, true, false, n, A, lda, W, n, nrhs);
    if (e != cudaSuccess) return e;
    e = trsv_any<T>(ctx, true, true, true, n, A, lda, W, n, nrhs);
    if (e != cudaSuccess) return e;
    ELGB_CHECK(launch_permute_rows<T>(W, n, B, ldb, n, nrhs, perm, true, ctx->stream), 1);
  }
  return cudaSuccess;
}

// ---------------------------------------------------------------------------
// Cholesky (src/lapack_like/factor/Cholesky.cpp:26-38)
// ---------------------------------------------------------------------------
template <typename T>
cudaError_t potrf(Context* ctx, int uplo, int n, T* A, long lda, int nb) {
  if (nb <= 0) nb = g_blocksize;
  if (nb > 128) nb = 128;
  cudaError_t e = ctx->begin_call();
  if (e != cudaSuccess) return e;
  const bool upper = uplo != 0;
  for (int k = 0; k < n; k += nb) {
    const int jb = std::min(nb, n - k), n2 = n - k - jb;
    T* A11 = A + k + (long)k * lda;
    ELGB_CHECK(launch_potf2_block<T>(A11, lda, jb, upper, k, ctx->status, ctx->stream), 1);
    if (n2 == 0) continue;
    if (!upper) {
      // LowerVariant3Blocked (Cholesky/LowerVariant3.hpp:43-68):
      // Trsm(RIGHT, LOWER, ADJOINT, NON_UNIT) then Herk(LOWER, NORMAL, -1).
      T* A21 = A + (k + jb) + (long)k * lda;
      ELGB_CHECK(launch_trsm_block<T>(A11, lda, A21, lda, jb, n2, true, false, false, true,
                                      ctx->stream), 1);
      ELGB_CHECK(launch_gemm_simt<T>(false, true, n2, n2, jb, T(-1), A21, lda, A21, lda, T(1),
                                     A + (k + jb) + (long)(k + jb) * lda, lda, 1, ctx->stream),
                 1);
    } else {
      // UpperVariant3Blocked (Cholesky/UpperVariant3.hpp:48-73):
      // Trsm(LEFT, UPPER, ADJOINT, NON_UNIT) then Herk(UPPER, ADJOINT, -1).
      T* A12 = A + k + (long)(k + jb) * lda;
      ELGB_CHECK(launch_trsm_block<T>(A11, lda, A12, lda, jb, n2, true, false, true, false,
                                      ctx->stream), 1);
      ELGB_CHECK(launch_gemm_simt<T>(true, false, n2, n2, jb, T(-1), A12, lda, A12, lda, T(1),
                                     A + (k + jb) + (long)(k + jb) * lda, lda, 2, ctx->stream),
                 1);
    }
  }
  return cudaSuccess;
}

// cholesky::SolveAfter(uplo, NORMAL) (Cholesky/SolveAfter.hpp:15-43).
template <typename T>
cudaError_t potrs(Context* ctx, int uplo, int n, const T* A, long lda, int nrhs, T* B,
                  long ldb) {
  cudaError_t e = ctx->begin_call();
  if (e != cudaSuccess) return e;
  if (uplo == 0) {
    e = trsv_any<T>(ctx, true, false, false, n, A, lda, B, ldb, nrhs);
    if (e != cudaSuccess) return e;
    return trsv_any<T>(ctx, true, true, false, n, A, lda, B, ldb, nrhs);
  }
  e = trsv_any<T>(ctx, false, true, false, n, A, lda, B, ldb, nrhs);
  if (e != cudaSuccess) return e;
  return trsv_any<T>(ctx, false, false, false, n, A, lda, B, ldb, nrhs);
}

// El::LinearSolve (src/lapack_like/solve/Linear.cpp:212-218): copy of A,
// RowEchelon on [A | B] (:30-77), then Trsm(LEFT, UPPER, NORMAL, NON_UNIT).
template <typename T>
cudaError_t linear_solve(Context* ctx, int n, const T* A, long lda, int nrhs, T* B, long ldb,
                         int nb) {
  if (nb <= 0) nb = g_blocksize;
  cudaError_t e = ctx->begin_call();
  if (e != cudaSuccess) return e;
  if (n == 0) return cudaSuccess;
  e = ctx->ensure(getrf_scratch_bytes<T>(ctx, nb, n, n) + align256((size_t)n * n * sizeof(T)) +
                  align256((size_t)n * sizeof(int)));
  if (e != cudaSuccess) return e;
  Carver cv(ctx);
  LuState<T> s{};
  e = setup_lu_state(ctx, s, cv, nb, n, n);
  if (e != cudaSuccess) return e;
  T* W = cv.take<T>((size_t)n * n);
  int* ipiv = cv.take<int>(n);
  if (!W || !ipiv) return cudaErrorMemoryAllocation;
  e = cudaMemcpy2DAsync(W, (size_t)n * sizeof(T), A, lda * sizeof(T), (size_t)n * sizeof(T), n,
                        cudaMemcpyDeviceToDevice, ctx->stream);
  if (e != cudaSuccess) return e;
  s.A = W;
  s.lda = n;
  s.m = n;
  s.n = n;
  s.ipiv = ipiv;
  s.Bc = nrhs > 0 ? B : nullptr;
  s.ldbc = ldb;
  s.nbc = nrhs;
  e = getrf_run(s, nb);
  if (e != cudaSuccess) return e;
  return trsv_any<T>(ctx, false, false, false, n, W, n, B, ldb, nrhs);
}

// El::HPDSolve (src/lapack_like/solve/HPD.cpp:47-55).
template <typename T>
cudaError_t hpd_solve(Context* ctx, int uplo, int n, const T* A, long lda, int nrhs, T* B,
                      long ldb, int nb) {
  cudaError_t e = ctx->begin_call();
  if (e != cudaSuccess) return e;
  if (n == 0) return cudaSuccess;
  e = ctx->ensure(align256((size_t)n * n * sizeof(T)));
  if (e != cudaSuccess) return e;
  Carver cv(ctx);
  T* W = cv.take<T>((size_t)n * n);
  if (!W) return cudaErrorMemoryAllocation;
  e = cudaMemcpy2DAsync(W, (size_t)n * sizeof(T), A, lda * sizeof(T), (size_t)n * sizeof(T), n,
                        cudaMemcpyDeviceToDevice, ctx->stream);
  if (e != cudaSuccess) return e;
  e = potrf<T>(ctx, uplo, n, W, n, nb);
  if (e != cudaSuccess) return e;
  if (uplo == 0) {
    e = trsv_any<T>(ctx, true, false, false, n, W, n, B, ldb, nrhs);
    if (e != cudaSuccess) return e;
    return trsv_any<T>(ctx, true, true, false, n, W, n, B, ldb, nrhs);
  }
  e = trsv_any<T>(ctx, false, true, false, n, W, n, B, ldb, nrhs);
  if (e != cudaSuccess) return e;
  return trsv_any<T>(ctx, false, false, false, n, W, n, B, ldb, nrhs);
}

cudaError_t residual(Context* ctx, int n, int q, const double* A, long lda, const double* X,
                     long ldx, const double* B, long ldb, double* R, long ldr) {
  if (n == 0 || q == 0) return cudaSuccess;
  const int nchunks = (n + 4095) / 4096;
  for (int c = 0; c < q; c += 16) {
    const int qc = std::min(16, q - c);
    cudaError_t e = ctx->ensure(align256((size_t)nchunks * n * 16 * sizeof(double)));
    if (e != cudaSuccess) return e;
    Carver cv(ctx);
    double* partial = cv.take<double>((size_t)nchunks * n * 16);
    if (!partial) return cudaErrorMemoryAllocation;
    ELGB_CHECK(launch_residual_f64(n, qc, A, lda, X + (long)c * ldx, ldx, B + (long)c * ldb,
                                   ldb, R + (long)c * ldr, ldr, partial, ctx->stream), 2);
  }
  return cudaSuccess;
}

cudaError_t backward_error(Context* ctx, int n, int q, const double* A, long lda,
                           const double* X, long ldx, const double* B, long ldb,
                           double* berr) {
  const size_t need = align256((size_t)n * q * sizeof(double)) +
                      align256((size_t)(n + 2) * sizeof(double)) +
                      3 * align256((size_t)(q + 2) * sizeof(double)) +
                      align256(((size_t)64 * (std::max(n, q) + 1) + 8) * sizeof(double)) +
                      align256((size_t)((n + 4095) / 4096) * n * 16 * sizeof(double));
  cudaError_t e = ctx->ensure(need);
  if (e != cudaSuccess) return e;
  Carver cv(ctx);
  double* R = cv.take<double>((size_t)n * q);
  double* nA = cv.take<double>(n + 2);
  double* nX = cv.take<double>(q + 2);
  double* nR = cv.take<double>(q + 2);
  double* nB = cv.take<double>(q + 2);
  double* partial = cv.take<double>((size_t)64 * (std::max(n, q) + 1) + 8);
  double* rpart = cv.take<double>((size_t)((n + 4095) / 4096) * n * 16);
  if (!R || !nA || !nX || !nR || !nB || !partial || !rpart) return cudaErrorMemoryAllocation;
  for (int c = 0; c < q; c += 16) {
    const int qc = std::min(16, q - c);
    ELGB_CHECK(launch_residual_f64(n, qc, A, lda, X + (long)c * ldx, ldx, B + (long)c * ldb,
                                   ldb, R + (long)c * n, n, rpart, ctx->stream), 2);
  }
  ELGB_CHECK(launch_col_sumsq<double>(A, lda, n, n, nA, partial, ctx->stream), 2);
  ELGB_CHECK(launch_col_sumsq<double>(X, ldx, n, q, nX, partial, ctx->stream), 2);
  ELGB_CHECK(launch_col_sumsq<double>(B, ldb, n, q, nB, partial, ctx->stream), 2);
  ELGB_CHECK(launch_col_sumsq<double>(R, n, n, q, nR, partial, ctx->stream), 2);
  std::vector<double> hx(q + 1), hb(q + 1), hr(q + 1);
  double hA[1];
  e = cudaMemcpyAsync(hA, nA + n, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  if (e != cudaSuccess) return e;
  e = cudaMemcpyAsync(hx.data(), nX, (q + 1) * sizeof(double), cudaMemcpyDeviceToHost,
                      ctx->stream);
  if (e != cudaSuccess) return e;
  e = cudaMemcpyAsync(hb.data(), nB, (q + 1) * sizeof(double), cudaMemcpyDeviceToHost,
                      ctx->stream);
  if (e != cudaSuccess) return e;
  e = cudaMemcpyAsync(hr.data(), nR, (q + 1) * sizeof(double), cudaMemcpyDeviceToHost,
                      ctx->stream);
  if (e != cudaSuccess) return e;
  e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return e;
  const double fa = std::sqrt(hA[0]);
  double worst = 0.0;
  for (int c = 0; c < q; ++c) {
    const double den = fa * std::sqrt(hx[c]) + std::sqrt(hb[c]);
    const double v = den > 0 ? std::sqrt(hr[c]) / den : (hr[c] > 0 ? INFINITY : 0.0);
    if (!(v <= worst)) worst = v;
  }
  *berr = worst;
  return cudaSuccess;
}

// ---------------------------------------------------------------------------
// El::Inverse and El::OneCondition
// ---------------------------------------------------------------------------
// max_j sum_i |A(i, j)|: one warp per column; the non-negative FP64 maxima
// order like their bit patterns, so an integer atomicMax combines them.
template <typename T>
__global__ void col_abs_sum_max_kernel(const T* __restrict__ A, long lda, int m, int n,
                                       unsigned long long* out) {
  const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  double best = 0.0;
  for (int j = blockIdx.x * wpb + (threadIdx.x >> 5); j < n; j += gridDim.x * wpb) {
    double sum = 0.0;
    for (int i = lane; i < m; i += 32) sum += fabs((double)A[i + (long)j * lda]);
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    best = fmax(best, sum);
  }
  if (lane == 0) atomicMax(out, (unsigned long long)__double_as_longlong(best));
}

template <typename T>
__global__ void set_identity_kernel(T* X, long ldx, int n) {
  for (int j = blockIdx.y; j < n; j += gridDim.y)
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
      X[i + (long)j * ldx] = i == j ? T(1) : T(0);
}

// One-norm of an m x n device matrix (synchronizes); tmp: one device word.
template <typename T>
static cudaError_t one_norm(Context* ctx, int m, int n, const T* A, long lda,
                            unsigned long long* tmp, double* out) {
  cudaError_t e = cudaMemsetAsync(tmp, 0, sizeof(unsigned long long), ctx->stream);
  if (e != cudaSuccess) return e;
  const int blocks = std::max(1, std::min(ceil_div(n, 8), 4 * ctx->num_sms));
  col_abs_sum_max_kernel<T><<<blocks, 256, 0, ctx->stream>>>(A, lda, m, n, tmp);
  ctx->launches += 1;
  unsigned long long h = 0;
  e = cudaMemcpyAsync(&h, tmp, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  double v;
  std::memcpy(&v, &h, sizeof(v));
  *out = v;
  return e;
}

// Reads the device status word (synchronizes).
static cudaError_t read_status(Context* ctx, int* info, int* err) {
  cudaError_t e = cudaMemcpyAsync(ctx->h_status, ctx->status, sizeof(DevStatus),
                                  cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  *info = ctx->h_status->info;
  *err = ctx->h_status->err;
  return e;
}

// inv(A) = inv(U) inv(L) P (funcs/Inverse/General/LUPartialPiv.hpp:21-62),
// formed as the solve of P A X = I by getrs on the factors: the same
// operator, column by column.  ipiv: n ints; X: n x n scratch.  With a zero
// pivot the status word keeps getrf's info and A holds the partial factors
// (the reference throws SingularMatrixException from El::LU).
template <typename T>
static cudaError_t getri_impl(Context* ctx, int n, T* A, long lda, int nb, int* ipiv, T* X) {
  cudaError_t e = getrf<T>(ctx, n, n, A, lda, ipiv, nb);
  if (e != cudaSuccess) return e;
  int info = 0, err = 0;
  e = read_status(ctx, &info, &err);
  if (e != cudaSuccess || info || err) return e;
  set_identity_kernel<T><<<dim3(ceil_div(n, 256), grid_y(n)), 256, 0, ctx->stream>>>(X, n, n);
  ctx->launches += 1;
  e = getrs<T>(ctx, 0, n, A, lda, ipiv, n, X, n, nullptr);
  if (e != cudaSuccess) return e;
  return cudaMemcpy2DAsync(A, lda * sizeof(T), X, (size_t)n * sizeof(T), (size_t)n * sizeof(T),
                           n, cudaMemcpyDeviceToDevice, ctx->stream);
}

template <typename T>
cudaError_t getri(Context* ctx, int n, T* A, long lda, int nb) {
  if (n == 0) return ctx->begin_call();
  cudaError_t e = ctx->ensure2(align256((size_t)n * sizeof(int)) +
                               align256((size_t)n * n * sizeof(T)));
  if (e != cudaSuccess) return e;
  char* p = static_cast<char*>(ctx->arena2);
  int* ipiv = reinterpret_cast<int*>(p);
  T* X = reinterpret_cast<T*>(p + align256((size_t)n * sizeof(int)));
  return getri_impl<T>(ctx, n, A, lda, nb, ipiv, X);
}

template <typename T>
cudaError_t one_condition(Context* ctx, int n, const T* A, long lda, int nb, double* cond) {
  cudaError_t e = ctx->begin_call();
  if (e != cudaSuccess) return e;
  if (n == 0) {
    *cond = 0.0;
    return cudaSuccess;
  }
  const size_t sm = align256((size_t)n * n * sizeof(T));
  e = ctx->ensure2(2 * sm + align256((size_t)n * sizeof(int)) + 256);
  if (e != cudaSuccess) return e;
  char* p = static_cast<char*>(ctx->arena2);
  T* B = reinterpret_cast<T*>(p);
  T* X = reinterpret_cast<T*>(p + sm);
  int* ipiv = reinterpret_cast<int*>(p + 2 * sm);
  auto* tmp = reinterpret_cast<unsigned long long*>(p + 2 * sm + align256((size_t)n * sizeof(int)));
  // Matrix<Field> B( A ); oneNorm = OneNorm( B ); Inverse( B ) (One.cpp:16-19)
  e = cudaMemcpy2DAsync(B, (size_t)n * sizeof(T), A, lda * sizeof(T), (size_t)n * sizeof(T), n,
                        cudaMemcpyDeviceToDevice, ctx->stream);
  double n1 = 0.0, n1inv = 0.0;
  if (e == cudaSuccess) e = one_norm<T>(ctx, n, n, B, n, tmp, &n1);
  if (e == cudaSuccess) e = getri_impl<T>(ctx, n, B, n, nb, ipiv, X);
  if (e != cudaSuccess) return e;
  int info = 0, err = 0;
  e = read_status(ctx, &info, &err);
  if (e != cudaSuccess) return e;
  if (err) return cudaErrorLaunchTimeout;
  if (info) {  // SingularMatrixException -> +inf (One.cpp:20-21), not an error
    *cond = std::numeric_limits<double>::infinity();
    return cudaMemsetAsync(ctx->status, 0, sizeof(DevStatus), ctx->stream);
  }
  e = one_norm<T>(ctx, n, n, B, n, tmp, &n1inv);
  *cond = n1 * n1inv;
  return e;
}

// El::LU(A, P, Q) with full pivoting (src/lapack_like/factor/LU/Full.hpp).
template <typename T>
cudaError_t getrf_full(Context* ctx, int m, int n, T* A, long lda, int* p, int* q) {
  cudaError_t e = ctx->begin_call();
  if (e != cudaSuccess || std::min(m, n) == 0) return e;
  const int grid = fullpiv_grid(ctx->num_sms);
  e = ctx->ensure(align256(sizeof(FullPivState<T>)) +
                  align256((size_t)grid * sizeof(FullPivCand<T>)));
  if (e != cudaSuccess) return e;
  Carver cv(ctx);
  auto* fs = cv.take<FullPivState<T>>(1);
  auto* part = cv.take<FullPivCand<T>>(grid);
  if (!fs || !part) return cudaErrorMemoryAllocation;
  return launch_lu_full<T>(A, lda, m, n, p, q, fs, part, grid, ctx->status, ctx->stream,
                           &ctx->launches);
}

// lu::SolveAfter(orientation, A, P, Q, B) (LU/SolveAfter.hpp:120-145):
// NORMAL = P, L, U as getrs, then Q.InversePermuteRows(B); TRANSPOSE /
// ADJOINT = Q.PermuteRows(B), then getrs's U^T, L^T and P^-1.
template <typename T>
cudaError_t getrs_full(Context* ctx, int orient, int n, const T* A, long lda, const int* p,
                       const int* q, int nrhs, T* B, long ldb) {
  if (n == 0 || nrhs == 0) return ctx->begin_call();
  auto permute_q = [&](bool inverse) -> cudaError_t {
    cudaError_t e = ctx->ensure(align256((size_t)n * sizeof(int)) +
                                align256((size_t)n * nrhs * sizeof(T)));
    if (e != cudaSuccess) return e;
    Carver cv(ctx);
    int* perm = cv.take<int>(n);
    T* W = cv.take<T>((size_t)n * nrhs);
    if (!perm || !W) return cudaErrorMemoryAllocation;
    ELGB_CHECK(launch_explicit_perm(q, n, n, perm, ctx->stream), 1);
    ELGB_CHECK(launch_permute_rows<T>(B, ldb, W, n, n, nrhs, perm, inverse, ctx->stream), 1);
    return cudaMemcpy2DAsync(B, ldb * sizeof(T), W, (size_t)n * sizeof(T), (size_t)n * sizeof(T),
                             nrhs, cudaMemcpyDeviceToDevice, ctx->stream);
  };
  cudaError_t e;
  if (orient == 0) {
    e = getrs<T>(ctx, 0, n, A, lda, p, nrhs, B, ldb, nullptr);
    if (e == cudaSuccess) e = permute_q(true);
  } else {
    e = ctx->begin_call();
    if (e == cudaSuccess) e = permute_q(false);
    if (e == cudaSuccess) e = getrs<T>(ctx, orient, n, A, lda, p, nrhs, B, ldb, nullptr);
  }
  return e;
}

// El::Cholesky(uplo, A, P) with diagonal pivoting (Cholesky.cpp:44-52).
template <typename T>
cudaError_t potrf_piv(Context* ctx, int uplo, int n, T* A, long lda, int* piv) {
  cudaError_t e = ctx->begin_call();
  if (e != cudaSuccess || n == 0) return e;
  const int grid = fullpiv_grid(ctx->num_sms);
  e = ctx->ensure(align256(sizeof(FullPivState<T>)) +
                  align256((size_t)grid * sizeof(FullPivCand<T>)));
  if (e != cudaSuccess) return e;
  Carver cv(ctx);
  auto* fs = cv.take<FullPivState<T>>(1);
  auto* part = cv.take<FullPivCand<T>>(grid);
  if (!fs || !part) return cudaErrorMemoryAllocation;
  return launch_cholesky_piv<T>(A, lda, n, uplo == 1, piv, fs, part, grid, ctx->stream,
                                &ctx->launches);
}

// cholesky::SolveAfter(uplo, orientation, A, P, B) on real data
// (Cholesky/SolveAfter.hpp:46-76): P.PermuteRows(B), the Cholesky solve,
// P.InversePermuteRows(B).
template <typename T>
cudaError_t potrs_piv(Context* ctx, int uplo, int n, const T* A, long lda, const int* piv,
                      int nrhs, T* B, long ldb) {
  if (n == 0 || nrhs == 0) return ctx->begin_call();
  auto permute = [&](bool inverse) -> cudaError_t {
    cudaError_t e = ctx->ensure(align256((size_t)n * sizeof(int)) +
                                align256((size_t)n * nrhs * sizeof(T)));
    if (e != cudaSuccess) return e;
    Carver cv(ctx);
    int* perm = cv.take<int>(n);
    T* W = cv.take<T>((size_t)n * nrhs);
    if (!perm || !W) return cudaErrorMemoryAllocation;
    ELGB_CHECK(launch_explicit_perm(piv, n, n, perm, ctx->stream), 1);
    ELGB_CHECK(launch_permute_rows<T>(B, ldb, W, n, n, nrhs, perm, inverse, ctx->stream), 1);
    return cudaMemcpy2DAsync(B, ldb * sizeof(T), W, (size_t)n * sizeof(T), (size_t)n * sizeof(T),
                             nrhs, cudaMemcpyDeviceToDevice, ctx->stream);
  };
  cudaError_t e = ctx->begin_call();
  if (e == cudaSuccess) e = permute(false);
  if (e == cudaSuccess) e = potrs<T>(ctx, uplo, n, A, lda, nrhs, B, ldb);
  if (e == cudaSuccess) e = permute(true);
  return e;
}

template cudaError_t potrf_piv<double>(Context*, int, int, double*, long, int*);
template cudaError_t potrf_piv<float>(Context*, int, int, float*, long, int*);
template cudaError_t potrs_piv<double>(Context*, int, int, const double*, long, const int*,
                                       int, double*, long);
template cudaError_t potrs_piv<float>(Context*, int, int, const float*, long, const int*, int,
                                      float*, long);
template cudaError_t getrf_full<double>(Context*, int, int, double*, long, int*, int*);
template cudaError_t getrf_full<float>(Context*, int, int, float*, long, int*, int*);
template cudaError_t getrs_full<double>(Context*, int, int, const double*, long, const int*,
                                        const int*, int, double*, long);
template cudaError_t getrs_full<float>(Context*, int, int, const float*, long, const int*,
                                       const int*, int, float*, long);
template cudaError_t getri<double>(Context*, int, double*, long, int);
template cudaError_t getri<float>(Context*, int, float*, long, int);
template cudaError_t one_condition<double>(Context*, int, const double*, long, int, double*);
template cudaError_t one_condition<float>(Context*, int, const float*, long, int, double*);

template cudaError_t getrf<double>(Context*, int, int, double*, long, int*, int, int, bool,
                                   bool);
template cudaError_t getrf<float>(Context*, int, int, float*, long, int*, int, int, bool, bool);
template cudaError_t getrs<double>(Context*, int, int, const double*, long, const int*, int,
                                   double*, long, const int*);
template cudaError_t getrs<float>(Context*, int, int, const float*, long, const int*, int,
                                  float*, long, const int*);
template cudaError_t potrf<double>(Context*, int, int, double*, long, int);
template cudaError_t potrf<float>(Context*, int, int, float*, long, int);
template cudaError_t potrs<double>(Context*, int, int, const double*, long, int, double*,
                                   long);
template cudaError_t potrs<float>(Context*, int, int, const float*, long, int, float*, long);

int get_blocksize() { return g_blocksize; }
void set_blocksize(int nb) { g_blocksize = nb; }

}  // namespace elgb

// ===========================================================================
// C ABI (include/elgb300.h)
// ===========================================================================
using elgb::Context;

static int arg_ok(bool c) { return c ? 0 : elgb::kElArgError; }

extern "C" {

int ElGBCreate(ElGBContext* out, int device) {
  if (!out) return elgb::kElArgError;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
    return elgb::kElRuntimeError;
  auto* c = new (std::nothrow) ElGBContextImpl();
  if (!c) return elgb::kElAllocError;
  c->device = device;
  int least_prio = 0, greatest_prio = 0;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device) !=
          cudaSuccess ||
      cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
      // the look-ahead panel's stream at the highest priority: its small,
      // latency-bound kernels (leaf panels, the panel's own interchanges,
      // TRSMs) are the critical path and must not queue behind the trailing
      // update's thousands of tensor-core CTAs on the other stream
      cudaDeviceGetStreamPriorityRange(&least_prio, &greatest_prio) != cudaSuccess ||
      cudaStreamCreateWithPriority(&c->side_stream, cudaStreamNonBlocking, greatest_prio) !=
          cudaSuccess ||
      // the deferred share of a block's interchanges at the lowest priority:
      // it only has to finish before the trailing update's second part
      cudaStreamCreateWithPriority(&c->swap_stream, cudaStreamNonBlocking, least_prio) !=
          cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_iter, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_swapped, cudaEventDisableTiming) != cudaSuccess ||
      cudaMalloc(&c->status, sizeof(elgb::DevStatus)) != cudaSuccess ||
      cudaMallocHost(&c->h_status, sizeof(elgb::DevStatus)) != cudaSuccess ||
      // zeroed on the legacy stream, which the context's non-blocking
      // streams do not wait for: drained before the first launch
      cudaMemset(c->status, 0, sizeof(elgb::DevStatus)) != cudaSuccess ||
      cudaStreamSynchronize(cudaStreamLegacy) != cudaSuccess) {
    delete c;
    return elgb::kElRuntimeError;
  }
  c->stream = c->own_stream;
  *out = c;
  return 0;
}

int ElGBDestroy(ElGBContext ctx) {
  if (!ctx) return elgb::kElArgError;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  delete ctx;
  return 0;
}

int ElGBSetStream(ElGBContext ctx, void* stream) {
  if (!ctx) return elgb::kElArgError;
  ctx->stream = static_cast<cudaStream_t>(stream);  // NULL: the legacy default stream
  return 0;
}

int ElGBSynchronize(ElGBContext ctx) {
  if (!ctx) return elgb::kElArgError;
  return elgb::to_el_error(cudaStreamSynchronize(ctx->stream));
}

int ElGBStatus(ElGBContext ctx, int* info, int* err) {
  if (!ctx) return elgb::kElArgError;
  cudaError_t e = cudaMemcpyAsync(ctx->h_status, ctx->status, sizeof(elgb::DevStatus),
                                  cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return elgb::kElRuntimeError;
  if (info) *info = ctx->h_status->info;
  if (err) *err = ctx->h_status->err;
  return 0;
}

int ElGBProfileStart(ElGBContext ctx) { return ElGBProfileStartTags(ctx, ~0u); }

int ElGBProfileStartTags(ElGBContext ctx, unsigned tags) {
  if (!ctx) return elgb::kElArgError;
  ctx->prof.clear();
  ctx->ev_used = 0;
  ctx->prof_mask = tags;
  ctx->prof_on = true;
  return 0;
}

int ElGBProfileStop(ElGBContext ctx, long long* launches, double* ms, double* flops,
                    double* bytes) {
  if (!ctx) return elgb::kElArgError;
  ctx->prof_on = false;
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return elgb::kElRuntimeError;
  for (auto& ps : ctx->prof_sum) ps = Context::ProfSum();
  for (auto& r : ctx->prof) {
    if (!r.b || r.tag < 0 || r.tag >= 16) continue;
    float x = 0;
    if (cudaEventElapsedTime(&x, r.a, r.b) != cudaSuccess) return elgb::kElRuntimeError;
    for (int t : {r.tag, r.side && r.tag < 8 ? r.tag + 8 : -1}) {
      if (t < 0) continue;
      auto& ps = ctx->prof_sum[t];
      ps.launches += 1;
      ps.ms += x;
      ps.flops += r.flops;
      ps.bytes += r.bytes;
    }
  }
  const auto& g = ctx->prof_sum[ELGB_PROF_TC_GEMM];
  const double t = g.ms, f = g.flops, b = g.bytes;
  if (launches) *launches = g.launches;
  if (ms) *ms = t;
  if (flops) *flops = f;
  if (bytes) *bytes = b;
  return 0;
}

int ElGBProfileTag(ElGBContext ctx, int tag, long long* launches, double* ms, double* flops,
                   double* bytes) {
  if (!ctx || tag < 0 || tag >= 16) return elgb::kElArgError;
  const auto& g = ctx->prof_sum[tag];
  if (launches) *launches = g.launches;
  if (ms) *ms = g.ms;
  if (flops) *flops = g.flops;
  if (bytes) *bytes = g.bytes;
  return 0;
}

int ElGBProfileRecords(ElGBContext ctx, int cap, int* count, float* start_ms, float* dur_ms,
                       int* tag, int* side) {
  if (!ctx || !count || cap < 0 || (cap > 0 && (!start_ms || !dur_ms || !tag || !side)))
    return elgb::kElArgError;
  if (ctx->prof_on) return elgb::kElLogicError;
  int n = 0;
  cudaEvent_t base = nullptr;
  for (auto& r : ctx->prof) {
    if (!r.a || !r.b || r.tag < 0 || r.tag >= 16) continue;
    if (!base) base = r.a;
    if (n < cap) {
      float t0 = 0, d = 0;
      if (cudaEventElapsedTime(&t0, base, r.a) != cudaSuccess ||
          cudaEventElapsedTime(&d, r.a, r.b) != cudaSuccess)
        return elgb::kElRuntimeError;
      start_ms[n] = t0;
      dur_ms[n] = d;
      tag[n] = r.tag;
      side[n] = r.lane;
    }
    ++n;
  }
  *count = n;
  return 0;
}

int ElGBSetOption(ElGBContext ctx, int option, int value) {
  if (!ctx) return elgb::kElArgError;
  switch (option) {
    case ELGB_OPT_LOOKAHEAD:
      ctx->opt_lookahead = value ? 1 : 0;
      return 0;
    case ELGB_OPT_PANEL_CTAS:
      if (value < 0) return elgb::kElArgError;
      ctx->opt_panel_ctas = value;
      return 0;
    case ELGB_OPT_TOURNAMENT:
      ctx->opt_tournament = value ? 1 : 0;
      return 0;
    case ELGB_OPT_PANEL_CLUSTER:
      if (value != 1 && value != 2 && value != 4 && value != 8 && value != 16)
        return elgb::kElArgError;
      elgb::g_panel_cluster = value;
      return 0;
    case ELGB_OPT_PANEL_REGS:
      if (value < 0 || value > 2) return elgb::kElArgError;
      elgb::g_panel_regs = value;
      return 0;
    case ELGB_OPT_RESIDUAL_DF:
      ctx->opt_residual_df = value ? 1 : 0;
      return 0;
    case ELGB_OPT_TRAIL_GRID:
      if (value < 0 || value > 3) return elgb::kElArgError;
      ctx->opt_trail_grid = value;
      return 0;
    case ELGB_OPT_TRAIL_SPLIT:
      if (value < 0 || value > 1000) return elgb::kElArgError;
      ctx->opt_trail_split = value;
      return 0;
    case ELGB_OPT_INV_TRSM:
      ctx->opt_inv_trsm = value ? 1 : 0;
      return 0;
    case ELGB_OPT_SWAP_STREAM:
      ctx->opt_swap_stream = value ? 1 : 0;
      return 0;
    case ELGB_OPT_PANEL_NODE:
      ctx->opt_panel_node = value ? 1 : 0;
      return 0;
    case ELGB_OPT_SIDE_TC_MIN_N:
      if (value < 16 || value > 4096) return elgb::kElArgError;
      ctx->opt_side_tc_min_n = value;
      return 0;
    case ELGB_OPT_PANEL_PDL:
      elgb::g_panel_pdl = value ? 1 : 0;
      return 0;
    case ELGB_OPT_PANEL_PUSH:
      if (value < 0 || value > 2) return elgb::kElArgError;
      elgb::g_panel_push = value;
      return 0;
    case ELGB_OPT_PANEL_ROWS:
      if (value < 64 || value > 1536) return elgb::kElArgError;
      elgb::g_panel_rows = value;
      return 0;
    case ELGB_OPT_PANEL_TRACE: {
      if (value < 0) return elgb::kElArgError;
      cudaSetDevice(ctx->device);
      if (ctx->trace_buf) cudaFree(ctx->trace_buf);
      ctx->trace_buf = nullptr;
      ctx->trace_cols = 0;
      if (value > 0) {
        const size_t bytes = 4 * (size_t)value * sizeof(unsigned long long);
        if (cudaMalloc(&ctx->trace_buf, bytes) != cudaSuccess) return elgb::kElAllocError;
        if (cudaMemset(ctx->trace_buf, 0, bytes) != cudaSuccess) return elgb::kElRuntimeError;
        ctx->trace_cols = value;
      }
      return 0;
    }
    default:
      return elgb::kElArgError;
  }
}

int ElGBPanelTrace(ElGBContext ctx, unsigned long long* out, int ncols) {
  if (!ctx || !out || ncols < 0 || ncols > ctx->trace_cols) return elgb::kElArgError;
  if (ncols == 0) return 0;
  cudaSetDevice(ctx->device);
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return elgb::kElRuntimeError;
  if (ctx->side_stream && cudaStreamSynchronize(ctx->side_stream) != cudaSuccess)
    return elgb::kElRuntimeError;
  return cudaMemcpy(out, ctx->trace_buf, 4 * (size_t)ncols * sizeof(unsigned long long),
                    cudaMemcpyDeviceToHost) == cudaSuccess
             ? 0
             : elgb::kElRuntimeError;
}

int ElGBBlocksize(void) { return elgb::get_blocksize(); }
int ElGBSetBlocksize(int nb) {
  if (nb < 1) return elgb::kElArgError;
  elgb::set_blocksize(nb);
  return 0;
}
long long ElGBLaunchCount(ElGBContext ctx) { return ctx ? ctx->launches : -1; }

#define ELGB_LU(S, T)                                                                      \
  int ElGBLUPartialPiv_##S(ElGBContext ctx, int m, int n, T* A, int lda, int* swapDests,   \
                           int nb) {                                                       \
    if (int r = arg_ok(ctx && m >= 0 && n >= 0 && lda >= std::max(m, 1) &&                 \
                       (m * n == 0 || (A && swapDests))))                                 \
      return r;                                                                            \
    return elgb::to_el_error(elgb::getrf<T>(ctx, m, n, A, lda, swapDests, nb, -1));        \
  }                                                                                        \
  int ElGBSolveAfterLUPartialPiv_##S(ElGBContext ctx, int orientation, int n, const T* A,  \
                                     int lda, const int* swapDests, int nrhs, T* B,        \
                                     int ldb) {                                            \
    if (int r = arg_ok(ctx && n >= 0 && nrhs >= 0 && lda >= std::max(n, 1) &&              \
                       ldb >= std::max(n, 1) && orientation >= 0 && orientation <= 2))      \
      return r;                                                                            \
    return elgb::to_el_error(                                                              \
        elgb::getrs<T>(ctx, orientation, n, A, lda, swapDests, nrhs, B, ldb, nullptr));    \
  }                                                                                        \
  int ElGBCholesky_##S(ElGBContext ctx, int uplo, int n, T* A, int lda, int nb) {          \
    if (int r = arg_ok(ctx && n >= 0 && lda >= std::max(n, 1) && (uplo == 0 || uplo == 1))) \
      return r;                                                                            \
    return elgb::to_el_error(elgb::potrf<T>(ctx, uplo, n, A, lda, nb));                    \
  }                                                                                        \
  int ElGBSolveAfterCholesky_##S(ElGBContext ctx, int uplo, int n, const T* A, int lda,    \
                                 int nrhs, T* B, int ldb) {                                \
    if (int r = arg_ok(ctx && n >= 0 && nrhs >= 0 && lda >= std::max(n, 1) &&              \
                       ldb >= std::max(n, 1) && (uplo == 0 || uplo == 1)))                 \
      return r;                                                                            \
    return elgb::to_el_error(elgb::potrs<T>(ctx, uplo, n, A, lda, nrhs, B, ldb));          \
  }                                                                                        \
  int ElGBLinearSolve_##S(ElGBContext ctx, int n, const T* A, int lda, int nrhs, T* B,     \
                          int ldb, int nb) {                                               \
    if (int r = arg_ok(ctx && n >= 0 && nrhs >= 0 && lda >= std::max(n, 1) &&              \
                       ldb >= std::max(n, 1)))                                             \
      return r;                                                                            \
    return elgb::to_el_error(elgb::linear_solve<T>(ctx, n, A, lda, nrhs, B, ldb, nb));     \
  }                                                                                        \
  int ElGBHPDSolve_##S(ElGBContext ctx, int uplo, int n, const T* A, int lda, int nrhs,    \
                       T* B, int ldb, int nb) {                                            \
    if (int r = arg_ok(ctx && n >= 0 && nrhs >= 0 && lda >= std::max(n, 1) &&              \
                       ldb >= std::max(n, 1) && (uplo == 0 || uplo == 1)))                 \
      return r;                                                                            \
    return elgb::to_el_error(elgb::hpd_solve<T>(ctx, uplo, n, A, lda, nrhs, B, ldb, nb));  \
  }                                                                                        \
  int ElGBLUNoPiv_##S(ElGBContext ctx, int m, int n, T* A, int lda, int nb) {              \
    if (int r = arg_ok(ctx && m >= 0 && n >= 0 && lda >= std::max(m, 1) &&                 \
                       (m * n == 0 || A)))                                                 \
      return r;                                                                            \
    const int mn = std::min(m, n);                                                         \
    cudaError_t e = ctx->ensure2(sizeof(int) * (size_t)std::max(mn, 1));                   \
    if (e != cudaSuccess) return elgb::to_el_error(e);                                     \
    return elgb::to_el_error(elgb::getrf<T>(ctx, m, n, A, lda,                             \
                                            static_cast<int*>(ctx->arena2), nb, -1, false, \
                                            true));                                        \
  }                                                                                        \
  int ElGBLUFullPiv_##S(ElGBContext ctx, int m, int n, T* A, int lda, int* rowDests,       \
                        int* colDests) {                                                   \
    if (int r = arg_ok(ctx && m >= 0 && n >= 0 && lda >= std::max(m, 1) &&                 \
                       (m * n == 0 || (A && rowDests && colDests))))                       \
      return r;                                                                            \
    return elgb::to_el_error(elgb::getrf_full<T>(ctx, m, n, A, lda, rowDests, colDests));  \
  }                                                                                        \
  int ElGBSolveAfterLUFullPiv_##S(ElGBContext ctx, int orientation, int n, const T* A,     \
                                  int lda, const int* rowDests, const int* colDests,       \
                                  int nrhs, T* B, int ldb) {                               \
    if (int r = arg_ok(ctx && n >= 0 && nrhs >= 0 && lda >= std::max(n, 1) &&              \
                       ldb >= std::max(n, 1) && orientation >= 0 && orientation <= 2))      \
      return r;                                                                            \
    return elgb::to_el_error(elgb::getrs_full<T>(ctx, orientation, n, A, lda, rowDests,    \
                                                 colDests, nrhs, B, ldb));                 \
  }                                                                                        \
  int ElGBCholeskyPiv_##S(ElGBContext ctx, int uplo, int n, T* A, int lda, int* piv) {     \
    if (int r = arg_ok(ctx && n >= 0 && lda >= std::max(n, 1) && (uplo == 0 || uplo == 1) && \
                       (n == 0 || (A && piv))))                                            \
      return r;                                                                            \
    return elgb::to_el_error(elgb::potrf_piv<T>(ctx, uplo, n, A, lda, piv));               \
  }                                                                                        \
  int ElGBSolveAfterCholeskyPiv_##S(ElGBContext ctx, int uplo, int n, const T* A, int lda,  \
                                    const int* piv, int nrhs, T* B, int ldb) {             \
    if (int r = arg_ok(ctx && n >= 0 && nrhs >= 0 && lda >= std::max(n, 1) &&              \
                       ldb >= std::max(n, 1) && (uplo == 0 || uplo == 1)))                 \
      return r;                                                                            \
    return elgb::to_el_error(elgb::potrs_piv<T>(ctx, uplo, n, A, lda, piv, nrhs, B, ldb)); \
  }                                                                                        \
  int ElGBInverse_##S(ElGBContext ctx, int n, T* A, int lda, int nb) {                     \
    if (int r = arg_ok(ctx && n >= 0 && lda >= std::max(n, 1) && (n == 0 || A))) return r; \
    return elgb::to_el_error(elgb::getri<T>(ctx, n, A, lda, nb));                          \
  }                                                                                        \
  int ElGBOneCondition_##S(ElGBContext ctx, int n, const T* A, int lda, int nb,            \
                           double* cond) {                                                 \
    if (int r = arg_ok(ctx && n >= 0 && lda >= std::max(n, 1) && cond && (n == 0 || A)))   \
      return r;                                                                            \
    return elgb::to_el_error(elgb::one_condition<T>(ctx, n, A, lda, nb, cond));            \
  }

ELGB_LU(d, double)
ELGB_LU(s, float)

int ElGBLUPartialPivMixed_s(ElGBContext ctx, int m, int n, float* A, int lda, int* swapDests,
                            int nb, int gemm_kind) {
  if (int r = arg_ok(ctx && m >= 0 && n >= 0 && lda >= std::max(m, 1) &&
                     gemm_kind >= -1 && gemm_kind <= 3 && (m * n == 0 || (A && swapDests))))
    return r;
  if (nb <= 0) nb = 512;
  return elgb::to_el_error(elgb::getrf<float>(ctx, m, n, A, lda, swapDests, nb, gemm_kind,
                                              ctx->opt_tournament != 0));
}

int ElGBGemmSubTC(ElGBContext ctx, int gemm_kind, int m, int n, int k, const float* A, int lda,
                  const float* B, int ldb, float* C, int ldc) {
  if (int r = arg_ok(ctx && gemm_kind >= 0 && gemm_kind <= 3 && m >= 0 && n >= 0 && k >= 0 &&
                     lda >= std::max(m, 1) && ldb >= std::max(k, 1) && ldc >= std::max(m, 1)))
    return r;
  cudaError_t e = ctx->begin_call();
  if (e == cudaSuccess) e = ctx->ensure(elgb::tc_gemm_workspace_bytes(gemm_kind, m, n, k));
  if (e != cudaSuccess) return elgb::kElRuntimeError;
  int nl = 0;
  e = elgb::launch_tc_gemm_sub(gemm_kind, m, n, k, A, lda, B, ldb, C, ldc, ctx->arena,
                               ctx->status, ctx->stream, &nl);
  ctx->launches += nl;
  return elgb::to_el_error(e);
}

int ElGBResidual_d(ElGBContext ctx, int n, int nrhs, const double* A, int lda, const double* X,
                   int ldx, const double* B, int ldb, double* R, int ldr) {
  if (int r = arg_ok(ctx && n >= 0 && nrhs >= 0 && lda >= std::max(n, 1) &&
                     ldx >= std::max(n, 1) && ldb >= std::max(n, 1) && ldr >= std::max(n, 1)))
    return r;
  return elgb::to_el_error(elgb::residual(ctx, n, nrhs, A, lda, X, ldx, B, ldb, R, ldr));
}

int ElGBBackwardError_d(ElGBContext ctx, int n, int nrhs, const double* A, int lda,
                        const double* X, int ldx, const double* B, int ldb, double* berr) {
  if (int r = arg_ok(ctx && berr && n > 0 && nrhs > 0 && lda >= n && ldx >= n && ldb >= n))
    return r;
  return elgb::to_el_error(elgb::backward_error(ctx, n, nrhs, A, lda, X, ldx, B, ldb, berr));
}

int ElGBProbeFP64Peak(ElGBContext ctx, double* tflops) {
  if (!ctx || !tflops) return elgb::kElArgError;
  cudaSetDevice(ctx->device);
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return elgb::kElAllocError;
  const int blocks = ctx->num_sms * 8, threads = 256, iters = 4096;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  elgb::launch_fp64_fma_probe(out, blocks, threads, iters, ctx->stream);  // warm-up
  cudaEventRecord(a, ctx->stream);
  for (int r = 0; r < 5; ++r) elgb::launch_fp64_fma_probe(out, blocks, threads, iters, ctx->stream);
  cudaEventRecord(b, ctx->stream);
  cudaError_t e = cudaEventSynchronize(b);
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  ctx->launches += 6;
  if (e != cudaSuccess) return elgb::kElRuntimeError;
  const double flops = 5.0 * blocks * threads * (double)iters * 8 * 2;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return 0;
}

}  // extern "C"
