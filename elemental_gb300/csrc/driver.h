// Host-side context and driver entry points shared by the C ABIs.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "common.cuh"
#include "../../include/elgb300.h"

namespace elgb {

// Elemental's ElError codes (include/El/core/types.h:45-54 of the reference).
enum ElErrorCode : int {
  kElSuccess = 0,
  kElAllocError = 1,
  kElOutOfBoundsError = 2,
  kElArgError = 3,
  kElLogicError = 4,
  kElRuntimeError = 5,
  kElError = -1,
};

struct Context {
  int device = 0;
  int num_sms = 1;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  cudaStream_t side_stream = nullptr;  // look-ahead panels run here
  cudaStream_t swap_stream = nullptr;  // interchanges of the columns updated last
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  cudaEvent_t ev_iter = nullptr, ev_swapped = nullptr;
  void* arena = nullptr;  // growable device scratch, reused across calls
  size_t arena_bytes = 0;
  DevStatus* status = nullptr;    // device status word of the last call
  DevStatus* h_status = nullptr;  // pinned host mirror
  long long launches = 0;         // kernels enqueued by this context
  int opt_lookahead = 1;          // ElGBSetOption(ELGB_OPT_LOOKAHEAD)
  int opt_panel_ctas = 0;         // ElGBSetOption(ELGB_OPT_PANEL_CTAS), 0 = automatic
  int opt_tournament = 0;         // ElGBSetOption(ELGB_OPT_TOURNAMENT)
  int opt_residual_df = 1;        // ElGBSetOption(ELGB_OPT_RESIDUAL_DF)
  int opt_trail_grid = 2;         // ElGBSetOption(ELGB_OPT_TRAIL_GRID)
  int opt_trail_split = 1;        // ElGBSetOption(ELGB_OPT_TRAIL_SPLIT)
  int opt_inv_trsm = 0;           // ElGBSetOption(ELGB_OPT_INV_TRSM)
  int opt_swap_stream = 0;        // ElGBSetOption(ELGB_OPT_SWAP_STREAM)
  int opt_side_tc_min_n = 256;    // ElGBSetOption(ELGB_OPT_SIDE_TC_MIN_N)
  int opt_panel_node = 0;         // ElGBSetOption(ELGB_OPT_PANEL_NODE)
  // ElGBSetOption(ELGB_OPT_PANEL_TRACE): per-column leaf-panel timestamps of
  // the last factorization, 4 per column, for its first trace_cols columns
  unsigned long long* trace_buf = nullptr;
  int trace_cols = 0;
  void* arena2 = nullptr;  // second arena for drivers that call the ones above
  size_t arena2_bytes = 0;

  // Live per-kernel timing (ElGBProfile*): CUDA event pairs recorded on the
  // launching stream around the tensor-core GEMM kernel, with its algorithmic
  // flops and bytes.
  struct ProfRec {
    cudaEvent_t a, b;
    double flops, bytes;
    int tag;            // ELGB_PROF_*
    bool side = false;  // recorded on the look-ahead panel stream
    int lane = 0;       // 0 main stream, 1 look-ahead stream, 2 swap stream
  };
  int stream_lane(cudaStream_t st) const {
    return (side_stream && st == side_stream) ? 1 : (swap_stream && st == swap_stream) ? 2 : 0;
  }
  struct ProfSum {
    long long launches = 0;
    double ms = 0, flops = 0, bytes = 0;
  };
  ProfSum prof_sum[16];
  // Brackets the launches issued between begin and end on `st` when
  // profiling is on; returns -1 when off.
  int prof_begin(cudaStream_t st, int tag);
  void prof_end(int idx, cudaStream_t st, int tag, double flops, double bytes);
  bool prof_on = false;
  unsigned prof_mask = ~0u;  // families (1 << ELGB_PROF_*) bracketed while prof_on
  bool prof_wants(int tag) const { return prof_on && ((prof_mask >> tag) & 1u); }
  std::vector<ProfRec> prof;        // records of the current window
  std::vector<cudaEvent_t> ev_pool;  // reusable events
  size_t ev_used = 0;
  cudaEvent_t next_event();

  ~Context();
  cudaError_t ensure(size_t bytes);   // grows the arena (synchronizes first)
  cudaError_t ensure2(size_t bytes);  // grows arena2 (synchronizes first)
  cudaError_t begin_call();          // selects the device, clears the status word
};

int to_el_error(cudaError_t e);
int get_blocksize();
void set_blocksize(int nb);

template <typename T>
cudaError_t getrf(Context* ctx, int m, int n, T* A, long lda, int* ipiv, int nb,
                  int tc_kind = -1, bool tournament = false, bool nopiv = false);
// El::LU(A, P, Q) with full pivoting and its lu::SolveAfter.
template <typename T>
cudaError_t getrf_full(Context* ctx, int m, int n, T* A, long lda, int* p, int* q);
template <typename T>
cudaError_t getrs_full(Context* ctx, int orient, int n, const T* A, long lda, const int* p,
                       const int* q, int nrhs, T* B, long ldb);
// El::Cholesky(uplo, A, P) with diagonal pivoting and its SolveAfter.
template <typename T>
cudaError_t potrf_piv(Context* ctx, int uplo, int n, T* A, long lda, int* piv);
template <typename T>
cudaError_t potrs_piv(Context* ctx, int uplo, int n, const T* A, long lda, const int* piv,
                      int nrhs, T* B, long ldb);
// El::Inverse (funcs/Inverse/General/LUPartialPiv.hpp): A := inv(A) in place
// through getrf and getrs on the identity; info (status) at a zero pivot.
template <typename T>
cudaError_t getri(Context* ctx, int n, T* A, long lda, int nb);
// El::OneCondition (props/Condition/One.cpp:12-24): ||A||_1 ||inv(A)||_1 on
// a device copy of A (A itself untouched); +inf when A is singular.
template <typename T>
cudaError_t one_condition(Context* ctx, int n, const T* A, long lda, int nb, double* cond);
template <typename T>
cudaError_t getrs(Context* ctx, int orient, int n, const T* A, long lda, const int* ipiv,
                  int nrhs, T* B, long ldb, const int* perm);
template <typename T>
cudaError_t potrf(Context* ctx, int uplo, int n, T* A, long lda, int nb);
template <typename T>
cudaError_t potrs(Context* ctx, int uplo, int n, const T* A, long lda, int nrhs, T* B,
                  long ldb);
template <typename T>
cudaError_t linear_solve(Context* ctx, int n, const T* A, long lda, int nrhs, T* B, long ldb,
                         int nb);
template <typename T>
cudaError_t hpd_solve(Context* ctx, int uplo, int n, const T* A, long lda, int nrhs, T* B,
                      long ldb, int nb);
cudaError_t residual(Context* ctx, int n, int q, const double* A, long lda, const double* X,
                     long ldx, const double* B, long ldb, double* R, long ldr);
cudaError_t backward_error(Context* ctx, int n, int q, const double* A, long lda,
                           const double* X, long ldx, const double* B, long ldb,
                           double* berr);
cudaError_t refined_solve(Context* ctx, int n, const double* A, long lda, int nrhs,
                          const double* B, long ldb, double* X, long ldx,
                          const ElGBRefineCtrl& c, ElGBRefineInfo* info);

}  // namespace elgb

struct ElGBContextImpl : public elgb::Context {};
