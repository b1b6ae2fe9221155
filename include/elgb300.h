/*
 * elgb300.h — device-level C ABI of the GB300 dense factor-and-solve library
 * (libelgb300.so).  Plain pointers and sizes only.
 *
 * Every routine here works on DEVICE memory of the context's GPU and is
 * enqueued on the context's stream; none of them synchronizes unless it says
 * so.  Matrices are column-major with a leading dimension, as El::Matrix
 * (reference include/El/core/Matrix/decl.hpp:17-241): element (i, j) of A is
 * A[i + j*lda].  Pivots are Elemental's swap destinations, 0-based, 32-bit
 * (Permutation::SwapDestinations, reference
 * src/lapack_like/perm/Permutation.cpp:205-250; equal to LAPACK ipiv - 1).
 *
 * Return codes are Elemental's ElError values (reference
 * include/El/core/types.h:45-54): 0 EL_SUCCESS, 1 EL_ALLOC_ERROR,
 * 3 EL_ARG_ERROR, 4 EL_LOGIC_ERROR, 5 EL_RUNTIME_ERROR (singular / not HPD /
 * CUDA failure), -1 EL_ERROR.
 *
 * Numerical failures are reported through the context's status word (see
 * ElGBStatus): info = first zero pivot (LU) or first non-positive diagonal
 * (Cholesky), 1-based, 0 if none — the conditions under which the reference
 * throws SingularMatrixException (src/lapack_like/factor/LU/Panel.hpp:51-52)
 * and NonHPDMatrixException
 * (src/lapack_like/factor/Cholesky/LowerVariant3.hpp:29-30).
 */
#ifndef ELGB300_H
#define ELGB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ElGBContextImpl* ElGBContext;

/* Context: one GPU, one stream, one growable scratch arena. */
int ElGBCreate(ElGBContext* ctx, int device);
int ElGBDestroy(ElGBContext ctx);
/* Use `stream` (a cudaStream_t) for subsequent calls; NULL selects the
 * legacy default stream.  A new context uses a stream of its own. */
int ElGBSetStream(ElGBContext ctx, void* stream);
int ElGBSynchronize(ElGBContext ctx);
/* Synchronizes, then reads the status word of the last call:
 * info (see above) and err (nonzero if a bounded device-side wait gave up). */
int ElGBStatus(ElGBContext ctx, int* info, int* err);
/* Algorithmic blocksize, El::Blocksize() / El::SetBlocksize()
 * (reference src/blas_like/blocksizes.cpp:37-60); default 128. */
int ElGBBlocksize(void);
int ElGBSetBlocksize(int nb);
/* Tuning switches of a context:
 *   ELGB_OPT_LOOKAHEAD  1 (default): factor the next panel on a second
 *                       stream while the trailing update runs; 0: in order
 *   ELGB_OPT_PANEL_CTAS CTAs of a panel launch, 0 (default) = automatic
 *   ELGB_OPT_TOURNAMENT 1: ElGBLUPartialPivMixed_s picks its leaf panels'
 *                       pivots by tournament (CALU); 0 (default): partial
 *                       pivoting, El::LU's pivot sequence
 *   ELGB_OPT_PANEL_CLUSTER largest thread-block cluster (1, 2, 4, 8 or 16;
 *                       default 16) for panels that fit one cluster's
 *                       shared memory: the per-column exchange then runs
 *                       through distributed shared memory and the cluster
 *                       barrier; 1: always the cooperative kernel.
 *                       Process-wide (every context).
 *   ELGB_OPT_PANEL_REGS FP32 leaf panels keep their rows in registers
 *                       (512 threads x 2 rows per CTA): 2 (default) on a
 *                       thread-block cluster where one holds the panel
 *                       (<= 1024 rows per CTA, i.e. up to 16384 rows), in
 *                       shared memory otherwise; 1 on a cooperative grid;
 *                       0 always in shared memory.  Process-wide.
 *   ELGB_OPT_RESIDUAL_DF 1 (default): ElGBRefinedSolve_d computes its
 *                       residuals and GMRES products for n >= 2048 in
 *                       double-float arithmetic on the FP32 pipe
 *                       (FP64-level accuracy, see ElGBResidualDF_d);
 *                       0: always in FP64 arithmetic.
 *   ELGB_OPT_PANEL_TRACE value > 0: the context keeps a device buffer of
 *                       4 timestamps per column (%globaltimer, ns) for the
 *                       first `value` columns of each LU it factors; CTA 0
 *                       of each leaf panel stamps, per pivot step: before
 *                       publishing its candidate, after the previous step's
 *                       deferred rank-1 update, once the pivot exchange is
 *                       complete, after the step's multipliers, next column
 *                       and argmax.  Read with ElGBPanelTrace.  0 (default):
 *                       off.
 *   ELGB_OPT_TRAIL_GRID how the FP32 LU's tensor-core updates share the SMs
 *                       while the look-ahead panel runs: 2 (default) the
 *                       trailing update holds all GPCs but one (16-CTA
 *                       clusters, persistent) and the panel's own updates
 *                       run one CTA per tile; 1 as 2 with the panel's
 *                       updates on at most 32 persistent CTAs; 0 the
 *                       trailing update holds every SM; 3 one CTA per tile
 *                       for both.
 *   ELGB_OPT_TRAIL_SPLIT 1 (default): in the tensor-core LU, the trailing
 *                       update takes the SMs it shares with the look-ahead
 *                       panel only for the columns it is expected to finish
 *                       while the panel runs, then waits for the panel and
 *                       updates the remaining columns on every SM; 0: the
 *                       whole update beside the panel; 2 .. 1000: as 1 with
 *                       the panel's expected time scaled by value / 100
 *                       (1 means 110).
 *   ELGB_OPT_PANEL_ROWS  rows of a leaf panel per CTA that the panel kernels
 *                       aim for (64 .. 1536, default 512): more CTAs make
 *                       each pivot step's local update shorter and its
 *                       exchange longer; at <= 512 rows a CTA the register
 *                       kernel holds one row a thread (half the step code;
 *                       LU 205.0 -> 202.2 ms at n = 32768 against 1024).
 *                       Process-wide, like ELGB_OPT_PANEL_CLUSTER.
 *   ELGB_OPT_INV_TRSM   0 (default): the tensor-core LU's trailing
 *                       triangular solve U12 = L11^-1 A12 is a blocked
 *                       substitution; 1: one tensor-core product,
 *                       U12 = A12 - N A12 with N = I - L11^-1 solved once
 *                       per block.  1 shortens the LU (236 vs 241 ms at
 *                       n = 32768) but the product's rounding grows with
 *                       |N|: the factors are less accurate and refinement
 *                       took one more iteration (5 vs 4), a net loss.
 *   ELGB_OPT_SWAP_STREAM 0 (default): a block's interchanges run on the
 *                       main stream; 1: with look-ahead and the split
 *                       trailing update, those on the columns updated after
 *                       the panel run on a third stream (lowest priority)
 *                       beside the panel and the first part of the update.
 *                       Same factors; no measured change in the LU at
 *                       n = 32768 (225.8 vs 225.9 ms), so off.
 *   ELGB_OPT_PANEL_PUSH 1 (default): the register leaf panels exchange each
 *                       column's candidates by pushing them into every CTA
 *                       of the cluster (asynchronous DSMEM stores completing
 *                       on the receiver's mbarrier); 0: each CTA publishes
 *                       into its own slot and the others read it after a
 *                       cluster barrier; 2: push for 32-column leaves only.
 *                       Same pivots and factors.  Process-wide, like
 *                       ELGB_OPT_PANEL_REGS.
 *   ELGB_OPT_PANEL_PDL  1 (default): register leaf panels are launched as
 *                       programmatic dependents of the kernel before them on
 *                       their stream (placed while it finishes, waiting for
 *                       it before touching memory); 0: normal launches.
 *                       Process-wide.
 *   ELGB_OPT_SIDE_TC_MIN_N  the fewest columns (16 .. 4096, default 256)
 *                       for which the look-ahead stream's recursion updates
 *                       (m x n x n) use the tensor cores; narrower ones run
 *                       on the CUDA cores (exact FP32 FMAs).  At n = 32768
 *                       the LU took 216.5 / 213.7 / 213.0 / 213.6 ms with
 *                       64 / 128 / 256 / 512.
 *   ELGB_OPT_PANEL_NODE 0 (default): a recursion node of two leaf panels
 *                       runs its TRSM and update as separate launches; 1:
 *                       the left leaf's register kernel applies them itself
 *                       (bit-identical factors).  1 saves two launches a
 *                       node but runs the update on the cluster's few SMs:
 *                       LU 207.5 -> 227.5 ms at n = 32768, so off. */
enum {
  ELGB_OPT_LOOKAHEAD = 1,
  ELGB_OPT_PANEL_CTAS = 2,
  ELGB_OPT_TOURNAMENT = 3,
  ELGB_OPT_PANEL_CLUSTER = 4,
  ELGB_OPT_PANEL_REGS = 5,
  ELGB_OPT_RESIDUAL_DF = 6,
  ELGB_OPT_PANEL_TRACE = 7,
  ELGB_OPT_TRAIL_GRID = 8,
  ELGB_OPT_PANEL_ROWS = 9,
  ELGB_OPT_TRAIL_SPLIT = 10,
  ELGB_OPT_INV_TRSM = 11,
  ELGB_OPT_SWAP_STREAM = 12,
  ELGB_OPT_PANEL_PUSH = 13,
  ELGB_OPT_PANEL_PDL = 14,
  ELGB_OPT_SIDE_TC_MIN_N = 15,
  ELGB_OPT_PANEL_NODE = 16
};
int ElGBSetOption(ElGBContext ctx, int option, int value);

/* Copies the first ncols columns' panel timestamps (4 * ncols values, see
 * ELGB_OPT_PANEL_TRACE) to host memory `out`; synchronizes the context.
 * Columns that no leaf panel traced (e.g. factored by the batched kernel)
 * hold zeros. */
int ElGBPanelTrace(ElGBContext ctx, unsigned long long* out, int ncols);

/* Number of kernel launches this context has issued so far. */
long long ElGBLaunchCount(ElGBContext ctx);
/* Live timing of the dominant kernel (the tensor-core trailing-update GEMM):
 * between Start and Stop every launch of it is bracketed by CUDA events on
 * its stream; Stop synchronizes and returns the number of launches, their
 * summed device time (ms) and their algorithmic flops (2 m n k) and bytes
 * (C read + write, packed operands read). */
int ElGBProfileStart(ElGBContext ctx);
/* The same for the kernel families whose bit (1 << ELGB_PROF_*, below) is set
 * in tags only: fewer events in the timeline, so a timed region perturbed
 * less (bracketing every launch group of a refined solve at n = 32768 costs
 * ~14 ms of its ~295). */
int ElGBProfileStartTags(ElGBContext ctx, unsigned tags);
int ElGBProfileStop(ElGBContext ctx, long long* launches, double* ms,
                    double* flops, double* bytes);
/* After ElGBProfileStop: the same sums for one kernel family (event-bracketed
 * launch groups; with look-ahead two streams overlap, so the sums can exceed
 * wall time). */
enum {
  ELGB_PROF_TC_GEMM = 0,   /* tcgen05 trailing / TRSM / panel updates        */
  ELGB_PROF_PANEL = 1,     /* cooperative getf2 leaf panels                  */
  ELGB_PROF_SWAP = 2,      /* row-interchange pair build + apply             */
  ELGB_PROF_TRSM = 3,      /* diagonal-block triangular solves (factorization) */
  ELGB_PROF_GEMM_SIMT = 4, /* CUDA-core GEMM (FP64 path, small FP32 updates) */
  ELGB_PROF_RESIDUAL = 5,  /* FP64 residual b - A x                          */
  ELGB_PROF_SOLVE = 6,     /* low-precision triangular solves of refinement  */
  ELGB_PROF_CONVERT = 7,   /* FP64 -> FP32 copy of A (with the double-float
                              words and the norms of A, when those are made) */
  ELGB_PROF_SIDE = 8       /* + tag: that kernel's launches on the look-ahead
                              panel stream only (the factorization's critical
                              chain); the plain tags count both streams     */
};
int ElGBProfileTag(ElGBContext ctx, int tag, long long* launches, double* ms,
                   double* flops, double* bytes);
/* After ElGBProfileStop: the event-bracketed launch groups one by one, in
 * issue order (the timeline of the streams).  Fills up to cap records:
 * start (ms after the first group's start), duration (ms), tag (the family
 * above) and side (the stream: 0 main, 1 look-ahead panel stream, 2 the
 * stream of the interchanges deferred to the second part of a split
 * trailing update); *count receives the number of groups recorded. */
int ElGBProfileRecords(ElGBContext ctx, int cap, int* count, float* start_ms,
                       float* dur_ms, int* tag, int* side);

/* El::LU(A, P) with partial pivoting (reference
 * src/lapack_like/factor/LU.cpp:104-138): A (m x n) is overwritten by the
 * packed unit-lower L and upper U; swapDests (min(m,n) ints, device) receives
 * P's swap destinations.  nb <= 0 uses ElGBBlocksize(). */
int ElGBLUPartialPiv_d(ElGBContext ctx, int m, int n, double* A, int lda,
                       int* swapDests, int nb);
int ElGBLUPartialPiv_s(ElGBContext ctx, int m, int n, float* A, int lda,
                       int* swapDests, int nb);

/* Operand precision of the tensor-core products used by the low-precision
 * factorization (accumulation is always FP32):
 *   ELGB_GEMM_SIMT_FP32  FP32 FMA on the CUDA cores (no tensor cores)
 *   ELGB_GEMM_BF16       tcgen05.mma kind::f16, BF16 operands
 *   ELGB_GEMM_TF32       tcgen05.mma kind::tf32
 *   ELGB_GEMM_TF32X3     kind::tf32 on hi + lo operand splits, three products
 *                        (close to FP32 accuracy)
 *   ELGB_GEMM_FP8        kind::f8f6f4 on E4M3 operands, each scaled per panel
 *                        (per call) by a power of two mapping its largest
 *                        magnitude near 448; in the LU only the trailing
 *                        update uses it, the panel and TRSM keep TF32X3 */
enum {
  ELGB_GEMM_SIMT_FP32 = -1,
  ELGB_GEMM_BF16 = 0,
  ELGB_GEMM_TF32 = 1,
  ELGB_GEMM_TF32X3 = 2,
  ELGB_GEMM_FP8 = 3
};

/* El::LU(A, P) on an FP32 matrix whose trailing updates, blocked-TRSM updates
 * and panel-internal updates run on the tensor cores in `gemm_kind`
 * precision; same output layout as ElGBLUPartialPiv_s.  nb <= 0 selects 512. */
int ElGBLUPartialPivMixed_s(ElGBContext ctx, int m, int n, float* A, int lda,
                            int* swapDests, int nb, int gemm_kind);

/* C -= A B on the tensor cores (FP32 in and out, column-major, device):
 * the Gemm(NORMAL, NORMAL, -1, A, B, 1, C) of reference
 * src/blas_like/level3/Gemm.cpp:19-71 in `gemm_kind` operand precision. */
int ElGBGemmSubTC(ElGBContext ctx, int gemm_kind, int m, int n, int k,
                  const float* A, int lda, const float* B, int ldb, float* C,
                  int ldc);

/* Factorization precision of the mixed-precision solve. */
enum {
  ELGB_PREC_FP64 = 0, /* plain FP64 getrf + getrs (no refinement)           */
  ELGB_PREC_FP32 = 1, /* FP32 storage, TF32x3 tensor-core products (~FP32)  */
  ELGB_PREC_TF32 = 2, /* FP32 storage, TF32 tensor-core products            */
  ELGB_PREC_BF16 = 3, /* FP32 storage, BF16 tensor-core products            */
  ELGB_PREC_FP8 = 4   /* FP32 storage, E4M3 trailing updates with per-panel
                         power-of-two scales (TF32x3 panel / TRSM)          */
};

typedef struct {
  int precision;  /* ELGB_PREC_*                                            */
  int method;     /* 0 LU-IR, 1 GMRES-IR                                    */
  double tol;     /* target normwise backward error; <= 0: n * eps64         */
  int max_iters;  /* refinement steps (LU-IR) / GMRES iterations; <= 0: 30   */
  int restart;    /* GMRES restart length; <= 0: 20                          */
  int fallback;   /* nonzero: FP64 LU when the low-precision factor is
                     singular or refinement stalls                           */
  int nb;         /* blocksize of the low-precision factorization; <= 0: 512 */
  int pivoting;   /* low-precision LU's pivoting: 0 partial pivoting
                     (El::LU's; default), 1 tournament (CALU: the leaf
                     panel's pivots by a reduction tree of small partial-
                     pivoting eliminations, no per-column grid exchange) */
} ElGBRefineCtrl;

typedef struct {
  int iterations;        /* refinement steps / GMRES iterations taken        */
  int converged;         /* 1 if every column reached tol                   */
  int fell_back;         /* 1 if the FP64 LU produced the answer             */
  int precision;         /* precision of the factorization that answered     */
  double backward_error; /* achieved max-over-columns normwise backward error */
} ElGBRefineInfo;

/* Mixed-precision solve A X = B (A n x n, B and X n x nrhs, FP64, device):
 * low-precision LU on the tensor cores + LU-IR or GMRES-IR with an FP64
 * residual (semantics of reference include/El/lapack_like/solve/Refined.hpp:44-119
 * and FGMRES.hpp:37-315), FP64 LU as the fallback.  A and B are not modified.
 * Synchronizes (the stopping test runs on the host). */
int ElGBRefinedSolve_d(ElGBContext ctx, int n, const double* A, int lda,
                       int nrhs, const double* B, int ldb, double* X, int ldx,
                       const ElGBRefineCtrl* ctrl, ElGBRefineInfo* info);

/* The learned precision selector (added form): a 16 -> 64 -> 64 -> 3 FP32
 * MLP (ReLU, softmax) over the batched solver's 16 per-system features,
 * classes 0 FP64, 1 FP32, 2 BF16 factors.  Parameters are one flat FP32
 * device vector of ElGBMLPParamCount() floats:
 *   W1[16][64] b1[64] W2[64][64] b2[64] W3[64][3] b3[3]   (row-major, in x out)
 * No reference counterpart (Elemental has no learned component). */
int ElGBMLPParamCount(void);
/* Inference for B samples X (B x 16, row-major, device): probs (B x 3) and /
 * or argmax (B ints) on the device; either may be NULL. */
int ElGBMLPForward(ElGBContext ctx, const float* params, const float* X, int B,
                   float* probs, int* argmax);
/* Mean softmax cross-entropy gradient over B labelled samples (labels in
 * {0, 1, 2}) into grad (ElGBMLPParamCount() floats, device); *loss (host,
 * optional) receives the mean loss and then the call synchronizes. */
int ElGBMLPGradient(ElGBContext ctx, const float* params, const float* X,
                    const int* labels, int B, float* grad, float* loss);
/* One Adam step (step >= 1, bias-corrected; weight_decay * params is added
 * to the gradient) on params with first / second moments m, v (device,
 * ElGBMLPParamCount() floats each). */
int ElGBMLPAdamStep(ElGBContext ctx, float* params, const float* grad, float* m,
                    float* v, float lr, float beta1, float beta2, float eps,
                    float weight_decay, int step);

/* Batched uneven-size solves (added form): `count` independent systems
 * A_i X_i = B_i, packed column-major on the device (A_i n_i x n_i, then the
 * next; B_i and X_i n_i x nrhs, nrhs <= 8), solved by ONE persistent launch
 * replayed from a CUDA graph.  Options (zero-initialised = defaults):
 *   kind[i]       0 LU with partial pivoting (El::LU + lu::SolveAfter),
 *                 1 lower Cholesky (El::Cholesky + cholesky::SolveAfter);
 *                 NULL: all LU
 *   precision[i]  0 FP64 factors, 1 FP32 factors, 2 FP32 storage with BF16
 *                 operand products; 1 and 2 refine with an FP64 residual
 *                 and, unless no_fallback, fall back BF16 -> FP32 -> FP64;
 *                 NULL: all FP32
 *   nb_table      8 panel widths for n <= 32, 64, ..., 2048, larger (the
 *                 autotuner's output); NULL: 32
 *   ctas_per_sm   persistent CTAs per SM (<= 0: 1)
 *   tol           target normwise backward error (<= 0: 1e-13)
 *   max_iters     refinement steps (<= 0: 10)
 *   no_fallback   1: report non-convergence instead of refactoring in FP64
 *   features_only 1: write the selector's 16 features per system to
 *                 `features` (count x 16 floats, device) instead of solving
 *   method        refinement of precision 1/2 factors: 0 LU-IR and, when it
 *                 stalls, flexible GMRES-IR (FP64 Arnoldi, the factors as
 *                 preconditioner, El's FGMRES semantics); 1 LU-IR only;
 *                 2 FGMRES-IR only
 * Execute enqueues the graph on the context's stream; Results synchronizes
 * and copies one ElGBBatchResult per system (features_only: backward_error
 * holds the 1-norm condition estimate). */
typedef struct ElGBBatchPlanImpl* ElGBBatchPlan;
typedef struct {
  int iterations, converged, fell_back, info;
  double backward_error;
  int gmres_iterations;
  int precision;       /* precision whose factors produced the result (0 FP64,
                          1 FP32, 2 BF16); fell_back = it differs from the
                          precision asked for */
  long long device_ns; /* device time the persistent CTA spent on the system */
  int selector_choice; /* fused selection: the network's class (0 FP64, 1 FP32,
                          2 BF16); otherwise 0 */
  int reserved;
} ElGBBatchResult;
typedef struct {
  const int* kind;
  const int* precision;
  const int* nb_table;
  int ctas_per_sm;
  double tol;
  int max_iters;
  int no_fallback;
  int features_only;
  float* features;
  int method;          /* 0 LU-IR then FGMRES-IR on stall, 1 LU-IR, 2 FGMRES-IR */
  int gmres_restart;   /* FGMRES restart length, <= 32 (0: 30) */
  int gmres_max_iters; /* FGMRES iterations per right-hand side; 0: max(16,
                          n / 24) (under ~half the time of an FP64 LU);
                          negative -d: max(16, n / d) */
  const int* precision_device; /* device int per system, read at each Execute
                                  (overrides precision; e.g. the selector's
                                  ElGBMLPForward argmax), or NULL */
  long long* phase_ns; /* device, count x 10, or NULL: per-system device time
                          of the low-precision LU's panel, row swaps, U12
                          solve, trailing update, then LU-IR, FGMRES-IR, the
                          FP64 path, the feature pass, and within LU-IR the
                          FP64 residuals and the low-precision solves (ns) */
  const float* selector_params; /* device, ElGBMLPParamCount() floats, or NULL:
                          fused selection in the same launch -- each
                          system's features (FP32 LU, kept), the network's
                          class (ElGBMLPForward's argmax), then the solve in
                          that precision; a low-precision class refines with
                          the kept FP32 factors.  `features` (if set) also
                          receives the features */
  int simt_update;     /* 1: FP32 / BF16 trailing updates on SIMT FMAs instead
                          of the tensor cores (tcgen05) */
} ElGBBatchOptions;
int ElGBBatchedPlanCreate(ElGBContext ctx, int count, const int* n, int nrhs,
                          const double* A, const double* B, double* X,
                          const ElGBBatchOptions* options, ElGBBatchPlan* plan);
int ElGBBatchedExecute(ElGBBatchPlan plan);
int ElGBBatchedResults(ElGBBatchPlan plan, ElGBBatchResult* out);
double ElGBBatchedFlops(ElGBBatchPlan plan);
int ElGBBatchedPlanDestroy(ElGBBatchPlan plan);

/* lu::SolveAfter(orientation, A, P, B) (reference
 * src/lapack_like/factor/LU/SolveAfter.hpp:66-92): orientation 0 NORMAL,
 * 1 TRANSPOSE, 2 ADJOINT (= TRANSPOSE for real data).  B is n x nrhs. */
int ElGBSolveAfterLUPartialPiv_d(ElGBContext ctx, int orientation, int n,
                                 const double* A, int lda,
                                 const int* swapDests, int nrhs, double* B,
                                 int ldb);
int ElGBSolveAfterLUPartialPiv_s(ElGBContext ctx, int orientation, int n,
                                 const float* A, int lda, const int* swapDests,
                                 int nrhs, float* B, int ldb);

/* El::Cholesky(uplo, A) (reference src/lapack_like/factor/Cholesky.cpp:26-38):
 * uplo 0 LOWER, 1 UPPER; only that triangle is read and written. */
int ElGBCholesky_d(ElGBContext ctx, int uplo, int n, double* A, int lda,
                   int nb);
int ElGBCholesky_s(ElGBContext ctx, int uplo, int n, float* A, int lda,
                   int nb);

/* cholesky::SolveAfter(uplo, NORMAL, A, B) (reference
 * src/lapack_like/factor/Cholesky/SolveAfter.hpp:15-43). */
int ElGBSolveAfterCholesky_d(ElGBContext ctx, int uplo, int n,
                             const double* A, int lda, int nrhs, double* B,
                             int ldb);
int ElGBSolveAfterCholesky_s(ElGBContext ctx, int uplo, int n,
                             const float* A, int lda, int nrhs, float* B,
                             int ldb);

/* El::LU(A) without pivoting (reference src/lapack_like/factor/LU.cpp:21-44,
 * lu::Unb LU/Local.hpp:42-61): packed unit-L \ U in place; a zero pivot
 * sets info (the reference throws SingularMatrixException).  Replaces
 * ElLU_d / ElLU_s (include/El/lapack_like/factor.h:467-468). */
int ElGBLUNoPiv_d(ElGBContext ctx, int m, int n, double* A, int lda, int nb);
int ElGBLUNoPiv_s(ElGBContext ctx, int m, int n, float* A, int lda, int nb);

/* El::LU(A, P, Q) with full pivoting (reference src/lapack_like/factor/LU.cpp:
 * 145-152 -> LU/Full.hpp:15-59): unblocked; per step the largest-magnitude
 * entry of the trailing block (first in column-major order on ties), row
 * and column swap, scaling, rank-1 update.  rowDests / colDests (min(m,n)
 * ints, device) receive the row and column swap destinations; a zero pivot
 * sets info.  Replaces ElLUFullPiv_d / _s (include/El/lapack_like/
 * factor.h:538-541); lu::SolveAfter(orientation, A, P, Q, B)
 * (LU/SolveAfter.hpp:120-145) replaces ElSolveAfterLUFullPiv_d / _s
 * (factor.h:557-563). */
int ElGBLUFullPiv_d(ElGBContext ctx, int m, int n, double* A, int lda, int* rowDests,
                    int* colDests);
int ElGBLUFullPiv_s(ElGBContext ctx, int m, int n, float* A, int lda, int* rowDests,
                    int* colDests);
int ElGBSolveAfterLUFullPiv_d(ElGBContext ctx, int orientation, int n, const double* A,
                              int lda, const int* rowDests, const int* colDests, int nrhs,
                              double* B, int ldb);
int ElGBSolveAfterLUFullPiv_s(ElGBContext ctx, int orientation, int n, const float* A,
                              int lda, const int* rowDests, const int* colDests, int nrhs,
                              float* B, int ldb);

/* El::Cholesky(uplo, A, P) with diagonal pivoting, P A P^T = L L^T = U^T U
 * (reference src/lapack_like/factor/Cholesky.cpp:44-52 ->
 * Cholesky/Pivoted{Lower,Upper}Variant3.hpp): per step the largest updated
 * diagonal entry (the first on ties), a symmetric swap in the uplo
 * triangle, scaling by 1/sqrt(pivot), the rank-1 update.  piv (n ints,
 * device) receives the swap destinations; no error for a non-positive pivot
 * (the reference takes its square root).  Replaces ElCholeskyPiv_d / _s
 * (include/El/lapack_like/factor.h:80-83); the solve
 * (Cholesky/SolveAfter.hpp:46-76) replaces ElSolveAfterCholeskyPiv_d / _s
 * (factor.h:100-105). */
int ElGBCholeskyPiv_d(ElGBContext ctx, int uplo, int n, double* A, int lda, int* piv);
int ElGBCholeskyPiv_s(ElGBContext ctx, int uplo, int n, float* A, int lda, int* piv);
int ElGBSolveAfterCholeskyPiv_d(ElGBContext ctx, int uplo, int n, const double* A, int lda,
                                const int* piv, int nrhs, double* B, int ldb);
int ElGBSolveAfterCholeskyPiv_s(ElGBContext ctx, int uplo, int n, const float* A, int lda,
                                const int* piv, int nrhs, float* B, int ldb);

/* El::Inverse(A) (reference src/lapack_like/funcs/Inverse/General.cpp:15-20 ->
 * General/LUPartialPiv.hpp:21-74): A := inv(A) in place via LU with partial
 * pivoting; a zero pivot sets info (SingularMatrixException).  Replaces
 * ElInverse_d / ElInverse_s (include/El/lapack_like/funcs.h:99-100). */
int ElGBInverse_d(ElGBContext ctx, int n, double* A, int lda, int nb);
int ElGBInverse_s(ElGBContext ctx, int n, float* A, int lda, int nb);

/* El::OneCondition(A) (reference src/lapack_like/props/Condition/One.cpp:12-24):
 * ||A||_1 ||inv(A)||_1 on a copy (A untouched), +inf when A is singular
 * (not an error).  Synchronizes.  Replaces ElOneCondition_d / _s
 * (include/El/lapack_like/props.h:81-82). */
int ElGBOneCondition_d(ElGBContext ctx, int n, const double* A, int lda, int nb,
                       double* cond);
int ElGBOneCondition_s(ElGBContext ctx, int n, const float* A, int lda, int nb,
                       double* cond);

/* El::LinearSolve(A, B) (reference src/lapack_like/solve/Linear.cpp:212-218):
 * A is left untouched (the reference copies it); B is overwritten by X.
 * Gaussian elimination on [A | B] as RowEchelon (Linear.cpp:30-77), then
 * the upper-triangular solve. */
int ElGBLinearSolve_d(ElGBContext ctx, int n, const double* A, int lda,
                      int nrhs, double* B, int ldb, int nb);
int ElGBLinearSolve_s(ElGBContext ctx, int n, const float* A, int lda,
                      int nrhs, float* B, int ldb, int nb);

/* El::HPDSolve(uplo, NORMAL, A, B) (reference src/lapack_like/solve/HPD.cpp:47-55). */
int ElGBHPDSolve_d(ElGBContext ctx, int uplo, int n, const double* A, int lda,
                   int nrhs, double* B, int ldb, int nb);
int ElGBHPDSolve_s(ElGBContext ctx, int uplo, int n, const float* A, int lda,
                   int nrhs, float* B, int ldb, int nb);

/* FP64 residual R = B - A X (n x nrhs, nrhs <= 16), deterministic order;
 * the residual of the refinement loop of reference
 * include/El/lapack_like/solve/Refined.hpp:70-73. */
int ElGBResidual_d(ElGBContext ctx, int n, int nrhs, const double* A,
                   int lda, const double* X, int ldx, const double* B,
                   int ldb, double* R, int ldr);

/* R = B - A X (n x nrhs, any nrhs) to FP64 accuracy in double-float
 * arithmetic on the FP32 pipe: the residual ElGBRefinedSolve_d computes by
 * default (ELGB_OPT_RESIDUAL_DF).  Each call splits A into two FP32 words
 * (8 n^2 bytes of context scratch), then 2 n^2 nrhs double-float products.
 * Each entry is within 16 ulps of sum_j |a_ij x_j| + |b_i| of the exact
 * residual for n >= 1024 (32 below); A's entries must lie in FP32's
 * exponent range (outside it the FP64 kernels run).  Deterministic order.  The residual of the refinement loop of reference
 * include/El/lapack_like/solve/Refined.hpp:70-73. */
int ElGBResidualDF_d(ElGBContext ctx, int n, int nrhs, const double* A,
                     int lda, const double* X, int ldx, const double* B,
                     int ldb, double* R, int ldr);

/* The residual of ElGBResidual_d for callers that cannot allocate device
 * memory: device memory budgeted up front or owned by another allocator, or
 * code that must not let cudaMalloc / cudaFree synchronize the device.  No
 * counterpart in the reference.  It calls no
 * cudaMalloc / cudaFree and needs no context: its scratch is a fixed 8 MiB
 * device array that the library holds on every GPU it is loaded on, so it
 * accepts only n * min(nrhs, 16) * ceil(n / 4096) <= 1048576 (e.g. n <= 16384
 * with 16 right-hand sides, n <= 32768 with 4) and returns EL_ARG_ERROR (3)
 * beyond that, before touching any memory.  Runs on `stream` (a cudaStream_t,
 * NULL = legacy default stream) of the current device.  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress).  All
 * calls share the array: calls that overlap on the GPU race on it, calls on
 * one stream do not. */
int ElGBResidualNoAlloc_d(int n, int nrhs, const double* A, int lda,
                          const double* X, int ldx, const double* B, int ldb,
                          double* R, int ldr, void* stream);

/* Normwise backward error max_j ||b_j - A x_j||_2 /
 * (||A||_F ||x_j||_2 + ||b_j||_2), computed in FP64 on the device;
 * synchronizes and writes the value to *berr (host). */
int ElGBBackwardError_d(ElGBContext ctx, int n, int nrhs, const double* A,
                        int lda, const double* X, int ldx, const double* B,
                        int ldb, double* berr);

/* Measures the device FP64 FMA rate (TFLOP/s) with a dependent-chain probe;
 * synchronizes. */
int ElGBProbeFP64Peak(ElGBContext ctx, double* tflops);

#ifdef __cplusplus
}
#endif

#endif /* ELGB300_H */
