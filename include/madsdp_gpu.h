/*
 * madsdp_gpu.h -- C ABI of the GB300 (sm_103a) interior-point library for
 * MadSDP.jl.  Plain pointers and sizes only; every call returns an int status
 * (0 = ok, negative = usage or CUDA error, see msdp_last_error).
 *
 * The library replaces, for one batch of SDPs resident on one GPU, the
 * per-iteration numerical work that MadSDP performs on the CPU:
 *
 *   msdp_batch_create       MadSDPSolver(model; components..., options...)
 *                           src/solver.jl:87-160 (workspace allocation) and
 *                           the model upload done by LowRankOpt.Model
 *   msdp_batch_initialize   initialize!(solver), src/solver.jl:286-293
 *                           (initial_point!, initialize_algorithm!)
 *   msdp_batch_iterate      iterate! + update_termination!,
 *                           src/primal_dual.jl:85-134, src/dual_centering.jl:266-303
 *   msdp_batch_solve        solve!(solver), src/solver.jl:385-396
 *   msdp_batch_get_stats    the fields read by SolverCore.solve!, src/moi.jl:53-72
 *   msdp_batch_get_solution MOI.get(::Solver, ::LRO.Solution), src/moi.jl:76-78
 *
 * and, for the Newton-system identity tests of the reference
 * (test/qr_schur.jl:16-66), component-granular entry points mirroring
 * update_residuals! (src/step.jl:12-47), _prepare! + _factorize_schur!
 * (src/primal_dual.jl:29-37,74-80), correction! (src/step.jl:128-136) and
 * _solve_directions! (src/primal_dual.jl:40-54).
 *
 * Storage conventions: dense matrices are column-major n x n float64;
 * constraint matrices are coordinate lists of full symmetric entries
 * (both triangles).  Host buffers are borrowed for the duration of a call.
 */
#ifndef MADSDP_GPU_H
#define MADSDP_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- component selectors (src/components.jl) ---------------------------- */
enum msdp_algorithm { MSDP_PRIMAL_DUAL = 0, MSDP_DUAL_CENTERING = 1 };
enum msdp_direction { MSDP_NT = 0, MSDP_HKM = 1 };
enum msdp_step_length { MSDP_EIGEN_STEP = 0, MSDP_CHOLESKY_BACKTRACK = 1 };
enum msdp_centering { MSDP_MEHROTRA = 0, MSDP_ADAPTIVE_MU = 1 };
enum msdp_initial_point { MSDP_SCALED_IDENTITY = 0, MSDP_INITIAL_POINT = 1, MSDP_DUAL_SHIFT = 2 };
enum msdp_schur_solver { MSDP_DENSE_CHOLESKY = 0, MSDP_MADNLP_SCHUR = 1, MSDP_QR_SCHUR = 2 };
/* MSDP_FP64_TENSOR: whole-GPU solver only; its dense double-precision
 * products run as cuBLAS's fixed-point FP64 emulation on tensor cores. */
enum msdp_precision { MSDP_FP64 = 0, MSDP_MIXED = 1, MSDP_FP64_TENSOR = 2 };

/* ---- statuses (MadNLP.Status values used by MadSDP, src/moi.jl:16-29) --- */
enum msdp_status {
  MSDP_SOLVE_SUCCEEDED = 1,
  MSDP_SOLVED_TO_ACCEPTABLE_LEVEL = 2,
  MSDP_SEARCH_DIRECTION_BECOMES_TOO_SMALL = 3,
  MSDP_MAXIMUM_ITERATIONS_EXCEEDED = 5,
  MSDP_MAXIMUM_WALLTIME_EXCEEDED = 6,
  MSDP_INFEASIBLE_PROBLEM_DETECTED = 8,
  MSDP_ERROR_IN_STEP_COMPUTATION = 11,
  MSDP_USER_REQUESTED_STOP = 13,
  MSDP_INITIAL = 100,
  MSDP_REGULAR = 101
};

/* ---- return codes ---------------------------------------------------------- */
enum msdp_error {
  MSDP_OK = 0,
  MSDP_ERR_INVALID_ARGUMENT = -1, /* ArgumentError of the reference        */
  MSDP_ERR_CUDA = -2,
  MSDP_ERR_OUT_OF_MEMORY = -3,
  MSDP_ERR_UNSUPPORTED = -4,      /* combination not built into the kernel */
  MSDP_ERR_INITIAL_POINT = -5,    /* ErrorException of the reference       */
  MSDP_ERR_TOO_LARGE = -6         /* beyond the limits of msdp_solve_static */
};

/* Components: mirror src/components.jl:30-300 with their default values. */
typedef struct msdp_components {
  int32_t algorithm;      /* msdp_algorithm     (PrimalDual)        */
  int32_t direction;      /* msdp_direction     (NT)                */
  int32_t step;           /* msdp_step_length   (EigenStep)         */
  int32_t centering;      /* msdp_centering     (Mehrotra)          */
  int32_t initial_point;  /* msdp_initial_point (ScaledIdentity)    */
  int32_t schur;          /* msdp_schur_solver  (DenseCholesky)     */
  int32_t precision;      /* msdp_precision     (FP64)              */
  int32_t centering_max_iter; /* DualCentering, 50                  */
  double tau;             /* EigenStep tau, 0.95                    */
  double shrink;          /* CholeskyBacktrack, 0.8                 */
  double boundary;        /* CholeskyBacktrack, 0.95                */
  double sigma_exponent;  /* Mehrotra, 3                            */
  double initial_ratio;   /* AdaptiveMu, 1/4                        */
  double ratio;           /* AdaptiveMu, 1/2                        */
  double scale;           /* ScaledIdentity(scale); <= 0: automatic */
  double initial_shift;   /* DualShift, 1                           */
  double max_shift;       /* DualShift, 1e10                        */
  double dc_beta;         /* DualCentering beta, 0.2                */
  double dc_delta;        /* DualCentering delta, 1                 */
  double dc_A;            /* DualCentering A, 2; NaN: theoretical   */
} msdp_components;

/* Options: src/options.jl:3-15, plus the precision switch of MSDP_MIXED. */
typedef struct msdp_options {
  double tol;              /* 1e-7  */
  int32_t max_iter;        /* 100   */
  int32_t max_schur_reg;   /* 8     */
  double max_wall_time;    /* 3600  */
  double mu_min;           /* 1e-14 */
  double regularize_schur; /* 1e-12 */
  int32_t datasparsity;    /* 8 (accepted, constraint storage is chosen per problem) */
  int32_t mixed_refine;    /* MSDP_MIXED: refinement passes of each FP32 direction against the float64 primal defect (2) */
  double switch_tol;       /* MSDP_MIXED: FP32 iterations while max(inf_pr, inf_du, gap) > switch_tol (0) */
} msdp_options;

/* One problem in the form of LowRankOpt.Model(C, A, b, d_lin, C_lin, sides). */
typedef struct msdp_problem_desc {
  int32_t nblocks, m, ns, pad0;
  const int32_t* sides;          /* [nblocks]                                   */
  const double* const* C;        /* [nblocks] -> n_i*n_i column-major            */
  const int64_t* A_nnz;          /* [nblocks] number of full symmetric entries   */
  const int32_t* const* A_con;   /* [nblocks] -> [nnz] constraint index (0-based) */
  const int32_t* const* A_row;   /* [nblocks] -> [nnz] row                       */
  const int32_t* const* A_col;   /* [nblocks] -> [nnz] column                    */
  const double* const* A_val;    /* [nblocks] -> [nnz] value                     */
  const double* b;               /* [m]                                         */
  const double* d_lin;           /* [ns]                                        */
  const double* C_lin;           /* [m*ns] column-major                          */
} msdp_problem_desc;

/* Iteration data of one problem (src/solver.jl:37-48, src/moi.jl:57-65). */
typedef struct msdp_stats {
  int32_t status, iter;
  int32_t iter_fp32, iter_fp64;  /* iterations run in each precision */
  double pobj, dobj;
  double inf_pr, inf_du, gap;    /* gap = inf_compl                  */
  double mu, sigma, alpha, beta;
  double solve_ns;               /* device time from initialize to termination */
  int32_t n_newton, n_predictor; /* DualCentering counters            */
} msdp_stats;

/* One row of the iteration log (src/solver.jl:367-383). */
typedef struct msdp_iter_record {
  double iter, pobj, dobj, inf_pr, inf_du, gap, mu, alpha, beta, phase;
} msdp_iter_record;

typedef struct msdp_context msdp_context;
typedef struct msdp_batch msdp_batch;

void msdp_default_components(msdp_components* c);
void msdp_default_options(msdp_options* o);

/* Context: one CUDA device and one stream. */
int msdp_context_create(int device, msdp_context** ctx);
int msdp_context_destroy(msdp_context* ctx);
const char* msdp_last_error(const msdp_context* ctx);
/* The cudaStream_t of the context (to time or order work against it). */
void* msdp_context_stream(const msdp_context* ctx);
int msdp_device_count(void);

/* A batch of problems solved together (one CTA per problem at a time).
 * Uploads every problem and allocates every workspace; nothing is
 * allocated afterwards. */
int msdp_batch_create(msdp_context* ctx, const msdp_problem_desc* problems, int32_t nprob,
                      const msdp_components* comp, const msdp_options* opt, msdp_batch** batch);
int msdp_batch_destroy(msdp_batch* batch);
/* Bytes of device memory the batch holds. */
int64_t msdp_batch_device_bytes(const msdp_batch* batch);

/* InitialPoint(X, y; x) of problem `prob` (src/components.jl:234-252); x may be NULL. */
int msdp_batch_set_initial_point(msdp_batch* batch, int32_t prob, const double* const* X,
                                 const double* y, const double* x);
/* Overwrite the iterate (X, S per block, y, x, z); NULL pointers keep the current value. */
int msdp_batch_set_iterate(msdp_batch* batch, int32_t prob, const double* const* X,
                           const double* const* S, const double* y, const double* x, const double* z);

int msdp_batch_initialize(msdp_batch* batch);
/* Enqueue initialize + iterate-to-termination on the context stream without
 * waiting (an initial-point failure shows as status 200 in the stats). */
int msdp_batch_launch_solve(msdp_batch* batch);
/* Enqueue initialize! only, without waiting. */
int msdp_batch_launch_initialize(msdp_batch* batch);
/* Bytes copied host -> device when the batch was created. */
int64_t msdp_batch_upload_bytes(const msdp_batch* batch);
/* Run up to `max_iterations` iterations (<= 0: until every problem stops). */
int msdp_batch_iterate(msdp_batch* batch, int32_t max_iterations);
int msdp_batch_solve(msdp_batch* batch);
int msdp_batch_synchronize(msdp_batch* batch);

int msdp_batch_get_stats(msdp_batch* batch, int32_t prob, msdp_stats* out);
int msdp_batch_get_all_stats(msdp_batch* batch, msdp_stats* out /* [nprob] */);
/* X per block (n_i*n_i each), y (m), x (ns), z (ns); NULL pointers are skipped. */
int msdp_batch_get_solution(msdp_batch* batch, int32_t prob, double* const* X, double* y,
                            double* x, double* z);
/* Every problem's solution in one download: for each problem in order, X of
 * each block (column-major n x n), then y (m), x (ns) and z (ns), packed into
 * `out` of msdp_batch_solution_size() doubles (MOI.get(::Solver,
 * ::LRO.Solution), src/moi.jl:76-78, for a whole batch). */
int64_t msdp_batch_solution_size(const msdp_batch* batch);
int msdp_batch_get_all_solutions(msdp_batch* batch, double* out);
int msdp_batch_get_trajectory(msdp_batch* batch, int32_t prob, msdp_iter_record* out,
                              int32_t capacity, int32_t* count);

/* Component-granular steps (identity tests). */
int msdp_batch_update_residuals(msdp_batch* batch);
int msdp_batch_prepare(msdp_batch* batch, int32_t* ok /* [nprob]: _prepare! && _factorize_schur! */);
int msdp_batch_solve_directions(msdp_batch* batch, double mu, int32_t corrected);
int msdp_batch_correction(msdp_batch* batch);
/* delX, delS per block; dely (m); delx, delz (ns); Rp (m); Rd per block. */
int msdp_batch_get_directions(msdp_batch* batch, int32_t prob, double* const* delX,
                              double* const* delS, double* dely, double* delx, double* delz);
int msdp_batch_get_residuals(msdp_batch* batch, int32_t prob, double* Rp, double* const* Rd,
                             double* Rd_lin);
/* The NT scaling W and the correction of each block (n_i*n_i each). */
int msdp_batch_get_block_matrix(msdp_batch* batch, int32_t prob, int32_t block, int32_t which,
                                double* out);
enum msdp_block_matrix { MSDP_MAT_W = 0, MSDP_MAT_CORR = 1, MSDP_MAT_SI = 2, MSDP_MAT_S = 3,
                         MSDP_MAT_X = 4 };

/* Device profile of problem `prob`: cycle counters per phase and work
 * counters of the last solve (names in the same order as
 * msdp_profile_field_name); returns the number of fields written. */
int msdp_batch_get_profile(msdp_batch* batch, int32_t prob, double* out, int32_t capacity);
const char* msdp_profile_field_name(int32_t index);

/* ---- continuous-batching server ---------------------------------------------
 * The serving loop of MadSDP's batched/served use (no counterpart in the
 * reference, which solves one model per call): requests of any size are
 * submitted at any time; each msdp_server_step admits pending requests in
 * arrival order while their data and workspaces fit the memory budget,
 * initializes them, advances every active request by `iterations`
 * interior-point iterations in one persistent launch, and moves finished
 * requests (stats and solution) to host memory, freeing their device memory
 * for the next admissions.  All device memory is allocated at creation. */
typedef struct msdp_server msdp_server;
int msdp_server_create(msdp_context* ctx, const msdp_components* comp, const msdp_options* opt,
                       int64_t memory_budget_bytes, int32_t max_slots, msdp_server** server);
int msdp_server_destroy(msdp_server* server);
/* Copies the problem; returns MSDP_ERR_TOO_LARGE if it can never fit. */
int msdp_server_submit(msdp_server* server, const msdp_problem_desc* problem, int64_t* request_id);
int msdp_server_step(msdp_server* server, int32_t iterations, int32_t* active, int32_t* completed);
/* Asynchronous, time-sliced waves: collects the waves that have finished
 * (their terminated requests become results), admits pending requests, and
 * starts one wave over every idle request on a free stream of the server
 * without waiting for it, so waves overlap on the GPU and new requests do
 * not wait for long-running ones.  Within a wave each request runs at least
 * one and at most `iterations` iterations, stopping once the wave has run
 * `budget_s` seconds and every request of the wave has iterated once.
 * msdp_server_step is the synchronous form (budget 0, waits for the wave). */
int msdp_server_step_budget(msdp_server* server, int32_t iterations, double budget_s, int32_t* active,
                            int32_t* completed);
int msdp_server_counts(const msdp_server* server, int32_t* pending, int32_t* active, int64_t* completed);
/* 1 while the request is not finished; 0 once its results are copied out
 * (the request is then forgotten).  latency_s = finish - submit, host clock. */
int msdp_server_result(msdp_server* server, int64_t request_id, msdp_stats* stats, double* const* X, double* y,
                       double* x, double* z, double* latency_s);
/* Ids of requests finished since the last call (up to `capacity`, oldest
 * first); each id is reported once. */
int msdp_server_finished(msdp_server* server, int64_t* ids, int32_t capacity, int32_t* count);
int64_t msdp_server_launch_count(const msdp_server* server);

/* ---- solve without allocating --------------------------------------------
 * msdp_solve_static has no counterpart in the reference.  It is for callers
 * that may not allocate device memory: a serving runtime or plugin host that
 * owns every byte of the GPU through its own pool, or a control loop that
 * must not pay for (or risk failing) a cudaMalloc/cudaFree.  It solves ONE
 * problem with the FP64 kernel of msdp_batch_solve, but every device-side
 * buffer lives in one static device array of MSDP_STATIC_SCRATCH_BYTES that
 * each GPU loading the library holds until exit.  It issues only
 * cudaMemcpyAsync, cudaMemsetAsync and kernel launches on `stream` (a
 * cudaStream_t; NULL = default stream) and waits for them; it calls no
 * cudaMalloc, cudaFree or allocating library routine.  Inputs are the host
 * problem description; outputs are written to the caller's host buffers
 * (X per block, y, x, z and stats; NULL pointers are skipped).
 *
 * Limits: at most MSDP_STATIC_MAX_BLOCKS blocks and a total layout (problem
 * data, constraint lists and workspaces) that fits the array, roughly
 * sum_i 250 n_i^2 + 8 m^2 + 52 nnz bytes; larger problems return
 * MSDP_ERR_TOO_LARGE.  PrimalDual + DenseCholesky in FP64 with ScaledIdentity
 * or DualShift only (MSDP_ERR_UNSUPPORTED otherwise).
 *
 * The first call on a device looks up the array's device address with
 * cudaGetSymbolAddress (with that device current); make that first call
 * before any stream capture.  Every call reuses the same array and zeroes it
 * before use, so calls that overlap on the GPU (other threads, other streams)
 * race and must be serialized by the caller. */
#define MSDP_STATIC_SCRATCH_BYTES (16ll * 1024 * 1024)
#define MSDP_STATIC_MAX_BLOCKS 16
int msdp_solve_static(const msdp_problem_desc* problem, const msdp_components* comp, const msdp_options* opt,
                      void* stream, double* const* X, double* y, double* x, double* z, msdp_stats* stats);

/* Number of kernel launches issued by this batch since creation. */
int64_t msdp_batch_launch_count(const msdp_batch* batch);

/* ---- one large problem on the whole GPU -------------------------------------
 * MadSDPSolver + solve! (src/solver.jl:87-160, 385-396) for a single problem
 * whose blocks or constraint count are too large for one thread block per
 * problem (max-cut n = 2000, dense constraints with m = 2000, ...).  Each
 * iteration runs as device-wide operations on the context's stream: dense
 * products, Cholesky factorizations and symmetric eigendecompositions
 * through cuBLAS/cuSOLVER, and this library's kernels for the Schur
 * assembly of coordinate-list constraints, A(X), A*(y), residuals, NT
 * scaling, correction and reductions.  Step lengths use exact eigenvalues.
 * PrimalDual (NT or HKM; EigenStep or CholeskyBacktrack; Mehrotra or
 * AdaptiveMu) with DenseCholesky in FP64; other components return
 * MSDP_ERR_UNSUPPORTED.  All device memory is allocated at creation. */
typedef struct msdp_solver msdp_solver;
int msdp_solver_create(msdp_context* ctx, const msdp_problem_desc* problem, const msdp_components* comp,
                       const msdp_options* opt, msdp_solver** solver);
int msdp_solver_destroy(msdp_solver* solver);
/* InitialPoint(X, y; x) (src/components.jl:234-252); x = NULL means ones. */
int msdp_solver_set_initial_point(msdp_solver* solver, const double* const* X, const double* y, const double* x);
/* initialize + iterate to termination; the status is in msdp_solver_get_stats. */
int msdp_solver_solve(msdp_solver* solver);
int msdp_solver_get_stats(const msdp_solver* solver, msdp_stats* out);
int msdp_solver_get_solution(msdp_solver* solver, double* const* X, double* y, double* x, double* z);
int msdp_solver_get_trajectory(const msdp_solver* solver, msdp_iter_record* out, int32_t capacity, int32_t* count);
int64_t msdp_solver_device_bytes(const msdp_solver* solver);
/* Device seconds per phase of the last solve (prepare, Schur assembly,
 * Schur factorization, directions, step lengths, correction, take step and
 * residuals); returns the number of fields written. */
int msdp_solver_get_profile(const msdp_solver* solver, double* seconds, int32_t capacity);
const char* msdp_solver_profile_field_name(int32_t index);
/* Work counters of the last msdp_solver_solve (no reference counterpart):
   Schur refinement steps and FP64 fallbacks, NT eigendecompositions by FP32
   eigensolver + FP64 refinement and by the dense FP64 eigensolver, the
   refinement steps, tensor-core products, and for the step-length
   lambda_min of blocks above 256 the Lanczos calls, their steps and the
   calls that fell back to the dense eigensolver.  Writes min(capacity,
   count) values; returns that number. */
int msdp_solver_get_counters(const msdp_solver* solver, int64_t* out, int32_t capacity);
const char* msdp_solver_counter_name(int32_t index);
/* Launches of this library's own kernels (library calls not counted). */
int64_t msdp_solver_launch_count(const msdp_solver* solver);
const char* msdp_solver_last_error(const msdp_solver* solver);

/* ---- component-granular calls on a whole-GPU solver ---------------------------
 * For running one GPU component beside the reference's CPU components, and
 * for identity tests.  The iterate is the one set last (or the solver's).
 *   msdp_solver_set_iterate       X, S, y, x, z of the host driver; updates
 *                                 the residuals (src/step.jl:12-47)
 *   msdp_solver_prepare           _prepare! (src/primal_dual.jl:29-37):
 *                                 chol(S) with the flush and S^-1
 *                                 (src/blocks.jl:94-130), the NT scaling
 *                                 W, G, D (src/directions.jl:45-75) and
 *                                 chol(X) for EigenStep; *ok as the reference
 *   msdp_solver_schur_assemble    LowRankOpt.schur_complement!(model, L, R, H)
 *                                 (called at src/solver.jl:304) with the
 *                                 prepared scaling, plus C_lin diag(x/z) C_lin';
 *                                 the lower triangle of H (m x m column-major)
 *                                 is written; MSDP_MIXED (NT, mixed-precision
 *                                 solvers) gives the split-precision assembly
 *   msdp_solver_get_block_matrix  the prepared W, G, S^-1, Ls, Lx (n x n) or D (n)
 *   msdp_solver_step_eig          lambda_min(L^-1 D L^-T) of EigenStep
 *                                 (src/step.jl:150-183) for a lower-triangular
 *                                 L and symmetric D of the block's size */
enum msdp_solver_matrix { MSDP_SMAT_W = 0, MSDP_SMAT_G = 1, MSDP_SMAT_SINV = 2, MSDP_SMAT_LS = 3, MSDP_SMAT_LX = 4,
                          MSDP_SMAT_D = 5 };
int msdp_solver_set_iterate(msdp_solver* solver, const double* const* X, const double* const* S, const double* y,
                            const double* x, const double* z);
int msdp_solver_prepare(msdp_solver* solver, int32_t* ok);
int msdp_solver_schur_assemble(msdp_solver* solver, int32_t precision, double* H);
int msdp_solver_get_block_matrix(msdp_solver* solver, int32_t block, int32_t which, double* out);
int msdp_solver_step_eig(msdp_solver* solver, int32_t block, const double* L, const double* D, double* lambda_min);

/* ---- a Schur-solver component (src/components.jl:253-266) ----------------------
 *   msdp_schur_create     schur_workspace(DenseCholesky(), Float64, m)
 *                         (src/schur_solvers.jl:10-14) on the device
 *   msdp_schur_factorize  factorize!(ws) (src/schur_solvers.jl:15-19) of the
 *                         host-assembled H (m x m column-major, lower
 *                         triangle read, Hermitian(H, :L)); *success =
 *                         issuccess
 *   msdp_schur_solve      schur_solve!(ws, rhs) (src/schur_solvers.jl:21):
 *                         rhs (m, host) is overwritten by the solution
 * MSDP_MIXED: FP32-class factor, each solve refined against H in FP64 until
 * the residual stops shrinking; a residual above 1e-11 |rhs| then refactors H
 * in FP64 for the remaining solves of this factorization, and a breakdown of
 * the FP32-class factorization falls back to FP64 at once
 * (msdp_schur_fp64_active reports either). */
typedef struct msdp_schur msdp_schur;
int msdp_schur_create(msdp_context* ctx, int32_t m, int32_t precision, msdp_schur** ws);
int msdp_schur_destroy(msdp_schur* ws);
int msdp_schur_factorize(msdp_schur* ws, const double* H, int32_t* success);
int msdp_schur_solve(msdp_schur* ws, double* rhs);
int msdp_schur_fp64_active(const msdp_schur* ws);

/* ---- split-precision products on the tensor cores ---------------------------
 * C = alpha op(A) op(B) + beta C for column-major float64 device arrays
 * (op = transpose when trans != 0), computed from bf16 slices of A and B on
 * the tcgen05 tensor cores with exact per-chunk accumulation:
 *   precision MSDP_FP64   7 slices, 28 slice products: error about 2e-14 of
 *                         |op(A)||op(B)| (the dense products of the FP64
 *                         whole-GPU path);
 *   precision MSDP_MIXED  3 slices, 6 slice products: about FP32 accuracy
 *                         (the split-precision Schur assembly).
 * lower != 0 (M == N) computes only the entries with row >= column.  This
 * is the dense contraction behind LowRankOpt's schur_complement! for dense
 * constraints (called at src/solver.jl:304) and the products of
 * src/directions.jl:45-100; the entry point allocates its slice buffers per
 * call and synchronizes `stream` (a cudaStream_t, NULL = default). */
int msdp_tc_gemm(int32_t precision, int32_t transa, int32_t transb, int64_t M, int64_t N, int64_t K, double alpha,
                 const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc,
                 int32_t lower, void* stream);

/* DenseCholesky's factorize! (src/schur_solvers.jl:15-19, cholesky! with
 * issuccess) for one dense n x n column-major float64 device matrix: the
 * lower factor overwrites the lower triangle (the strict upper triangle is
 * not touched).  *info = k + 1 for the first pivot k that is not positive
 * and finite, else 0 (LAPACK potrf).  Blocked right-looking factorization
 * whose trailing updates are tensor-core products as in msdp_tc_gemm;
 * MSDP_MIXED gives an FP32-class factor (the refinement-based Schur solve).
 * Allocates its workspace per call and synchronizes `stream`. */
int msdp_dense_cholesky(int32_t precision, int32_t n, double* A, int64_t lda, int32_t* info, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MADSDP_GPU_H */
