// Device-side data layout shared by the kernel (ipm.cuh) and the host code
// (capi.cu).  All problem data and all workspaces of a batch live in a few
// arenas; descriptors hold offsets into them.
#pragma once
#include <stdint.h>

#include "../../include/madsdp_gpu.h"

// ---- FP64 matrices of one block (offsets in units of n*n, from BlockDesc::m64)
enum { M_X = 0, M_S, M_RD, M_DX, M_DS, M_BUF, M_ATY, M_SHAT, M_DC, M_COUNT };
// per-block FP64 scalars after the matrices
enum { BS_RDNZ = 0, BS_COUNT = 8 };

// ---- compute-type workspace of one block (units of n*n, from w64 / w32)
enum {
  W_LS = 0, W_SI, W_LX, W_LSI, W_LXI, W_W, W_G, W_GI, W_RNT, W_CORR,
  W_T1, W_T2, W_T3, W_Q, W_DXT, W_DST, W_XT, W_ERD, W_COUNT
};
// vectors after the matrices (units of n+1): D, lanczos alpha, beta, w, coef, q
enum { WV_D = 0, WV_LA, WV_LB, WV_LW, WV_LC, WV_LA2, WV_LB2, WV_LW2, WV_LC2, WV_EIG, WV_COUNT };

// ---- FP64 vectors of one problem (from ProbDesc::v64)
// m-vectors
enum { V_Y = 0, V_DELY, V_RP, V_H, V_WM, V_WM2, V_DCD, V_DCG, V_DCGZ, V_DCDY, V_DCYHAT, V_MCOUNT };
// ns-vectors
enum { S_X = 0, S_Z, S_DELX, S_DELZ, S_RDLIN, S_ZINV, S_CORR, S_WS, S_WS2, S_COUNT };
// scalars
enum {
  SC_MU = 0, SC_SIGMA, SC_ALPHA, SC_BETA, SC_INFPR, SC_INFDU, SC_GAP, SC_POBJ, SC_DOBJ,
  SC_STATUS, SC_ITER, SC_PHASE, SC_N32, SC_N64, SC_START, SC_SOLVE_NS, SC_BNORM, SC_DNORM,
  SC_CMAX, SC_DC_T, SC_DC_LAM, SC_DC_A, SC_DC_NU, SC_NNEWTON, SC_NPRED, SC_OK, SC_NTRAJ,
  // device cycle counters per phase and work counters (profiling)
  SC_T_CHOL = 32, SC_T_TRTRI, SC_T_JACOBI, SC_T_NTPROD, SC_T_ASSEMBLY, SC_T_FACTOR, SC_T_RHS, SC_T_SOLVE,
  SC_T_DIRECTIONS, SC_T_STEP, SC_T_LANCZOS, SC_T_CORRECTION, SC_T_TAKE, SC_T_TERM, SC_T_ITER,
  SC_N_JACOBI_SWEEPS, SC_N_JACOBI_CALLS, SC_N_LANCZOS_STEPS, SC_N_LANCZOS_CALLS, SC_N_FACTOR,
  SC_PROFILE_END,
  // the counters above hold the FP32 phase; the FP64 phase uses the same
  // fields shifted by SC_PROFILE_F64
  SC_PROFILE_F64 = 24,
  SC_COUNT = 96
};
#define SC_PROFILE_N (SC_PROFILE_END - SC_T_CHOL)
#define TRAJ_FIELDS 10

// Status value written when the initial point cannot be built (the
// reference throws ErrorException, src/solver.jl:280-283).
#define MSDP_STATUS_INITIAL_POINT_ERROR 200

struct ProbDesc {
  int32_t nblocks, m, ns, blk0;
  int64_t bdat;  // data arena: b (m), d_lin (ns), C_lin (m*ns), then ||b||, ||d||, max ||C_i||
  int64_t v64;   // FP64 vectors: V_MCOUNT*m + S_COUNT*ns + SC_COUNT
  int64_t H64;   // FP64 Schur matrix m*m
  int64_t Hf;    // FP32 Schur matrix m*m (mixed), -1 if absent
  int64_t Lf;    // FP32 Schur factor m*m (mixed), -1 if absent
  int64_t traj;  // FP64 trajectory (max_iter+2)*TRAJ_FIELDS
  int32_t ntraj, K;  // K: rows of the QRSchur matrix (sum n(n+1)/2 + ns)
  int64_t qr;    // FP64 QRSchur workspace: B (K*m), tau (m), scale (m), base (K), dir (K); -1 if absent
  int64_t piv;   // FP64 MadNLPSchur pivot record (m), -1 if absent
};

// constraint structure of a block (detected at upload)
enum { STRUCT_GENERAL = 0, STRUCT_HANKEL = 1, STRUCT_DENSE = 2 };

// Schur assembly of one block: Hankel 0/1 constraints by their closed form;
// otherwise entry pairs (cost nnz^2) unless forming T_k = L A_k R per
// constraint and reading A_j(T_k) (cost m (4 n^3 + nnz)) is cheaper.
__host__ __device__ inline int choose_structure(bool hankel, int64_t n, int64_t m, int64_t nnz) {
  if (hankel) return STRUCT_HANKEL;
  const double pairs = (double)nnz * (double)nnz;
  const double cols = (double)m * (4.0 * (double)n * (double)n * (double)n + (double)nnz);
  return pairs > 2.0 * cols ? STRUCT_DENSE : STRUCT_GENERAL;
}

struct BlockDesc {
  int32_t n, structure;
  int64_t nnz;
  int64_t cdat;    // data arena: C (n*n)
  int64_t m64;     // FP64 matrices M_COUNT*n*n + BS_COUNT
  int64_t w64;     // FP64 compute workspace W_COUNT*n*n + WV_COUNT*(n+1)
  int64_t w32;     // FP32 compute workspace (mixed), -1 if absent
  int64_t ent;     // first entry in the coordinate arrays
  int64_t conptr;  // m+1 offsets (relative to ent) in the int64 arena
  int64_t posptr;  // n*n+1 offsets (relative to ent) in the int64 arena
  double cnorm;    // ||C_i||_inf (max-abs entry, src/solver.jl:119-120)
};

struct Params {
  // components
  int32_t algorithm, direction, step, centering, initial_point, schur, precision, centering_max_iter;
  double tau, shrink, boundary, sigma_exponent, initial_ratio, ratio, scale, initial_shift, max_shift;
  double dc_beta, dc_delta, dc_A;
  // options
  double tol, max_wall_time, mu_min, regularize_schur, switch_tol;
  int32_t max_iter, max_schur_reg;
  int32_t mixed_refine, pad1;
  // per-launch arguments
  int32_t op, max_iterations;
  double op_mu;
  int32_t op_corrected, pad;
  double wave_ns;  // OP_ITERATE: stop a problem's iterations once this long after the launch began (0: no limit)
};

enum { OP_INITIALIZE = 0, OP_ITERATE = 1, OP_UPDATE_RESIDUALS = 2, OP_PREPARE = 3,
       OP_SOLVE_DIRECTIONS = 4, OP_CORRECTION = 5 };

struct BatchDev {
  int32_t nprob, pad;
  const ProbDesc* prob;
  const BlockDesc* blk;
  const int32_t* order;   // problem order for the work queue
  const double* dd;  // problem data (uploaded)
  double* d64;       // FP64 workspace (zero-filled on the device)
  float* d32;        // FP32 workspace (mixed)
  const int32_t* e_row;   // by constraint
  const int32_t* e_col;
  const double* e_val;
  const int32_t* p_con;   // by position
  const double* p_val;
  const int64_t* ptr;     // conptr / posptr arena
  int32_t* queue;         // work counter
  // time-sliced waves (OP_ITERATE with prm.wave_ns > 0): problems of this
  // launch that have not yet run their first iteration; a CTA keeps
  // iterating its problem past the time budget until this reaches zero
  int32_t* wave_pending;
  Params prm;
};
