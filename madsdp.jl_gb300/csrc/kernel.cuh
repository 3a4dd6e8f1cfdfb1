// The persistent batch kernel: each CTA takes problems from a work queue
// and runs the requested operation (initialize, iterate, or one of the
// component steps) on each of them.
#pragma once
#include "ipm.cuh"

#define MSDP_EPS 2.220446049250313e-16

namespace {

// ---------------------------------------------------------------- termination
// update_termination!(solver, ::PrimalDual) (src/primal_dual.jl:123-134)
// with _update_infeasibilities! and _update_status! (src/solver.jl:318-347).
__device__ void update_termination(const BatchDev& B, Prob& P, unsigned char* smem, SharedState& sh) {
  Algo<double> A(B, P, smem, sh);
  const Params& prm = B.prm;
  if (prm.algorithm == MSDP_DUAL_CENTERING) A.update_residuals();
  double pobj = 0.0, rdmax = 0.0;
  for (int i = 0; i < P.nblocks; ++i) {
    Blk<double> b = A.blk(i);
    double t = 0.0, r = 0.0;
    for (int64_t k = threadIdx.x; k < b.nn; k += NTHREADS) {
      t = fma(b.C[k], b.X[k], t);
      r = fmax(r, fabs(b.Rd[k]));
    }
    pobj += block_sum(t, &sh.rb);
    rdmax = fmax(rdmax, block_max(r, &sh.rb));
  }
  double t = 0.0, r = 0.0;
  for (int k = threadIdx.x; k < P.ns; k += NTHREADS) {
    t = fma(P.dlin[k], P.x[k], t);
    r = fmax(r, fabs(P.Rdlin[k]));
  }
  pobj += block_sum(t, &sh.rb);
  rdmax = fmax(rdmax, block_max(r, &sh.rb));
  double d = 0.0, rp = 0.0;
  for (int j = threadIdx.x; j < P.m; j += NTHREADS) {
    d = fma(P.b[j], P.y[j], d);
    rp = fmax(rp, fabs(P.Rp[j]));
  }
  const double dobj = block_sum(d, &sh.rb);
  rp = block_max(rp, &sh.rb);
  if (threadIdx.x == 0) {
    double* sc = P.sc;
    const double inf_pr = rp / fmax(1.0, sc[SC_BNORM]);
    double cn = sc[SC_CMAX];
    if (P.ns > 0) cn = fmax(cn, sc[SC_DNORM]);
    const double inf_du = rdmax / fmax(1.0, cn);
    double gap;
    if (prm.algorithm == MSDP_DUAL_CENTERING)
      gap = sc[SC_DC_NU] / fmax(sc[SC_DC_T], MSDP_EPS) / fmax(1.0, fabs(pobj) + fabs(dobj));
    else
      gap = fabs(pobj - dobj) / fmax(1.0, fabs(pobj) + fabs(dobj));
    sc[SC_POBJ] = pobj; sc[SC_DOBJ] = dobj;
    sc[SC_INFPR] = inf_pr; sc[SC_INFDU] = inf_du; sc[SC_GAP] = gap;
    const bool converged = (prm.algorithm == MSDP_DUAL_CENTERING)
                               ? (gap <= prm.tol)
                               : (fmax(fmax(inf_pr, inf_du), gap) <= prm.tol);
    const double elapsed = (double)(globaltimer_ns() - (uint64_t)sc[SC_START]) * 1e-9;
    int status = (int)sc[SC_STATUS];
    if (converged) status = MSDP_SOLVE_SUCCEEDED;
    else if (sc[SC_ITER] >= (double)prm.max_iter) status = MSDP_MAXIMUM_ITERATIONS_EXCEEDED;
    else if (elapsed >= prm.max_wall_time) status = MSDP_MAXIMUM_WALLTIME_EXCEEDED;
    if (prm.algorithm != MSDP_DUAL_CENTERING && status == MSDP_REGULAR && sc[SC_MU] < prm.mu_min)
      status = MSDP_SEARCH_DIRECTION_BECOMES_TOO_SMALL;
    sc[SC_STATUS] = (double)status;
    if (status != MSDP_REGULAR) sc[SC_SOLVE_NS] = (double)(globaltimer_ns() - (uint64_t)sc[SC_START]);
    const int kt = (int)sc[SC_NTRAJ];
    if (kt < P.ntraj) {
      double* rec = P.traj + (int64_t)kt * TRAJ_FIELDS;
      rec[0] = sc[SC_ITER]; rec[1] = pobj; rec[2] = dobj; rec[3] = inf_pr; rec[4] = inf_du;
      rec[5] = gap; rec[6] = sc[SC_MU]; rec[7] = sc[SC_ALPHA]; rec[8] = sc[SC_BETA]; rec[9] = sc[SC_PHASE];
      sc[SC_NTRAJ] = kt + 1;
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------- initialize!
// initial_point! (src/solver.jl:213-284) and initialize_algorithm!
// (src/primal_dual.jl:21-25).  Returns false if no initial point exists.
__device__ bool initialize(const BatchDev& B, Prob& P, unsigned char* smem, SharedState& sh) {
  Algo<double> A(B, P, smem, sh);
  const Params& prm = B.prm;
  const int nu = A.nu();
  if (prm.initial_point == MSDP_SCALED_IDENTITY) {
    double beta = prm.scale;
    if (!(beta > 0.0)) {
      double cs = P.norms[2];
      if (P.ns > 0) cs = fmax(cs, P.norms[1]);
      beta = fmax(10.0, sqrt(fmax(P.norms[0], 1.0) * fmax(cs, 1.0)) * sqrt((double)nu));
    }
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<double> b = A.blk(i);
      cta_set_identity<double>(b.n, b.X, beta);
      cta_set_identity<double>(b.n, b.S, beta);
    }
    for (int j = threadIdx.x; j < P.m; j += NTHREADS) P.y[j] = 0.0;
    for (int k = threadIdx.x; k < P.ns; k += NTHREADS) { P.x[k] = beta; P.z[k] = beta; }
    __syncthreads();
  } else if (prm.initial_point == MSDP_INITIAL_POINT) {
    // X, y, x were written by the host.
    A.set_dual_slacks();
  } else {  // DualShift
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<double> b = A.blk(i);
      cta_set_identity<double>(b.n, b.X, 1.0);
    }
    for (int k = threadIdx.x; k < P.ns; k += NTHREADS) P.x[k] = 1.0;
    __syncthreads();
    double rho = 0.0;
    bool found = false;
    // rho doubles each round; the round cap bounds the loop for any options
    for (int round = 0; round < 4096 && rho <= prm.max_shift; ++round) {
      for (int j = threadIdx.x; j < P.m; j += NTHREADS) P.y[j] = -rho;
      __syncthreads();
      A.set_dual_slacks();
      bool interior = true;
      for (int i = 0; i < P.nblocks && interior; ++i) {
        Blk<double> b = A.blk(i);
        interior = chol_factor<double, double>(b.n, b.S, b.W(W_LS), true, smem, sh);
      }
      if (interior) {
        int neg = 0;
        for (int k = threadIdx.x; k < P.ns; k += NTHREADS) neg |= !(P.z[k] > 0.0);
        neg = __syncthreads_or(neg);
        interior = !neg;
      }
      if (interior) {
        if (rho != 0.0) {
          for (int j = threadIdx.x; j < P.m; j += NTHREADS) P.y[j] = -2.0 * rho;
          __syncthreads();
          A.set_dual_slacks();
        }
        found = true;
        break;
      }
      rho = (rho == 0.0) ? prm.initial_shift : 2.0 * rho;
    }
    if (!found) return false;
  }
  if (threadIdx.x == 0) {
    P.sc[SC_BNORM] = P.norms[0];
    P.sc[SC_DNORM] = P.norms[1];
    P.sc[SC_CMAX] = P.norms[2];
    P.sc[SC_ITER] = 0.0;
    P.sc[SC_STATUS] = (double)MSDP_REGULAR;
    P.sc[SC_START] = (double)globaltimer_ns();
    P.sc[SC_NTRAJ] = 0.0;
    P.sc[SC_PHASE] = prm.precision == MSDP_MIXED ? 0.0 : 1.0;
    P.sc[SC_N32] = 0.0; P.sc[SC_N64] = 0.0;
    P.sc[SC_ALPHA] = 0.0; P.sc[SC_BETA] = 0.0; P.sc[SC_SIGMA] = 0.0;
    P.sc[SC_INFPR] = INFINITY; P.sc[SC_INFDU] = INFINITY; P.sc[SC_GAP] = INFINITY;
    for (int k = SC_T_CHOL; k < SC_PROFILE_END; ++k) { P.sc[k] = 0.0; P.sc[k + SC_PROFILE_F64] = 0.0; }
  }
  __syncthreads();
  if (prm.algorithm == MSDP_DUAL_CENTERING) return A.dc_initialize();
  // initialize_algorithm!(solver, ::PrimalDual)
  A.update_residuals();
  const double mu = A.total_complementarity() / fmax((double)nu, 1.0);
  if (threadIdx.x == 0)
    P.sc[SC_MU] = (prm.centering == MSDP_ADAPTIVE_MU) ? prm.initial_ratio * mu : mu;
  __syncthreads();
  return true;
}

// ---------------------------------------------------------------- one iteration
template <int MIXED>
__device__ void iterate_one(const BatchDev& B, Prob& P, unsigned char* smem, SharedState& sh) {
  const Params& prm = B.prm;
  if (prm.algorithm == MSDP_DUAL_CENTERING) {
    Algo<double> A(B, P, smem, sh);
    A.dc_iterate();
    return;
  }
  if constexpr (MIXED != 0) {
    int phase = (int)P.sc[SC_PHASE];
    if (phase == 0 && fmax(fmax(P.sc[SC_INFPR], P.sc[SC_INFDU]), P.sc[SC_GAP]) < prm.switch_tol) phase = 1;
    if (prm.schur != MSDP_DENSE_CHOLESKY) phase = 1;  // the FP32 phase factors by Cholesky only
    if (phase == 0) {
      const double pr_old = P.sc[SC_INFPR];
      Algo<float> A(B, P, smem, sh);
      const bool ok = A.iterate_pd(false);
      if (ok) {
        // The dual residual update is exact in float64 (dS = Rd - A*(dy));
        // the primal one is not: Rp_new = (1 - a) Rp - a (A(dX) - Rp).  If
        // the estimated error of the FP32 direction exceeds 10% of the
        // residual it had to remove, later iterations run in FP64.
        double rp = 0.0;
        for (int j = threadIdx.x; j < P.m; j += NTHREADS) rp = fmax(rp, fabs(P.Rp[j]));
        rp = block_max(rp, &sh.rb) / fmax(1.0, P.sc[SC_BNORM]);
        const double a = P.sc[SC_ALPHA];
        const double err = fmax(0.0, rp - (1.0 - a) * pr_old) / fmax(a, 1e-300);
        if (threadIdx.x == 0) {
          P.sc[SC_N32] += 1.0;
          // a primal residual already below a tenth of the tolerance needs no
          // more accuracy than FP32 gives
          if (err > fmax(0.1 * pr_old, 0.1 * prm.tol)) P.sc[SC_PHASE] = 1.0;
        }
        __syncthreads();
        return;
      }
      phase = 1;  // FP32 failed or stalled: this and later iterations in FP64
    }
    if (threadIdx.x == 0) P.sc[SC_PHASE] = (double)phase;
    __syncthreads();
  }
  Algo<double> A(B, P, smem, sh);
  const bool ok = A.iterate_pd(true);
  if (threadIdx.x == 0) {
    P.sc[SC_N64] += 1.0;
    if (!ok) P.sc[SC_STATUS] = (double)MSDP_ERROR_IN_STEP_COMPUTATION;
  }
  __syncthreads();
}

template <int MIXED>
__device__ void run_op(const BatchDev& B, Prob& P, unsigned char* smem, SharedState& sh) {
  const Params& prm = B.prm;
  switch (prm.op) {
    case OP_INITIALIZE: {
      const bool ok = initialize(B, P, smem, sh);
      if (!ok) {
        if (threadIdx.x == 0) P.sc[SC_STATUS] = (double)MSDP_STATUS_INITIAL_POINT_ERROR;
        __syncthreads();
        return;
      }
      update_termination(B, P, smem, sh);
      break;
    }
    case OP_ITERATE: {
      bool counted = false;  // this problem's first iteration reported to wave_pending
      for (int k = 0; (prm.max_iterations <= 0 || k < prm.max_iterations) && k < 1000000; ++k) {
        if (k > 0 && B.wave_pending && !counted) {
          if (threadIdx.x == 0) atomicSub(B.wave_pending, 1);
          counted = true;
        }
        if ((int)P.sc[SC_STATUS] != MSDP_REGULAR) break;
        if (k > 0 && prm.wave_ns > 0.0) {
          // time-sliced waves: at least one iteration, then stop once the
          // launch has run wave_ns and every problem of the launch has run
          // its first iteration (decided by thread 0 for the whole CTA; no
          // waiting: until then the CTA keeps iterating its own problem)
          if (threadIdx.x == 0) {
            const bool late = (double)(globaltimer_ns() - sh.t0) >= prm.wave_ns;
            sh.stop = late && (!B.wave_pending || atomicAdd(B.wave_pending, 0) <= 0);
          }
          __syncthreads();
          const int stop = sh.stop;
          __syncthreads();
          if (stop) break;
        }
        const long long t_it = clock64();
        iterate_one<MIXED>(B, P, smem, sh);
        if (threadIdx.x == 0) P.sc[SC_T_ITER] += (double)(clock64() - t_it);
        if ((int)P.sc[SC_STATUS] != MSDP_REGULAR) break;
        const long long t_tm = clock64();
        update_termination(B, P, smem, sh);
        if (threadIdx.x == 0) P.sc[SC_T_TERM] += (double)(clock64() - t_tm);
      }
      if (B.wave_pending && !counted && threadIdx.x == 0) atomicSub(B.wave_pending, 1);
      break;
    }
    case OP_UPDATE_RESIDUALS: {
      Algo<double> A(B, P, smem, sh);
      A.update_residuals();
      break;
    }
    case OP_PREPARE: {
      Algo<double> A(B, P, smem, sh);
      const bool ok = A.prepare() && A.factorize_schur();
      if (threadIdx.x == 0) P.sc[SC_OK] = ok ? 1.0 : 0.0;
      __syncthreads();
      break;
    }
    case OP_SOLVE_DIRECTIONS: {
      Algo<double> A(B, P, smem, sh);
      A.solve_directions(prm.op_mu, prm.op_corrected != 0);
      break;
    }
    case OP_CORRECTION: {
      Algo<double> A(B, P, smem, sh);
      A.correction();
      break;
    }
    default:
      break;
  }
}

template <int MIXED>
#ifndef MSDP_MIN_CTAS
#define MSDP_MIN_CTAS 3
#endif
__global__ void __launch_bounds__(NTHREADS, MSDP_MIN_CTAS) msdp_ipm_kernel(const __grid_constant__ BatchDev B) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ SharedState sh;
  if (threadIdx.x == 0) sh.t0 = globaltimer_ns();
  for (;;) {
    if (threadIdx.x == 0) {
      const int q = atomicAdd(B.queue, 1);
      sh.prob = q < B.nprob ? B.order[q] : -1;
    }
    __syncthreads();
    const int p = sh.prob;
    __syncthreads();
    if (p < 0) break;
    Prob P = make_prob(B, p);
    run_op<MIXED>(B, P, smem, sh);
    __syncthreads();
  }
}

#ifdef MSDP_DEFINE_GATHER
// Copy the scalar block of every problem into out[nprob * SC_COUNT].
__global__ void msdp_gather_scalars(const __grid_constant__ BatchDev B, double* out) {
  const int p = blockIdx.x;
  if (p >= B.nprob) return;
  Prob P = make_prob(B, p);
  for (int k = threadIdx.x; k < SC_COUNT; k += blockDim.x) out[(int64_t)p * SC_COUNT + k] = P.sc[k];
}

// Copy the scalar blocks of the listed problems into out[count * SC_COUNT].
__global__ void msdp_gather_scalars_idx(const __grid_constant__ BatchDev B, const int32_t* idx, double* out) {
  const int q = blockIdx.x;
  Prob P = make_prob(B, idx[q]);
  for (int k = threadIdx.x; k < SC_COUNT; k += blockDim.x) out[(int64_t)q * SC_COUNT + k] = P.sc[k];
}
#endif

}  // namespace
