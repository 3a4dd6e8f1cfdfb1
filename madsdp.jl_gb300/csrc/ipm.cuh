// The interior-point iteration of MadSDP as CTA-cooperative device code.
//
// One CTA owns one problem at a time and runs its whole iteration: the
// block factorizations and NT/HKM scalings, the Schur complement assembly,
// its Cholesky factorization and solves, the directions, the step lengths
// and the update.  Each function names the reference function it follows
// (paths relative to blegat/MadSDP.jl).
//
// The iterate (X, S, y, x, z), the residuals and every quantity that enters
// a residual or an objective are float64.  The template parameter T is the
// type of the block linear algebra (factorizations, scalings, E(.), the
// Schur matrix): double for the FP64 path, float for the FP32 phase of the
// mixed path.
#pragma once
#include "la.cuh"
#include "layout.h"

#ifndef MSDP_SMEM_BYTES
#ifndef MSDP_SMEM_KB
#define MSDP_SMEM_KB 72
#endif
#define MSDP_SMEM_BYTES (MSDP_SMEM_KB * 1024)
#endif

// Device code of one translation unit: internal linkage.
namespace {

struct SharedState {
  RedBuf rb;
  int flag;
  int counter;
  int prob;
  int stop;
  int erd64;     // FP32 phase: E(Rd) in float64 formed for this iteration
  int pad2;
  double bc[8];  // broadcast scalars
  uint64_t t0;   // launch start on this CTA (globaltimer)
};

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Per-phase device cycle counters (thread 0 accumulates into the scalars).
#define PROF_BEGIN(tag) const long long prof_##tag = clock64()
#define PROF_SHIFT (sizeof(T) == 8 ? SC_PROFILE_F64 : 0)
#define PROF_END(tag, slot)                                                         \
  do {                                                                              \
    if (threadIdx.x == 0) P.sc[(slot) + PROF_SHIFT] += (double)(clock64() - prof_##tag); \
  } while (0)
#define PROF_COUNT(slot, v)                                                         \
  do {                                                                              \
    if (threadIdx.x == 0) P.sc[(slot) + PROF_SHIFT] += (double)(v);                 \
  } while (0)

// ------------------------------------------------------------------ views
struct Prob {
  int p, nblocks, m, ns;
  double *b, *y, *dely, *Rp, *h, *wm, *wm2, *dcd, *dcg, *dcgz, *dcdy, *dcyhat;
  double *dlin, *x, *z, *delx, *delz, *Rdlin, *zinv, *corrlin, *ws, *ws2;
  double* Clin;  // m x ns column-major
  const double* norms;  // ||b||_inf, ||d_lin||_inf, max_i ||C_i||_inf
  double* sc;
  double* H64;
  float *Hf, *Lf;
  double* traj;
  int ntraj;
  int K;
  double *qrB, *qrtau, *qrscale, *qrbase, *qrdir;
  double* piv;
};

__device__ __forceinline__ Prob make_prob(const BatchDev& B, int p) {
  const ProbDesc& d = B.prob[p];
  Prob P;
  P.p = p; P.nblocks = d.nblocks; P.m = d.m; P.ns = d.ns;
  double* v = B.d64 + d.v64;
  const int m = d.m, ns = d.ns;
  const double* dat = B.dd + d.bdat;
  P.b = const_cast<double*>(dat);
  P.dlin = const_cast<double*>(dat + m);
  P.Clin = const_cast<double*>(dat + m + ns);
  P.norms = dat + m + ns + (int64_t)m * ns;
  P.y = v + (int64_t)V_Y * m; P.dely = v + (int64_t)V_DELY * m;
  P.Rp = v + (int64_t)V_RP * m; P.h = v + (int64_t)V_H * m; P.wm = v + (int64_t)V_WM * m;
  P.wm2 = v + (int64_t)V_WM2 * m; P.dcd = v + (int64_t)V_DCD * m; P.dcg = v + (int64_t)V_DCG * m;
  P.dcgz = v + (int64_t)V_DCGZ * m; P.dcdy = v + (int64_t)V_DCDY * m; P.dcyhat = v + (int64_t)V_DCYHAT * m;
  double* s = v + (int64_t)V_MCOUNT * m;
  P.x = s + (int64_t)S_X * ns; P.z = s + (int64_t)S_Z * ns;
  P.delx = s + (int64_t)S_DELX * ns; P.delz = s + (int64_t)S_DELZ * ns; P.Rdlin = s + (int64_t)S_RDLIN * ns;
  P.zinv = s + (int64_t)S_ZINV * ns; P.corrlin = s + (int64_t)S_CORR * ns; P.ws = s + (int64_t)S_WS * ns;
  P.ws2 = s + (int64_t)S_WS2 * ns;
  P.sc = s + (int64_t)S_COUNT * ns;
  P.H64 = B.d64 + d.H64;
  P.Hf = d.Hf >= 0 ? B.d32 + d.Hf : nullptr;
  P.Lf = d.Lf >= 0 ? B.d32 + d.Lf : nullptr;
  P.traj = B.d64 + d.traj;
  P.ntraj = d.ntraj;
  P.K = d.K;
  if (d.qr >= 0) {
    P.qrB = B.d64 + d.qr;
    P.qrtau = P.qrB + (int64_t)d.K * m;
    P.qrscale = P.qrtau + m;
    P.qrbase = P.qrscale + m;
    P.qrdir = P.qrbase + d.K;
  } else {
    P.qrB = P.qrtau = P.qrscale = P.qrbase = P.qrdir = nullptr;
  }
  P.piv = d.piv >= 0 ? B.d64 + d.piv : nullptr;
  return P;
}

template <class T>
struct Blk {
  int n;
  int64_t nn;
  double *C, *base, *X, *S, *Rd, *dX, *dS, *buf, *ATy, *Shat, *Dc, *bsc;
  T* w;
  int64_t nnz;
  const int32_t *erow, *ecol, *pcon;
  const double *eval, *pval;
  const int64_t *cptr, *pptr;
  double cnorm;
  int structure;
  int index;
  __device__ __forceinline__ T* W(int k) const { return w + (int64_t)k * nn; }
  __device__ __forceinline__ T* V(int k) const { return w + (int64_t)W_COUNT * nn + (int64_t)k * (n + 1); }
  __device__ __forceinline__ double* M(int k) const { return base + (int64_t)k * nn; }
};

template <class T> __device__ __forceinline__ T* wbase(const BatchDev& B, const BlockDesc& d);
template <> __device__ __forceinline__ double* wbase<double>(const BatchDev& B, const BlockDesc& d) { return B.d64 + d.w64; }
template <> __device__ __forceinline__ float* wbase<float>(const BatchDev& B, const BlockDesc& d) { return B.d32 + d.w32; }

template <class T>
__device__ __forceinline__ Blk<T> make_blk(const BatchDev& B, const Prob& P, int i) {
  const BlockDesc& d = B.blk[B.prob[P.p].blk0 + i];
  Blk<T> b;
  b.n = d.n; b.nn = (int64_t)d.n * d.n;
  b.C = const_cast<double*>(B.dd + d.cdat);
  b.base = B.d64 + d.m64;
  b.X = b.M(M_X); b.S = b.M(M_S); b.Rd = b.M(M_RD); b.dX = b.M(M_DX); b.dS = b.M(M_DS);
  b.buf = b.M(M_BUF); b.ATy = b.M(M_ATY); b.Shat = b.M(M_SHAT); b.Dc = b.M(M_DC);
  b.bsc = b.base + (int64_t)M_COUNT * b.nn;
  b.w = wbase<T>(B, d);
  b.nnz = d.nnz;
  b.erow = B.e_row + d.ent; b.ecol = B.e_col + d.ent; b.eval = B.e_val + d.ent;
  b.pcon = B.p_con + d.ent; b.pval = B.p_val + d.ent;
  b.cptr = B.ptr + d.conptr; b.pptr = B.ptr + d.posptr;
  b.cnorm = d.cnorm;
  b.structure = d.structure;
  b.index = i;
  return b;
}

// "T view" of a float64 array: the array itself for T = double, else a
// converted copy in `slot`.
template <class T> __device__ __forceinline__ T* as_T(int64_t len, const double* src, T* slot);
template <> __device__ __forceinline__ double* as_T<double>(int64_t, const double* src, double*) {
  return const_cast<double*>(src);
}
template <> __device__ __forceinline__ float* as_T<float>(int64_t len, const double* src, float* slot) {
  cta_convert<float, double>(len, slot, src);
  return slot;
}

// ------------------------------------------------------------------ A(.) and A*(.)
// out[j] += <A_ij, X_i> (LowRankOpt.add_jprod!, src/step.jl:19)
template <class T, class U>
__device__ void jprod_add(const Blk<T>& b, int m, const U* X, double* out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int j = warp; j < m; j += NWARPS) {
    const int64_t s = b.cptr[j], e = b.cptr[j + 1];
    double acc = 0.0;
    for (int64_t q = s + lane; q < e; q += 32)
      acc = fma(b.eval[q], (double)X[b.erow[q] + (int64_t)b.ecol[q] * b.n], acc);
    acc = warp_sum(acc);
    if (lane == 0) out[j] += acc;
  }
  __syncthreads();
}

// out = base1 - base2 + sgn * A_i*(y) (LowRankOpt.unsafe_jtprod, src/step.jl:30).
template <class T>
__device__ void jtprod_combine(const Blk<T>& b, const double* y, double sgn, const double* base1,
                               const double* base2, double* out) {
  for (int64_t k = threadIdx.x; k < b.nn; k += NTHREADS) {
    double s = 0.0;
    const int64_t q1 = b.pptr[k + 1];
    for (int64_t q = b.pptr[k]; q < q1; ++q) s = fma(y[b.pcon[q]], b.pval[q], s);
    double v = base1 ? base1[k] : 0.0;
    if (base2) v -= base2[k];
    out[k] = v + sgn * s;
  }
  __syncthreads();
}

// out += sgn * C_lin * v   (m)      /   out = base + sgn * C_lin' v  (ns)
__device__ void clin_mv(const Prob& P, const double* v, double sgn, double* out) {
  for (int j = threadIdx.x; j < P.m; j += NTHREADS) {
    double s = 0.0;
    for (int k = 0; k < P.ns; ++k) s = fma(P.Clin[j + (int64_t)k * P.m], v[k], s);
    out[j] += sgn * s;
  }
  __syncthreads();
}
__device__ void clin_tmv(const Prob& P, const double* v, const double* base, double sgn, double* out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = warp; k < P.ns; k += NWARPS) {
    double s = 0.0;
    for (int j = lane; j < P.m; j += 32) s = fma(P.Clin[j + (int64_t)k * P.m], v[j], s);
    s = warp_sum(s);
    if (lane == 0) out[k] = (base ? base[k] : 0.0) + sgn * s;
  }
  __syncthreads();
}

// ------------------------------------------------------------------ block helpers
// L = chol(sym(M)) with the flush of src/blocks.jl:94-113 (flush = true),
// or a plain positive-definiteness test (out = nullptr).
template <class T, class U>
__device__ bool chol_factor(int n, const U* M, T* out, bool flush, unsigned char* smem, SharedState& sh) {
  const int64_t nn = (int64_t)n * n;
  T* A = (nn * (int64_t)sizeof(T) <= MSDP_SMEM_BYTES) ? (T*)smem : out;
  cta_sym_copy<T, U>(n, A, M);
  if (!cta_potrf<T>(n, A, n, &sh.flag)) return false;
  if (out == nullptr) return true;
  if (flush) cta_flush_lower<T>(n, A, n, &sh.rb);
  if (A != out) {
    for (int64_t k = threadIdx.x; k < nn; k += NTHREADS) out[k] = A[k];
    __syncthreads();
  }
  return true;
}

// Whether X + a dX is positive definite (src/blocks.jl:133-137); `work` is
// an n x n T buffer used when shared memory is too small.
template <class T>
__device__ bool add_mul_posdef(int n, const double* X, double a, const double* dX, T* work,
                               unsigned char* smem, SharedState& sh) {
  const int64_t nn = (int64_t)n * n;
  T* A = (nn * (int64_t)sizeof(T) <= MSDP_SMEM_BYTES) ? (T*)smem : work;
  for (int64_t k = threadIdx.x; k < nn; k += NTHREADS) A[k] = (T)(X[k] + a * dX[k]);
  __syncthreads();
  return cta_potrf<T>(n, A, n, &sh.flag);
}

template <class T>
__device__ void tri_inverse(int n, const T* L, T* Li, unsigned char* smem) {
  const int64_t nn = (int64_t)n * n;
  if (2 * nn * (int64_t)sizeof(T) <= MSDP_SMEM_BYTES) {
    T* sL = (T*)smem;
    T* sLi = sL + nn;
    for (int64_t k = threadIdx.x; k < nn; k += NTHREADS) sL[k] = L[k];
    __syncthreads();
    cta_trtri_lower<T>(n, sL, sLi);
    for (int64_t k = threadIdx.x; k < nn; k += NTHREADS) Li[k] = sLi[k];
    __syncthreads();
  } else {
    cta_trtri_lower<T>(n, L, Li);
  }
}

// ------------------------------------------------------------------ Lanczos
// Smallest eigenvalue of the symmetric Z (n x n) by Lanczos with full
// reorthogonalization (the role of LowRankOpt.lanczos_eigmin!,
// src/step.jl:151-183).  Q (n x n) holds the basis; a, bb, w, coef are
// vectors of length n+1.  Stops when the smallest Ritz value is stable or
// the Krylov space is exhausted.
template <class T>
__device__ T lanczos_eigmin(int n, const T* Z, T* Q, T* a, T* bb, T* w, T* coef, SharedState& sh, int* steps) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // deterministic pseudo-random start vector
  double nrm2 = 0.0;
  for (int i = threadIdx.x; i < n; i += NTHREADS) {
    uint32_t hsh = (uint32_t)(i + 1) * 2654435761u;
    hsh ^= hsh >> 15; hsh *= 2246822519u; hsh ^= hsh >> 13;
    const T v = (T)((double)(hsh & 0xffffff) / 16777216.0 - 0.5) + (T)0.01;
    Q[i] = v;
    nrm2 += (double)v * v;
  }
  nrm2 = block_sum(nrm2, &sh.rb);
  {
    const T inv = (T)(1.0 / sqrt(nrm2));
    for (int i = threadIdx.x; i < n; i += NTHREADS) Q[i] *= inv;
    __syncthreads();
  }
  *steps = 0;
  T theta = (T)0, theta_prev = (T)INFINITY;
  T znorm = (T)0;
  int k = 0;
  for (int j = 0; j < n; ++j) {
    const T* qj = Q + (int64_t)j * n;
    // w = Z q_j (Z symmetric: w_i = column i . q_j)
    for (int i = warp; i < n; i += NWARPS) {
      const T* zi = Z + (int64_t)i * n;
      T s = 0;
      for (int r = lane; r < n; r += 32) s = fma(zi[r], qj[r], s);
      s = warp_sum(s);
      if (lane == 0) w[i] = s;
    }
    __syncthreads();
    double aj = 0.0;
    for (int i = threadIdx.x; i < n; i += NTHREADS) aj += (double)qj[i] * w[i];
    aj = block_sum(aj, &sh.rb);
    if (threadIdx.x == 0) a[j] = (T)aj;
    {
      const T* qp = j > 0 ? Q + (int64_t)(j - 1) * n : nullptr;
      const T bj = j > 0 ? bb[j] : (T)0;
      for (int i = threadIdx.x; i < n; i += NTHREADS) {
        T v = w[i] - (T)aj * qj[i];
        if (qp) v -= bj * qp[i];
        w[i] = v;
      }
      __syncthreads();
    }
    // full reorthogonalization, twice
    for (int pass = 0; pass < 2; ++pass) {
      for (int l = warp; l <= j; l += NWARPS) {
        const T* ql = Q + (int64_t)l * n;
        T s = 0;
        for (int r = lane; r < n; r += 32) s = fma(ql[r], w[r], s);
        s = warp_sum(s);
        if (lane == 0) coef[l] = s;
      }
      __syncthreads();
      for (int i = threadIdx.x; i < n; i += NTHREADS) {
        T v = w[i];
        for (int l = 0; l <= j; ++l) v = fma(-coef[l], Q[i + (int64_t)l * n], v);
        w[i] = v;
      }
      __syncthreads();
    }
    double bn = 0.0;
    for (int i = threadIdx.x; i < n; i += NTHREADS) bn += (double)w[i] * w[i];
    bn = sqrt(block_sum(bn, &sh.rb));
    k = j + 1;
    *steps = k;
    if (threadIdx.x == 0) {
      znorm = fmax(znorm, fabs(a[j]) + (T)bn + (j > 0 ? fabs(bb[j]) : (T)0));
      if (j + 1 <= n) bb[j + 1] = (T)bn;
    }
    // broadcast znorm through shared memory
    if (threadIdx.x == 0) sh.bc[0] = (double)znorm;
    __syncthreads();
    znorm = (T)sh.bc[0];
    const bool exhausted = (k == n) || !(bn > (double)Num<T>::eps() * (double)znorm * 4.0);
    const bool check = exhausted || (k >= 4 && (k % 4) == 0);
    if (check) {
      if (warp == 0) {
        const T th = warp_tridiag_eigmin<T>(k, a, bb);
        if (lane == 0) sh.bc[1] = (double)th;
      }
      __syncthreads();
      theta = (T)sh.bc[1];
      __syncthreads();
      const T tolr = (T)(Num<T>::eps() * 64) * fmax((T)1, fabs(theta));
      if (exhausted || fabs(theta - theta_prev) <= tolr) break;
      theta_prev = theta;
    }
    // q_{j+1} = w / b_{j+1}
    T* qn = Q + (int64_t)(j + 1) * n;
    const T inv = (T)(1.0 / bn);
    for (int i = threadIdx.x; i < n; i += NTHREADS) qn[i] = w[i] * inv;
    __syncthreads();
  }
  return theta;
}

// (j, k) with j >= k of the idx-th entry of a packed lower triangle (row major).
__device__ __forceinline__ void tri_index(int64_t idx, int& j, int& k) {
  int r = (int)((sqrt(8.0 * (double)idx + 1.0) - 1.0) * 0.5);
  while ((int64_t)(r + 1) * (r + 2) / 2 <= idx) ++r;
  while ((int64_t)r * (r + 1) / 2 > idx) --r;
  j = r;
  k = (int)(idx - (int64_t)r * (r + 1) / 2);
}

// ------------------------------------------------------------------ algorithm
template <class T>
struct Algo {
  const BatchDev& B;
  const Params& prm;
  Prob& P;
  unsigned char* smem;
  SharedState& sh;

  __device__ Algo(const BatchDev& B_, Prob& P_, unsigned char* smem_, SharedState& sh_)
      : B(B_), prm(B_.prm), P(P_), smem(smem_), sh(sh_) {}

  __device__ __forceinline__ Blk<T> blk(int i) const { return make_blk<T>(B, P, i); }
  // the whole shared-memory scratch (callers hold nothing there)
  __device__ __forceinline__ Scratch scr() const { return Scratch{smem, MSDP_SMEM_BYTES}; }
  __device__ __forceinline__ int blk_index(const Blk<T>& b) const { return b.index; }
  __device__ __forceinline__ int nu() const {
    int s = P.ns;
    for (int i = 0; i < P.nblocks; ++i) s += B.blk[B.prob[P.p].blk0 + i].n;
    return s;
  }
  // X in the compute type: X itself for double, the converted copy for float
  __device__ __forceinline__ const T* xt(const Blk<T>& b) const;
  __device__ __forceinline__ bool is_nt() const {
    return prm.algorithm == MSDP_PRIMAL_DUAL && prm.direction == MSDP_NT;
  }

  // ---------------- residuals (src/step.jl:12-47)
  __noinline__ __device__ void update_residuals() {
    for (int j = threadIdx.x; j < P.m; j += NTHREADS) P.Rp[j] = 0.0;
    __syncthreads();
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      jprod_add(b, P.m, b.X, P.Rp);
    }
    if (P.ns > 0) clin_mv(P, P.x, 1.0, P.Rp);
    for (int j = threadIdx.x; j < P.m; j += NTHREADS) P.Rp[j] = P.b[j] - P.Rp[j];
    __syncthreads();
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      jtprod_combine(b, P.y, -1.0, b.C, b.S, b.Rd);
      double mx = 0.0;
      for (int64_t k = threadIdx.x; k < b.nn; k += NTHREADS) mx = fmax(mx, fabs(b.Rd[k]));
      mx = block_max(mx, &sh.rb);
      if (threadIdx.x == 0) b.bsc[BS_RDNZ] = (mx > 100.0 * 2.220446049250313e-16 * fmax(1.0, b.cnorm)) ? 1.0 : 0.0;
      __syncthreads();
    }
    if (P.ns > 0) {
      clin_tmv(P, P.y, nullptr, 1.0, P.Rdlin);
      for (int k = threadIdx.x; k < P.ns; k += NTHREADS) P.Rdlin[k] = P.dlin[k] - P.z[k] - P.Rdlin[k];
      __syncthreads();
    }
  }

  __device__ double total_complementarity() {
    double s = 0.0;
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      double t = 0.0;
      for (int64_t k = threadIdx.x; k < b.nn; k += NTHREADS) t = fma(b.X[k], b.S[k], t);
      s += block_sum(t, &sh.rb);
    }
    if (P.ns > 0) {
      double t = 0.0;
      for (int k = threadIdx.x; k < P.ns; k += NTHREADS) t = fma(P.x[k], P.z[k], t);
      s += block_sum(t, &sh.rb);
    }
    return s;
  }

  // ---------------- S = sym(C - A*(y)), z = d - C_lin' y (src/solver.jl:192-211)
  __device__ void slack(const Blk<T>& b, const double* y, double* out) {
    jtprod_combine(b, y, -1.0, b.C, nullptr, out);
    cta_symmetrize<double>(b.n, out);
  }
  __device__ void set_dual_slacks() {
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      slack(b, P.y, b.S);
    }
    if (P.ns > 0) clin_tmv(P, P.y, P.dlin, -1.0, P.z);
  }

  // ---------------- _prepare! (src/primal_dual.jl:29-37)
  // NT scaling (src/directions.jl:45-75).  With M = Ls' Lx and the
  // one-sided Jacobi SVD M V = U diag(D) (so N = M'M = V diag(D)^2 V'), the
  // rotations are also applied to Lx, which yields Lx V directly; then
  //   G  = Lx V D^-1/2,   Gi = D^1/2 V' Lx^-1 = D^-3/2 (M V)' Ls',
  //   W  = G G',          S^-1 = G D^-1 G'   (since G' S G = D),
  // so no triangular inverse is needed.
  __noinline__ __device__ bool prepare_nt(const Blk<T>& b) {
    const int n = b.n;
    const int64_t nn = b.nn;
    T* M = b.W(W_T1);
    T* GV = b.W(W_G);
    T* D = b.V(WV_D);
    cta_gemm<T>(n, 1, 0, 1, 1, (T)1, b.W(W_LS), b.W(W_LX), (T)0, M, scr());
    bool conv;
    int sweeps = 0;
    PROF_BEGIN(j);
    const bool f32ws = prm.precision == MSDP_MIXED;  // an FP32 workspace exists
    const bool smem32 = (2 * nn + n) * (int64_t)sizeof(float) <= MSDP_SMEM_BYTES;
    if (sizeof(T) == 8 && (f32ws || smem32)) {
      // float64 NT scaling (the FP64 path and the FP64 phase of the mixed
      // path): eigenvectors by FP32 Jacobi, then M V and Lx V in FP64 and
      // FP64 polishing sweeps to float64 convergence (quadratic from the
      // FP32 basis).  Operands live in shared memory when they fit, else in
      // the (idle) FP32 workspace of a mixed batch and FP64 scratch.
      float *sMf, *sVf, *Df;
      if (smem32) {
        sMf = (float*)smem;
        sVf = sMf + nn;
        Df = sVf + nn;
      } else {
        const Blk<float> bf = make_blk<float>(B, P, blk_index(b));
        sMf = bf.W(W_T1);
        sVf = bf.W(W_T2);
        Df = bf.V(WV_D);
      }
      for (int64_t k = threadIdx.x; k < nn; k += NTHREADS) {
        sMf[k] = (float)M[k];
        sVf[k] = ((k % n) == (k / n)) ? 1.0f : 0.0f;
      }
      __syncthreads();
      int sw32 = 0;
      cta_jacobi_svd<float>(n, sMf, sVf, Df, 40, &sh.counter, &sw32);
      T* V64 = b.W(W_T2);
      for (int64_t k = threadIdx.x; k < nn; k += NTHREADS) V64[k] = (T)sVf[k];
      __syncthreads();
      const bool smem64 = 2 * nn * (int64_t)sizeof(T) <= MSDP_SMEM_BYTES;
      T* sM = smem64 ? (T*)smem : b.W(W_T3);
      T* sB = smem64 ? sM + nn : GV;
      const Scratch gs = smem64 ? Scratch{nullptr, 0} : scr();
      cta_gemm<T>(n, 0, 0, 0, 0, (T)1, M, V64, (T)0, sM, gs);
      cta_gemm<T>(n, 0, 0, 1, 0, (T)1, b.W(W_LX), V64, (T)0, sB, gs);
      conv = cta_jacobi_svd<T>(n, sM, sB, D, 40, &sh.counter, &sweeps);
      sweeps += 1000 * sw32;
      for (int64_t k = threadIdx.x; k < nn; k += NTHREADS) {
        M[k] = sM[k];
        if (sB != GV) GV[k] = sB[k];
      }
      __syncthreads();
    } else if (2 * nn * (int64_t)sizeof(T) <= MSDP_SMEM_BYTES) {
      T* sM = (T*)smem;
      T* sB = sM + nn;
      const T* Lx = b.W(W_LX);
      for (int64_t k = threadIdx.x; k < nn; k += NTHREADS) { sM[k] = M[k]; sB[k] = Lx[k]; }
      __syncthreads();
      conv = cta_jacobi_svd<T>(n, sM, sB, D, 40, &sh.counter, &sweeps);
      for (int64_t k = threadIdx.x; k < nn; k += NTHREADS) { M[k] = sM[k]; GV[k] = sB[k]; }
      __syncthreads();
    } else {
      const T* Lx = b.W(W_LX);
      for (int64_t k = threadIdx.x; k < nn; k += NTHREADS) GV[k] = Lx[k];
      __syncthreads();
      conv = cta_jacobi_svd<T>(n, M, GV, D, 40, &sh.counter, &sweeps);
    }
    PROF_END(j, SC_T_JACOBI);
    PROF_COUNT(SC_N_JACOBI_SWEEPS, sweeps);
    PROF_COUNT(SC_N_JACOBI_CALLS, 1);
    PROF_BEGIN(np);
    if (threadIdx.x == 0) {
      int bad = conv ? 0 : 1;
      for (int k = 0; k < n; ++k)
        if (!(D[k] > (T)0) || !Num<T>::finite(D[k])) bad = 1;
      sh.flag = bad;
    }
    __syncthreads();
    if (sh.flag) return false;
    T* G = GV;
    T* t2 = b.W(W_T2);
    for (int64_t k = threadIdx.x; k < nn; k += NTHREADS) {
      const int j = (int)(k / n);
      const T sq = Num<T>::sqrt_(D[j]);
      G[k] = G[k] / sq;                 // G = Lx V D^-1/2
      M[k] = M[k] / (D[j] * sq);        // (M V) D^-3/2
    }
    __syncthreads();
    // Gi = ((M V) D^-3/2)' Ls'
    cta_gemm<T>(n, 1, 1, 0, 1, (T)1, M, b.W(W_LS), (T)0, b.W(W_GI), scr());
    cta_gemm<T>(n, 0, 1, 0, 0, (T)1, G, G, (T)0, b.W(W_W), scr(), 1);
    cta_lower_to_full<T>(n, b.W(W_W));
    // S^-1 = G D^-1 G'
    for (int64_t k = threadIdx.x; k < nn; k += NTHREADS) t2[k] = G[k] / D[k / n];
    __syncthreads();
    cta_gemm<T>(n, 0, 1, 0, 0, (T)1, t2, G, (T)0, b.W(W_SI), scr(), 1);
    cta_lower_to_full<T>(n, b.W(W_SI));
    PROF_END(np, SC_T_NTPROD);
    return true;
  }

  __noinline__ __device__ bool prepare() {
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      // Ls = chol(S) with flush (src/blocks.jl:94-113,126-130)
      PROF_BEGIN(c);
      bool ok = chol_factor<T, double>(b.n, b.S, b.W(W_LS), true, smem, sh);
      PROF_END(c, SC_T_CHOL);
      if (!ok) return false;
      const bool need_lx = is_nt() || prm.step == MSDP_EIGEN_STEP;
      if (need_lx) {
        // Lx = chol(X) (src/directions.jl:46 and src/step.jl:177; computed once)
        PROF_BEGIN(cx);
        ok = chol_factor<T, double>(b.n, b.X, b.W(W_LX), true, smem, sh);
        PROF_END(cx, SC_T_CHOL);
        if (!ok) return false;
      }
      if (is_nt()) {
        if (!prepare_nt(b)) return false;
      } else {
        // S^-1 = Ls^-T Ls^-1 (potri, src/blocks.jl:116-123)
        PROF_BEGIN(t);
        tri_inverse<T>(b.n, b.W(W_LS), b.W(W_LSI), smem);
        cta_gemm<T>(b.n, 1, 0, 1, 1, (T)1, b.W(W_LSI), b.W(W_LSI), (T)0, b.W(W_SI), scr());
        cta_symmetrize<T>(b.n, b.W(W_SI));
        if (prm.step == MSDP_EIGEN_STEP) tri_inverse<T>(b.n, b.W(W_LX), b.W(W_LXI), smem);
        PROF_END(t, SC_T_TRTRI);
        // the compute-type view of X used by HKM's E(.) and Schur scaling
        (void)as_T<T>(b.nn, b.X, b.W(W_XT));
      }
    }
    for (int k = threadIdx.x; k < P.ns; k += NTHREADS) P.zinv[k] = 1.0 / P.z[k];
    __syncthreads();
    return true;
  }

  // ---------------- Schur complement (LowRankOpt.schur_complement!)
  // H_jk += <A_j, L A_k R> over the coordinate lists.  Only the (j >= k)
  // half is computed; both halves are written.
  __noinline__ __device__ void schur_block_add(const Blk<T>& b, const T* Lg, const T* Rg, T* H) {
    const int n = b.n, m = P.m;
    const int64_t nn = b.nn;
    if (b.structure == STRUCT_DENSE) {
      // by columns: T_k = L A_k R, then H_jk = <A_j, T_k> = A_j(T_k) for j >= k
      T* Ak = b.W(W_T1);
      T* Lk = b.W(W_T2);
      T* Tk = b.W(W_T3);
      const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
      for (int k = 0; k < m; ++k) {
        for (int64_t q = threadIdx.x; q < nn; q += NTHREADS) Ak[q] = (T)0;
        __syncthreads();
        for (int64_t q = b.cptr[k] + threadIdx.x; q < b.cptr[k + 1]; q += NTHREADS)
          atomicAdd(&Ak[b.erow[q] + (int64_t)b.ecol[q] * n], (T)b.eval[q]);
        __syncthreads();
        cta_gemm<T>(n, 0, 0, 0, 0, (T)1, Lg, Ak, (T)0, Lk, scr());
        cta_gemm<T>(n, 0, 0, 0, 0, (T)1, Lk, Rg, (T)0, Tk, scr());
        for (int j = k + warp; j < m; j += NWARPS) {
          T acc = (T)0;
          for (int64_t q = b.cptr[j] + lane; q < b.cptr[j + 1]; q += 32)
            acc = fma((T)b.eval[q], Tk[b.erow[q] + (int64_t)b.ecol[q] * n], acc);
          acc = warp_sum(acc);
          if (lane == 0) {
            H[j + (int64_t)k * m] += acc;
            if (j != k) H[k + (int64_t)j * m] += acc;
          }
        }
        __syncthreads();
      }
      return;
    }
    if constexpr (sizeof(T) == 8) {
      // float64 Hankel blocks from n = 32 on: FFT along the column index;
      // the scratch is the eight consecutive n x n matrices T1 .. ERD of the
      // block, free during assembly ((2n-1)(N/2+1) complex <= 8 n^2 doubles)
      int N = 1;
      while (N < 2 * n - 1) N <<= 1;
      const bool fits = (int64_t)(N / 2 + NWARPS * N) * 16 <= MSDP_SMEM_BYTES;  // twiddles + warp buffers
      if (b.structure == STRUCT_HANKEL && Lg == Rg && n >= 32 && fits) {
        hankel_fft(n, Lg, H, b.W(W_T1));
        return;
      }
    }
    if (b.structure == STRUCT_HANKEL && Lg == Rg) {
      constexpr int PAD = 4;  // >= tile - 1: window indices leave [0, n) by at most 3
      const int64_t np = n + 2 * PAD;
      // the padded copy of W: shared memory, else the three consecutive
      // n x n scratch matrices T1..T3 of the block (free during assembly)
      T* Wp = np * np * (int64_t)sizeof(T) <= MSDP_SMEM_BYTES ? (T*)smem
              : (np * np <= 3 * nn ? b.W(W_T1) : nullptr);
      if (Wp) {
        hankel_tiled(n, Lg, H, Wp);
        return;
      }
    }
    const T* L = Lg;
    const T* R = Rg;
    const int64_t need = (Lg == Rg ? 1 : 2) * nn * (int64_t)sizeof(T);
    if (need <= MSDP_SMEM_BYTES) {
      T* sL = (T*)smem;
      T* sR = (Lg == Rg) ? sL : sL + nn;
      for (int64_t k = threadIdx.x; k < nn; k += NTHREADS) {
        sL[k] = Lg[k];
        if (Lg != Rg) sR[k] = Rg[k];
      }
      __syncthreads();
      L = sL;
      R = sR;
    }
    const int64_t npairs = (int64_t)m * (m + 1) / 2;
    if (b.structure == STRUCT_HANKEL) {
      // A_j = sum_{a+b=j} E_ab (0/1): H_jk = sum_a sum_c L[a,c] R[k-c, j-a]
      for (int64_t idx = threadIdx.x; idx < npairs; idx += NTHREADS) {
        int j, k;
        tri_index(idx, j, k);
        const int a0 = max(0, j - n + 1), a1 = min(j, n - 1);
        const int c0 = max(0, k - n + 1), c1 = min(k, n - 1);
        T acc = (T)0;
        for (int a = a0; a <= a1; ++a) {
          const T* Ra = R + (int64_t)(j - a) * n + k;   // R[k-c, j-a] = Ra[-c]
          const T* La = L + a;                          // L[a, c] = La[c*n]
          for (int c = c0; c <= c1; ++c) acc = fma(La[(int64_t)c * n], Ra[-c], acc);
        }
        H[j + (int64_t)k * m] += acc;
        if (j != k) H[k + (int64_t)j * m] += acc;
      }
      __syncthreads();
      return;
    }
    for (int64_t idx = threadIdx.x; idx < npairs; idx += NTHREADS) {
      int j, k;
      tri_index(idx, j, k);
      const int64_t e0 = b.cptr[j], e1 = b.cptr[j + 1];
      const int64_t f0 = b.cptr[k], f1 = b.cptr[k + 1];
      T acc = (T)0;
      for (int64_t e = e0; e < e1; ++e) {
        const int re = b.erow[e], ce = b.ecol[e];
        const T ve = (T)b.eval[e];
        T part = (T)0;
        for (int64_t f = f0; f < f1; ++f) {
          const int rf = b.erow[f], cf = b.ecol[f];
          part = fma((T)b.eval[f] * L[re + (int64_t)rf * n], R[cf + (int64_t)ce * n], part);
        }
        acc = fma(ve, part, acc);
      }
      H[j + (int64_t)k * m] += acc;
      if (j != k) H[k + (int64_t)j * m] += acc;
    }
    __syncthreads();
  }

  // Hankel 0/1 constraints with L = R = W (NT, DualCentering):
  // H_jk = sum_a sum_c W[a,c] W[k-c, j-a], a 2-D correlation of W with
  // itself.  W is copied into Wp (shared memory, or global scratch for large
  // n) with a zero border of 4, so the index ranges need no bounds tests.  Each thread computes a 4 x 4 tile of
  // H (lower tile triangle) and slides a 4 x 4 register window along c: per
  // (a, c) step it loads W[a,c] and 4 new window values for 16 FMAs.
  __noinline__ __device__ void hankel_tiled(int n, const T* W, T* H, T* Wp) {
    constexpr int PAD = 4, TJ = 4, TK = 4;
    const int m = 2 * n - 1, np = n + 2 * PAD;
    for (int64_t q = threadIdx.x; q < (int64_t)np * np; q += NTHREADS) {
      const int r = (int)(q % np) - PAD, c = (int)(q / np) - PAD;
      Wp[q] = (r >= 0 && r < n && c >= 0 && c < n) ? W[r + (int64_t)c * n] : (T)0;
    }
    __syncthreads();
    // Wp(r, s) = W[r, s] for r, s in [-PAD, n + PAD)
    const T* W0 = Wp + PAD + (int64_t)PAD * np;
    const int tiles = (m + TJ - 1) / TJ;
    const int64_t ntp = (int64_t)tiles * (tiles + 1) / 2;
    for (int64_t idx = threadIdx.x; idx < ntp; idx += NTHREADS) {
      int tj, tk;
      tri_index(idx, tj, tk);
      const int j0 = tj * TJ, k0 = tk * TK;
      const int a_lo = max(0, j0 - n + 1), a_hi = min(j0 + TJ - 1, n - 1);
      const int c_lo = max(0, k0 - n + 1), c_hi = min(k0 + TK - 1, n - 1);
      T acc[TJ][TK];
#pragma unroll
      for (int dj = 0; dj < TJ; ++dj)
#pragma unroll
        for (int dk = 0; dk < TK; ++dk) acc[dj][dk] = (T)0;
      for (int a = a_lo; a <= a_hi; ++a) {
        const T* Wa = W0 + a;  // W[a, c] = Wa[c * np]
        T win[TJ][TK];         // win[dj][dk] = W[k0 + dk - c, j0 + dj - a]
#pragma unroll
        for (int dj = 0; dj < TJ; ++dj) {
          const T* col = W0 + (int64_t)(j0 + dj - a) * np + k0 - c_lo;
#pragma unroll
          for (int dk = 0; dk < TK; ++dk) win[dj][dk] = col[dk];
        }
        for (int c = c_lo; c <= c_hi; ++c) {
          const T w = Wa[(int64_t)c * np];
#pragma unroll
          for (int dj = 0; dj < TJ; ++dj)
#pragma unroll
            for (int dk = 0; dk < TK; ++dk) acc[dj][dk] = fma(w, win[dj][dk], acc[dj][dk]);
#pragma unroll
          for (int dj = 0; dj < TJ; ++dj) {
#pragma unroll
            for (int dk = TK - 1; dk > 0; --dk) win[dj][dk] = win[dj][dk - 1];
            win[dj][0] = W0[(int64_t)(j0 + dj - a) * np + k0 - (c + 1)];
          }
        }
      }
#pragma unroll
      for (int dj = 0; dj < TJ; ++dj)
#pragma unroll
        for (int dk = 0; dk < TK; ++dk) {
          const int j = j0 + dj, k = k0 + dk;
          if (j < m && k < m && j >= k) {
            H[j + (int64_t)k * m] += acc[dj][dk];
            if (j != k) H[k + (int64_t)j * m] += acc[dj][dk];
          }
        }
    }
    __syncthreads();
  }

  // Hankel 0/1 constraints with L = R = W in float64 for larger blocks:
  // H(j, k) = sum_{a+b=j} (row_a * row_b)(k), the linear convolution of
  // rows of W.  Rows are transformed by a length-N FFT along the column
  // index (N = power of two >= 2n-1, so circular = linear convolution);
  // per frequency w, Hh(j, w) = sum_{a+b=j} F_a(w) F_b(w) (n^2 complex
  // multiply-adds); an inverse FFT per j gives H(j, :).  O(n^3) instead of
  // the O(n^4) of the direct sum.  Only w <= N/2 is stored (real rows give
  // Hermitian spectra).  S: (2n-1) (N/2+1) complex scratch, column w at
  // S + w (2n-1).
  __device__ static void warp_fft(int N, int logN, double2* buf, const double2* tw, bool inverse) {
    const int lane = threadIdx.x & 31;
    for (int i = lane; i < N; i += 32) {
      const int r = (int)(__brev((unsigned)i) >> (32 - logN));
      if (i < r) {
        const double2 t = buf[i];
        buf[i] = buf[r];
        buf[r] = t;
      }
    }
    __syncwarp();
    for (int len = 2; len <= N; len <<= 1) {
      const int half = len >> 1, step = N / len;
      for (int q = lane; q < N / 2; q += 32) {
        const int pos = q % half;
        const int i = (q / half) * len + pos, i2 = i + half;
        double2 w = tw[pos * step];
        if (inverse) w.y = -w.y;
        const double2 u = buf[i], v0 = buf[i2];
        const double2 v = make_double2(v0.x * w.x - v0.y * w.y, v0.x * w.y + v0.y * w.x);
        buf[i] = make_double2(u.x + v.x, u.y + v.y);
        buf[i2] = make_double2(u.x - v.x, u.y - v.y);
      }
      __syncwarp();
    }
  }

  __noinline__ __device__ void hankel_fft(int n, const double* W, double* H, double* S) {
    // S: interleaved (re, im) doubles; the workspace is only 8-byte aligned
    const int m = 2 * n - 1;
    int N = 1, logN = 0;
    while (N < m) { N <<= 1; ++logN; }
    const int Nh = N / 2 + 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double2* tw = (double2*)smem;                      // N/2 twiddles e^{-2 pi i t / N}
    double2* buf = tw + N / 2 + (int64_t)warp * N;     // per-warp FFT buffer
    for (int t = threadIdx.x; t < N / 2; t += NTHREADS) {
      double sn, cs;
      sincospi(2.0 * (double)t / (double)N, &sn, &cs);
      tw[t] = make_double2(cs, -sn);
    }
    __syncthreads();
    // forward transforms of the rows
    for (int a = warp; a < n; a += NWARPS) {
      for (int c = lane; c < N; c += 32) buf[c] = make_double2(c < n ? W[a + (int64_t)c * n] : 0.0, 0.0);
      __syncwarp();
      warp_fft(N, logN, buf, tw, false);
      for (int w = lane; w < Nh; w += 32) {
        double* e = S + 2 * ((int64_t)w * m + a);
        e[0] = buf[w].x;
        e[1] = buf[w].y;
      }
      __syncwarp();
    }
    __syncthreads();
    // per frequency: convolution over the row index (in place per column)
    for (int w = warp; w < Nh; w += NWARPS) {
      double* col = S + 2 * (int64_t)w * m;
      for (int a = lane; a < n; a += 32) buf[a] = make_double2(col[2 * a], col[2 * a + 1]);
      __syncwarp();
      for (int j = lane; j < m; j += 32) {
        const int a0 = max(0, j - n + 1), a1 = min(j, n - 1);
        double re = 0.0, im = 0.0;
        for (int a = a0; a <= a1; ++a) {
          const double2 f = buf[a], g2 = buf[j - a];
          re = fma(f.x, g2.x, fma(-f.y, g2.y, re));
          im = fma(f.x, g2.y, fma(f.y, g2.x, im));
        }
        col[2 * j] = re;
        col[2 * j + 1] = im;
      }
      __syncwarp();
    }
    __syncthreads();
    // inverse transforms per j (Hermitian completion), real part / N
    const double invN = 1.0 / (double)N;
    for (int j = warp; j < m; j += NWARPS) {
      for (int w = lane; w < N; w += 32) {
        if (w < Nh) {
          const double* e = S + 2 * ((int64_t)w * m + j);
          buf[w] = make_double2(e[0], e[1]);
        } else {
          const double* e = S + 2 * ((int64_t)(N - w) * m + j);
          buf[w] = make_double2(e[0], -e[1]);
        }
      }
      __syncwarp();
      warp_fft(N, logN, buf, tw, true);
      for (int k = lane; k < m; k += 32) H[j + (int64_t)k * m] += buf[k].x * invN;
      __syncwarp();
    }
    __syncthreads();
  }

  __noinline__ __device__ void schur_complement(T* H) {
    const int m = P.m;
    const int64_t mm = (int64_t)m * m;
    for (int64_t k = threadIdx.x; k < mm; k += NTHREADS) H[k] = (T)0;
    __syncthreads();
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      const T *L, *R;
      if (prm.algorithm == MSDP_DUAL_CENTERING) { L = b.W(W_SI); R = b.W(W_SI); }
      else if (prm.direction == MSDP_NT) { L = b.W(W_W); R = b.W(W_W); }
      else { L = b.W(W_SI); R = xt(b); }
      schur_block_add(b, L, R, H);
    }
    if (P.ns > 0) {
      // + C_lin diag(x ./ z) C_lin' (scalar scalings x and 1 ./ z, src/solver.jl:30-31)
      for (int k = threadIdx.x; k < P.ns; k += NTHREADS) P.ws2[k] = P.x[k] * P.zinv[k];
      __syncthreads();
      for (int64_t idx = threadIdx.x; idx < mm; idx += NTHREADS) {
        const int j = (int)(idx % m), k = (int)(idx / m);
        double s = 0.0;
        for (int l = 0; l < P.ns; ++l)
          s = fma(P.Clin[j + (int64_t)l * m] * P.ws2[l], P.Clin[k + (int64_t)l * m], s);
        H[idx] = (T)((double)H[idx] + s);
      }
      __syncthreads();
    }
  }

  // The Schur matrix and its factor for this compute type.
  __device__ T* schur_H();
  __device__ T* schur_L();

  // factorize_schur! with the regularization retry loop (src/solver.jl:299-314)
  __noinline__ __device__ bool factorize_schur() {
    if (prm.schur == MSDP_QR_SCHUR) return qr_factorize();
    const int m = P.m;
    const int64_t mm = (int64_t)m * m;
    T* H = schur_H();
    T* L = schur_L();
    double reg = prm.regularize_schur;
    for (int attempt = 0; attempt < prm.max_schur_reg; ++attempt) {
      PROF_BEGIN(a);
      schur_complement(H);
      PROF_END(a, SC_T_ASSEMBLY);
      PROF_COUNT(SC_N_FACTOR, 1);
      PROF_BEGIN(f);
      if (reg > 0.0) {
        for (int i = threadIdx.x; i < m; i += NTHREADS) H[i + (int64_t)i * m] += (T)reg;
        __syncthreads();
      }
      T* A = (mm * (int64_t)sizeof(T) <= MSDP_SMEM_BYTES) ? (T*)smem : L;
      if (A != H) {
        for (int64_t k = threadIdx.x; k < mm; k += NTHREADS) A[k] = H[k];
        __syncthreads();
      }
      bool ok = (prm.schur == MSDP_MADNLP_SCHUR)
                    ? cta_sytrf_lower<T>(m, A, m, P.piv, (T*)P.wm, &sh.rb, &sh.flag)
                    : cta_potrf<T>(m, A, m, &sh.flag);
      if (ok) {
        if (A != L) {
          for (int64_t k = threadIdx.x; k < mm; k += NTHREADS) L[k] = A[k];
          __syncthreads();
        }
        PROF_END(f, SC_T_FACTOR);
        return true;
      }
      PROF_END(f, SC_T_FACTOR);
      reg = (reg == 0.0) ? 1e-12 : 10.0 * reg;
    }
    return false;
  }

  // x = H^-1 x (src/schur_solvers.jl:21); the float factor is followed by
  // two steps of iterative refinement with float64 residuals.
  __device__ void schur_solve(double* x);

  // ---------------- E(.) (src/directions.jl:80-84,116-120)
  __noinline__ __device__ void apply_E(const Blk<T>& b, const T* Min, T* out) {
    const int n = b.n;
    T* tmp = b.W(W_T3);
    if (is_nt()) {
      // W M W is symmetric: the second product only for the lower triangle
      cta_gemm<T>(n, 0, 0, 0, 0, (T)1, b.W(W_W), Min, (T)0, tmp, scr());
      cta_gemm<T>(n, 0, 0, 0, 0, (T)1, tmp, b.W(W_W), (T)0, out, scr(), 1);
      cta_lower_to_full<T>(n, out);
    } else {
      cta_gemm<T>(n, 0, 0, 0, 0, (T)1, xt(b), Min, (T)0, tmp, scr());
      cta_gemm<T>(n, 0, 0, 0, 0, (T)1, tmp, b.W(W_SI), (T)0, out, scr());
      cta_symmetrize<T>(n, out);
    }
  }

  // ---------------- rhs! (src/step.jl:63-89)
  __noinline__ __device__ void rhs(double mu, bool corrected) {
    for (int j = threadIdx.x; j < P.m; j += NTHREADS) P.h[j] = P.Rp[j];
    __syncthreads();
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      const bool rdnz = b.bsc[BS_RDNZ] != 0.0;
      if (rdnz) {
        T* rdt = as_T<T>(b.nn, b.Rd, b.W(W_T2));
        apply_E(b, rdt, b.W(W_ERD));
      }
      const T* Si = b.W(W_SI);
      const T* erd = b.W(W_ERD);
      const T* corr = b.W(W_CORR);
      for (int64_t k = threadIdx.x; k < b.nn; k += NTHREADS) {
        double v = b.X[k] - mu * (double)Si[k];
        if (rdnz) v += (double)erd[k];
        if (corrected) v -= (double)corr[k];
        b.buf[k] = v;
      }
      __syncthreads();
      jprod_add(b, P.m, b.buf, P.h);
    }
    if (P.ns > 0) {
      for (int k = threadIdx.x; k < P.ns; k += NTHREADS) {
        const double x = P.x[k], zi = P.zinv[k];
        double v = x - mu * zi + x * zi * P.Rdlin[k];
        if (corrected) v -= P.corrlin[k];
        P.ws[k] = v;
      }
      __syncthreads();
      clin_mv(P, P.ws, 1.0, P.h);
    }
  }

  // ---------------- directions! (src/step.jl:94-124)
  __noinline__ __device__ void directions(double mu, bool corrected) {
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      const bool rdnz = b.bsc[BS_RDNZ] != 0.0;
      // A*(dely), and dS = sym(Rd - A*(dely))
      jtprod_combine(b, P.dely, 1.0, nullptr, nullptr, b.ATy);
      for (int64_t k = threadIdx.x; k < b.nn; k += NTHREADS) b.dS[k] = b.Rd[k] - b.ATy[k];
      __syncthreads();
      cta_symmetrize<double>(b.n, b.dS);
      T* at = as_T<T>(b.nn, b.ATy, b.W(W_T2));
      apply_E(b, at, b.W(W_T1));
      const T* Si = b.W(W_SI);
      const T* e1 = b.W(W_T1);
      const T* erd = b.W(W_ERD);
      const T* corr = b.W(W_CORR);
      for (int64_t k = threadIdx.x; k < b.nn; k += NTHREADS) {
        double v = mu * (double)Si[k] - b.X[k] + (double)e1[k];
        if (rdnz) v -= (double)erd[k];
        if (corrected) v += (double)corr[k];
        b.dX[k] = v;
      }
      __syncthreads();
      cta_symmetrize<double>(b.n, b.dX);
    }
    if (P.ns > 0) {
      clin_tmv(P, P.dely, P.Rdlin, -1.0, P.delz);
      for (int k = threadIdx.x; k < P.ns; k += NTHREADS) {
        const double x = P.x[k], zi = P.zinv[k];
        double v = mu * zi - x - x * zi * P.delz[k];
        if (corrected) v += P.corrlin[k];
        P.delx[k] = v;
      }
      __syncthreads();
    }
  }

  // ---------------- correction! (src/step.jl:128-136, src/directions.jl:90-100,123-127)
  __noinline__ __device__ void correction() {
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      const int n = b.n;
      T* dxt = as_T<T>(b.nn, b.dX, b.W(W_DXT));
      T* dst = as_T<T>(b.nn, b.dS, b.W(W_DST));
      T* t1 = b.W(W_T1);
      T* t2 = b.W(W_T2);
      T* t3 = b.W(W_T3);
      T* corr = b.W(W_CORR);
      if (is_nt()) {
        T* RNT = b.W(W_RNT);
        const T* D = b.V(WV_D);
        cta_gemm<T>(n, 0, 0, 0, 0, (T)1, b.W(W_GI), dxt, (T)0, t1, scr());
        cta_gemm<T>(n, 0, 0, 0, 0, (T)1, t1, dst, (T)0, t2, scr());
        cta_gemm<T>(n, 0, 0, 0, 0, (T)1, t2, b.W(W_G), (T)0, t3, scr());
        for (int64_t k = threadIdx.x; k < b.nn; k += NTHREADS) {
          const int p = (int)(k % n), q = (int)(k / n);
          RNT[k] = -(t3[k] + t3[q + (int64_t)p * n]) / (D[p] + D[q]);
        }
        __syncthreads();
        // G RNT G' with RNT symmetric: lower triangle only
        cta_gemm<T>(n, 0, 0, 0, 0, (T)1, b.W(W_G), RNT, (T)0, t1, scr());
        cta_gemm<T>(n, 0, 1, 0, 0, (T)1, t1, b.W(W_G), (T)0, corr, scr(), 1);
        cta_lower_to_full<T>(n, corr);
      } else {
        cta_gemm<T>(n, 0, 0, 0, 0, (T)1, dxt, dst, (T)0, t1, scr());
        cta_gemm<T>(n, 0, 0, 0, 0, (T)-1, t1, b.W(W_SI), (T)0, corr, scr());
        cta_symmetrize<T>(n, corr);
      }
    }
    for (int k = threadIdx.x; k < P.ns; k += NTHREADS) P.corrlin[k] = -P.delx[k] * P.delz[k] * P.zinv[k];
    __syncthreads();
  }

  // ---------------- step lengths (src/step.jl:148-228)
  __device__ double max_scalar_step(const double* x, const double* dx) {
    double a = INFINITY;
    for (int k = threadIdx.x; k < P.ns; k += NTHREADS)
      if (dx[k] < 0.0) a = fmin(a, -x[k] / dx[k]);
    // min reduction via max of negatives
    return -block_max(-a, &sh.rb);
  }

  // Fraction tau of the largest step keeping X + a dX and S + b dS positive
  // definite, from the smallest eigenvalues of L^-1 D L^-T (src/step.jl:178-183).
  // NT forms them in the scaled space (X = G D G', S = Gi' D Gi):
  //   Z_X = D^-1/2 Gi dX Gi' D^-1/2,  Z_S = D^-1/2 G' dS G D^-1/2,
  // which are congruent to Lx^-1 dX Lx^-T and Ls^-1 dS Ls^-T; HKM uses the
  // triangular inverses.  Warp 0 and warp 1 run the two Lanczos iterations
  // concurrently.
  // Smallest eigenvalues of ZX and ZS (n <= 256) by two warps, with Z, the
  // first basis columns and the work vectors staged in shared memory when
  // they fit; results in sh.bc[2] (X side) and sh.bc[3] (S side).
  template <class U>
  __device__ void lanczos_pair(int n, const U* ZX, const U* ZS, U* QX, U* QS, U* vX, U* vS, int& steps) {
    const int64_t nn = (int64_t)n * n;
      // per Lanczos: Z (n^2), kq basis columns and 4 vectors in shared memory
      const int64_t vec = 4 * (int64_t)(n + 1);
      const int64_t cap = MSDP_SMEM_BYTES / (int64_t)sizeof(U);
      int kq2 = (int)min((int64_t)n, max((int64_t)0, (cap / 2 - nn - vec) / n));   // two concurrent
      int kq1 = (int)min((int64_t)n, max((int64_t)0, (cap - nn - vec) / n));       // one at a time
      const bool concurrent = kq2 >= min(n, 16);
      const int kq = concurrent ? kq2 : kq1;
      const bool staged = (kq >= 1);
      const int64_t per = nn + (int64_t)kq * n + vec;
      U* base0 = (U*)smem;
      U* base1 = concurrent ? base0 + per : base0;
      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
      for (int pass = 0; pass < (concurrent || !staged ? 1 : 2); ++pass) {
        // stage the Z matrices this pass needs
        if (staged) {
          if (concurrent || pass == 0)
            for (int64_t k = threadIdx.x; k < nn; k += NTHREADS) base0[k] = ZX[k];
          if (concurrent || pass == 1)
            for (int64_t k = threadIdx.x; k < nn; k += NTHREADS) base1[k] = ZS[k];
          __syncthreads();
        }
        const bool runx = (concurrent || !staged) ? (warp == 0) : (pass == 0 && warp == 0);
        const bool runs = (concurrent || !staged) ? (warp == 1) : (pass == 1 && warp == 0);
        if (runx) {
          U* bs = base0;
          const U* z = staged ? bs : ZX;
          U* v = staged ? bs + nn + (int64_t)kq * n : vX;
          const U lam = staged
              ? warp_lanczos_eigmin<U>(n, z, bs + nn, kq, QX, v, v + (n + 1), v + 2 * (n + 1), v + 3 * (n + 1), &steps)
              : warp_lanczos_eigmin<U>(n, z, QX, n, QX, vX, vX + (n + 1), vX + 2 * (n + 1), vX + 3 * (n + 1), &steps);
          if (lane == 0) { sh.bc[2] = (double)lam; sh.bc[4] = (double)steps; }
        } else if (runs) {
          U* bs = base1;
          const U* z = staged ? bs : ZS;
          U* v = staged ? bs + nn + (int64_t)kq * n : vS;
          const U lam = staged
              ? warp_lanczos_eigmin<U>(n, z, bs + nn, kq, QS, v, v + (n + 1), v + 2 * (n + 1), v + 3 * (n + 1), &steps)
              : warp_lanczos_eigmin<U>(n, z, QS, n, QS, vS, vS + (n + 1), vS + 2 * (n + 1), vS + 3 * (n + 1), &steps);
          if (lane == 0) { sh.bc[3] = (double)lam; sh.bc[5] = (double)steps; }
        }
        __syncthreads();
      }
      steps = (int)(sh.bc[4] + sh.bc[5]);
  }

  __noinline__ __device__ void eigen_steps(const Blk<T>& b, double tau, double& ax, double& as) {
    const int n = b.n;
    const int64_t nn = b.nn;
    T* dxt = as_T<T>(nn, b.dX, b.W(W_DXT));
    T* dst = as_T<T>(nn, b.dS, b.W(W_DST));
    T* t1 = b.W(W_T1);
    T* ZX = b.W(W_T2);
    T* ZS = b.W(W_T3);
    if (is_nt()) {
      cta_gemm<T>(n, 0, 0, 0, 0, (T)1, b.W(W_GI), dxt, (T)0, t1, scr());
      cta_gemm<T>(n, 0, 1, 0, 0, (T)1, t1, b.W(W_GI), (T)0, ZX, scr());
      cta_gemm<T>(n, 1, 0, 0, 0, (T)1, b.W(W_G), dst, (T)0, t1, scr());
      cta_gemm<T>(n, 0, 0, 0, 0, (T)1, t1, b.W(W_G), (T)0, ZS, scr());
      const T* D = b.V(WV_D);
      for (int64_t k = threadIdx.x; k < nn; k += NTHREADS) {
        const T sc = Num<T>::rsqrt_(D[k % n]) * Num<T>::rsqrt_(D[k / n]);
        ZX[k] *= sc;
        ZS[k] *= sc;
      }
      __syncthreads();
    } else {
      cta_gemm<T>(n, 0, 0, 1, 0, (T)1, b.W(W_LXI), dxt, (T)0, t1, scr());
      cta_gemm<T>(n, 0, 1, 0, 1, (T)1, t1, b.W(W_LXI), (T)0, ZX, scr());
      cta_gemm<T>(n, 0, 0, 1, 0, (T)1, b.W(W_LSI), dst, (T)0, t1, scr());
      cta_gemm<T>(n, 0, 1, 0, 1, (T)1, t1, b.W(W_LSI), (T)0, ZS, scr());
    }
    PROF_BEGIN(l);
    int steps = 0;
    bool f32 = false;
    if constexpr (sizeof(T) == 8) {
      // FP64 phase of the mixed path: the step-length eigenvalues in FP32
      // (the iteration's float64 positive-definiteness check guards the step)
      f32 = prm.precision == MSDP_MIXED && n <= 256;
      if (f32) {
        const Blk<float> bf = make_blk<float>(B, P, blk_index(b));
        float* zx = bf.W(W_T2);
        float* zs = bf.W(W_T3);
        for (int64_t k = threadIdx.x; k < nn; k += NTHREADS) {
          zx[k] = (float)ZX[k];
          zs[k] = (float)ZS[k];
        }
        __syncthreads();
        lanczos_pair<float>(n, zx, zs, bf.W(W_Q), bf.W(W_RNT), bf.V(WV_LA), bf.V(WV_LA2), steps);
      }
    }
    if (f32) {
    } else if (n <= 256) {
      lanczos_pair<T>(n, ZX, ZS, b.W(W_Q), b.W(W_RNT), b.V(WV_LA), b.V(WV_LA2), steps);
    } else {
      const T* zx = ZX;
      const T* zs = ZS;
      int s1 = 0, s2 = 0;
      const T lx = lanczos_eigmin<T>(n, zx, b.W(W_Q), b.V(WV_LA), b.V(WV_LB), b.V(WV_LW), b.V(WV_LC), sh, &s1);
      const T ls = lanczos_eigmin<T>(n, zs, b.W(W_RNT), b.V(WV_LA2), b.V(WV_LB2), b.V(WV_LW2), b.V(WV_LC2), sh, &s2);
      if (threadIdx.x == 0) { sh.bc[2] = (double)lx; sh.bc[3] = (double)ls; }
      __syncthreads();
      steps = s1 + s2;
    }
    PROF_END(l, SC_T_LANCZOS);
    PROF_COUNT(SC_N_LANCZOS_STEPS, steps);
    PROF_COUNT(SC_N_LANCZOS_CALLS, 2);
    const double lx = sh.bc[2], ls = sh.bc[3];
    __syncthreads();
    const double thr = -sqrt(2.220446049250313e-16);
    ax = lx > thr ? 1.0 : fmin(1.0, -tau / lx);
    as = ls > thr ? 1.0 : fmin(1.0, -tau / ls);
  }

  __noinline__ __device__ double backtrack(bool primal) {
    double a = 1.0;
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      const double* X = primal ? b.X : b.S;
      const double* dX = primal ? b.dX : b.dS;
      int trials = 0;
      while (!add_mul_posdef<T>(b.n, X, a, dX, b.W(W_T1), smem, sh)) {
        a *= prm.shrink;
        if (a < 2.220446049250313e-16 || ++trials > 4096) return 0.0;
      }
    }
    if (a != 1.0) a *= prm.boundary;
    if (P.ns > 0) a = fmin(a, prm.boundary * max_scalar_step(primal ? P.x : P.z, primal ? P.delx : P.delz));
    return a;
  }

  __device__ void step_lengths(double& a, double& bt) {
    if (prm.step == MSDP_EIGEN_STEP) {
      a = 1.0; bt = 1.0;
      for (int i = 0; i < P.nblocks; ++i) {
        Blk<T> b = blk(i);
        double ax, as;
        eigen_steps(b, prm.tau, ax, as);
        a = fmin(a, ax);
        bt = fmin(bt, as);
      }
      if (P.ns > 0) {
        a = fmin(a, prm.tau * max_scalar_step(P.x, P.delx));
        bt = fmin(bt, prm.tau * max_scalar_step(P.z, P.delz));
      }
    } else {
      a = backtrack(true);
      bt = backtrack(false);
    }
  }

  // src/step.jl:231-243
  __device__ double affine_complementarity(double a, double bt) {
    double s = 0.0;
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      double t = 0.0;
      for (int64_t k = threadIdx.x; k < b.nn; k += NTHREADS) {
        const double x = b.X[k], sv = b.S[k], dx = b.dX[k], ds = b.dS[k];
        t += x * sv + bt * (x * ds) + a * (dx * sv) + a * bt * (dx * ds);
      }
      s += block_sum(t, &sh.rb);
    }
    double t = 0.0;
    for (int k = threadIdx.x; k < P.ns; k += NTHREADS) t += (P.x[k] + a * P.delx[k]) * (P.z[k] + bt * P.delz[k]);
    s += block_sum(t, &sh.rb);
    return s / fmax((double)nu(), 1.0);
  }

  // src/primal_dual.jl:56-72
  __noinline__ __device__ void take_step(double a, double bt) {
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      const int n = b.n;
      for (int64_t k = threadIdx.x; k < b.nn; k += NTHREADS) {
        const int r = (int)(k % n), c = (int)(k / n);
        if (r > c) {
          const int64_t kt = c + (int64_t)r * n;
          const double xv = ((b.X[k] + a * b.dX[k]) + (b.X[kt] + a * b.dX[kt])) / 2;
          b.X[k] = xv; b.X[kt] = xv;
          const double sv = ((b.S[k] + bt * b.dS[k]) + (b.S[kt] + bt * b.dS[kt])) / 2;
          b.S[k] = sv; b.S[kt] = sv;
        } else if (r == c) {
          b.X[k] += a * b.dX[k];
          b.S[k] += bt * b.dS[k];
        }
      }
      __syncthreads();
    }
    for (int j = threadIdx.x; j < P.m; j += NTHREADS) P.y[j] += bt * P.dely[j];
    for (int k = threadIdx.x; k < P.ns; k += NTHREADS) {
      P.x[k] += a * P.delx[k];
      P.z[k] += bt * P.delz[k];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      P.sc[SC_ALPHA] = a;
      P.sc[SC_BETA] = bt;
      P.sc[SC_ITER] += 1.0;
    }
    __syncthreads();
    update_residuals();
  }

  __noinline__ __device__ void solve_directions(double mu, bool corrected) {
    if (prm.schur == MSDP_QR_SCHUR) {
      qr_solve_directions(mu, corrected);
      return;
    }
    PROF_BEGIN(r);
    rhs(mu, corrected);
    for (int j = threadIdx.x; j < P.m; j += NTHREADS) P.dely[j] = P.h[j];
    __syncthreads();
    PROF_END(r, SC_T_RHS);
    PROF_BEGIN(s);
    schur_solve(P.dely);
    PROF_END(s, SC_T_SOLVE);
    PROF_BEGIN(d);
    if (sizeof(T) == 4 && prm.mixed_refine > 0) {
      // FP32 phase: directions with E applied in float64 to the FP32
      // scaling, then `mixed_refine` passes of Schur solves on the float64
      // primal defect r = Rp - A(dX) - C_lin dx, so that the primal
      // equation holds to float64 accuracy for that scaling.
      const double bn = fmax(1.0, P.sc[SC_BNORM]);
      double dmax = 0.0, rmax = 0.0;
      if (!corrected && threadIdx.x == 0) sh.erd64 = 0;
      __syncthreads();
      // the FP32 direction as is, when its float64 primal defect is already
      // far below the acceptance bound (large residuals early in the solve)
      directions(mu, corrected);
      primal_defect(dmax, rmax);
      if (dmax / bn <= 1e-3 * fmax(0.1 * rmax / bn, 0.01 * prm.tol)) {
        if (threadIdx.x == 0) sh.bc[7] = 0.0;
        __syncthreads();
        PROF_END(d, SC_T_DIRECTIONS);
        return;
      }
      const bool fresh = sh.erd64 == 0;
      __syncthreads();
      directions64(mu, corrected, fresh);
      if (fresh && threadIdx.x == 0) sh.erd64 = 1;
      __syncthreads();
      for (int pass = 0;; ++pass) {
        primal_defect(dmax, rmax);
        // at least one pass; stop early once the defect is far below the
        // acceptance bound (further passes would not change the decision)
        const double bound = fmax(0.1 * rmax / bn, 0.01 * prm.tol);
        if (pass >= prm.mixed_refine || (pass >= 1 && dmax / bn <= 1e-3 * bound)) break;
        schur_solve(P.h);
        for (int j = threadIdx.x; j < P.m; j += NTHREADS) P.dely[j] += P.h[j];
        __syncthreads();
        directions64(mu, corrected, false);
      }
      // the caller rejects an FP32 direction whose remaining float64 primal
      // defect (relative as inf_pr) exceeds the bound
      if (threadIdx.x == 0) sh.bc[7] = (dmax / bn > fmax(0.1 * rmax / bn, 0.01 * prm.tol)) ? 1.0 : 0.0;
      __syncthreads();
    } else {
      directions(mu, corrected);
      if (threadIdx.x == 0) sh.bc[7] = 0.0;
      __syncthreads();
    }
    PROF_END(d, SC_T_DIRECTIONS);
  }
  // P.h = Rp - A(dX) - C_lin dx in float64; its max norm and that of Rp
  __device__ void primal_defect(double& dmax, double& rmax) {
    for (int j = threadIdx.x; j < P.m; j += NTHREADS) P.h[j] = P.Rp[j];
    __syncthreads();
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      for (int64_t k = threadIdx.x; k < b.nn; k += NTHREADS) b.buf[k] = -b.dX[k];
      __syncthreads();
      jprod_add(b, P.m, b.buf, P.h);
    }
    if (P.ns > 0) clin_mv(P, P.delx, -1.0, P.h);
    double dl = 0.0, rl = 0.0;
    for (int j = threadIdx.x; j < P.m; j += NTHREADS) {
      dl = fmax(dl, fabs(P.h[j]));
      rl = fmax(rl, fabs(P.Rp[j]));
    }
    dmax = block_max(dl, &sh.rb);
    rmax = block_max(rl, &sh.rb);
  }

  // whether the last solve_directions left a primal defect above its bound
  __device__ __forceinline__ bool inexact_direction() const { return sh.bc[7] != 0.0; }

  // directions! with E(M) evaluated in float64 on the compute-type scaling
  // (NT: W M W; HKM: sym(X M S^-1)); E(Rd) is formed when `fresh_erd`.
  __noinline__ __device__ void directions64(double mu, bool corrected, bool fresh_erd) {
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      Blk<double> bd = make_blk<double>(B, P, i);
      const int n = b.n;
      const bool rdnz = b.bsc[BS_RDNZ] != 0.0;
      double* L64 = bd.W(W_W);
      double* R64 = bd.W(W_SI);
      double* erd = bd.W(W_ERD);
      double* e1 = bd.W(W_T1);
      double* tmp = bd.W(W_T3);
      if (fresh_erd) {
        const T* Lc = is_nt() ? b.W(W_W) : xt(b);
        const T* Rc = is_nt() ? b.W(W_W) : b.W(W_SI);
        for (int64_t k = threadIdx.x; k < b.nn; k += NTHREADS) { L64[k] = (double)Lc[k]; R64[k] = (double)Rc[k]; }
        __syncthreads();
        if (rdnz) {
          cta_gemm<double>(n, 0, 0, 0, 0, 1.0, L64, b.Rd, 0.0, tmp, scr());
          cta_gemm<double>(n, 0, 0, 0, 0, 1.0, tmp, R64, 0.0, erd, scr(), is_nt() ? 1 : 0);
          if (is_nt()) cta_lower_to_full<double>(n, erd);
          else cta_symmetrize<double>(n, erd);
        }
      }
      jtprod_combine(b, P.dely, 1.0, nullptr, nullptr, b.ATy);
      for (int64_t k = threadIdx.x; k < b.nn; k += NTHREADS) b.dS[k] = b.Rd[k] - b.ATy[k];
      __syncthreads();
      cta_symmetrize<double>(n, b.dS);
      cta_gemm<double>(n, 0, 0, 0, 0, 1.0, L64, b.ATy, 0.0, tmp, scr());
      cta_gemm<double>(n, 0, 0, 0, 0, 1.0, tmp, R64, 0.0, e1, scr(), is_nt() ? 1 : 0);
      if (is_nt()) cta_lower_to_full<double>(n, e1);
      else cta_symmetrize<double>(n, e1);
      const T* Si = b.W(W_SI);
      const T* corr = b.W(W_CORR);
      for (int64_t k = threadIdx.x; k < b.nn; k += NTHREADS) {
        double v = mu * (double)Si[k] - b.X[k] + e1[k];
        if (rdnz) v -= erd[k];
        if (corrected) v += (double)corr[k];
        b.dX[k] = v;
      }
      __syncthreads();
      cta_symmetrize<double>(n, b.dX);
    }
    if (P.ns > 0) {
      clin_tmv(P, P.dely, P.Rdlin, -1.0, P.delz);
      for (int k = threadIdx.x; k < P.ns; k += NTHREADS) {
        const double x = P.x[k], zi = P.zinv[k];
        double v = mu * zi - x - x * zi * P.delz[k];
        if (corrected) v += P.corrlin[k];
        P.delx[k] = v;
      }
      __syncthreads();
    }
  }

  // One Mehrotra predictor-corrector iteration (src/primal_dual.jl:85-101).
  // Returns false if it failed before taking a step.
  __noinline__ __device__ bool iterate_mehrotra(bool strict) {
    if (!prepare() || !factorize_schur()) return false;
    const double mu = total_complementarity() / fmax((double)nu(), 1.0);
    if (threadIdx.x == 0) P.sc[SC_MU] = mu;
    __syncthreads();
    solve_directions(0.0, false);
    if (!strict && inexact_direction()) return false;
    double a_aff, b_aff;
    {
      PROF_BEGIN(st);
      step_lengths(a_aff, b_aff);
      PROF_END(st, SC_T_STEP);
    }
    const double mu_aff = affine_complementarity(a_aff, b_aff);
    const double sigma = fmin(fmax(pow(mu_aff / fmax(mu, 2.220446049250313e-16), prm.sigma_exponent), 1e-8), 1.0);
    if (threadIdx.x == 0) P.sc[SC_SIGMA] = sigma;
    __syncthreads();
    {
      PROF_BEGIN(c);
      correction();
      PROF_END(c, SC_T_CORRECTION);
    }
    solve_directions(sigma * mu, true);
    if (!strict && inexact_direction()) return false;
    double a, bt;
    {
      PROF_BEGIN(st);
      step_lengths(a, bt);
      PROF_END(st, SC_T_STEP);
    }
    if (!strict && (!(fmin(a, bt) >= 0.2) || !step_keeps_interior(a, bt))) return false;
    if (strict) shrink_to_interior(a, bt);
    PROF_BEGIN(tk);
    take_step(a, bt);
    PROF_END(tk, SC_T_TAKE);
    return true;
  }

  // One mc_psd iteration (src/primal_dual.jl:104-121).
  __noinline__ __device__ bool iterate_adaptive(bool strict) {
    if (!prepare() || !factorize_schur()) return false;
    const double mu0 = P.sc[SC_MU];
    solve_directions(mu0, false);
    if (!strict && inexact_direction()) return false;
    double a, bt;
    step_lengths(a, bt);
    if (!strict && (!(fmin(a, bt) >= 0.2) || !step_keeps_interior(a, bt))) return false;
    if (strict) shrink_to_interior(a, bt);
    take_step(a, bt);
    double mu = prm.ratio * total_complementarity() / fmax((double)nu(), 1.0);
    if (fmin(a, bt) < 0.5) mu *= 1.5;
    if (a + bt > 1.6) mu *= 0.75;
    if (a + bt > 1.9) mu /= 1.0 + 0.1 * P.sc[SC_ITER];
    if (threadIdx.x == 0) P.sc[SC_MU] = mu;
    __syncthreads();
    return true;
  }

  // A step whose lengths came from compute-type (FP32) factors is taken
  // only if X + a dX and S + b dS are positive definite in float64: with
  // cond(S) near 1/eps_f32 the FP32 eigenvalue bound can overshoot.
  __noinline__ __device__ bool step_keeps_interior(double a, double bt) {
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      if (!add_mul_posdef<double>(b.n, b.X, a, b.dX, b.Shat, smem, sh)) return false;
      if (!add_mul_posdef<double>(b.n, b.S, bt, b.dS, b.Shat, smem, sh)) return false;
    }
    return true;
  }

  // FP64 iterations of the mixed path take their step-length eigenvalues
  // in FP32: the lengths are shrunk by 0.9 until X + a dX and S + b dS
  // factor in float64 (at most 64 times).  A no-op on the FP64 path.
  __noinline__ __device__ void shrink_to_interior(double& a, double& bt) {
    if (sizeof(T) != 8 || prm.precision != MSDP_MIXED || prm.step != MSDP_EIGEN_STEP) return;
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      if (b.n > 256) continue;  // larger blocks keep float64 eigenvalues
      for (int t = 0; t < 64 && !add_mul_posdef<double>(b.n, b.X, a, b.dX, b.Shat, smem, sh); ++t) a *= 0.9;
      for (int t = 0; t < 64 && !add_mul_posdef<double>(b.n, b.S, bt, b.dS, b.Shat, smem, sh); ++t) bt *= 0.9;
    }
  }

  __device__ bool iterate_pd(bool strict) {
    return prm.centering == MSDP_MEHROTRA ? iterate_mehrotra(strict) : iterate_adaptive(strict);
  }

  // ================================================================ QRSchur
  // src/qr_schur.jl: B[:, j] = svec(G' A_j G) (off-diagonals times sqrt 2)
  // over the blocks, then sqrt(x/z) C_lin' for the scalars; columns are
  // equilibrated and B D = Q R by Householder reflections (dense QR in
  // place of SPQR; the projection solve does not depend on the ordering).

  // svec position of (p, q), p <= q, column-major upper triangle
  __device__ __forceinline__ static int64_t svec_index(int p, int q) { return (int64_t)q * (q + 1) / 2 + p; }

  __noinline__ __device__ bool qr_factorize() {
    const int m = P.m, K = P.K;
    double* B = P.qrB;
    // ---- assemble B
    int64_t off = 0;
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      const int n = b.n;
      const int64_t nv = (int64_t)n * (n + 1) / 2;
      const T* G = b.W(W_G);
      for (int j = 0; j < m; ++j) {
        const int64_t e0 = b.cptr[j], e1 = b.cptr[j + 1];
        double* col = B + (int64_t)j * K + off;
        for (int64_t t = threadIdx.x; t < nv; t += NTHREADS) {
          int q = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
          while ((int64_t)(q + 1) * (q + 2) / 2 <= t) ++q;
          while ((int64_t)q * (q + 1) / 2 > t) --q;
          const int p = (int)(t - (int64_t)q * (q + 1) / 2);
          double v = 0.0;
          for (int64_t e = e0; e < e1; ++e)
            v = fma(b.eval[e] * (double)G[b.erow[e] + (int64_t)p * n], (double)G[b.ecol[e] + (int64_t)q * n], v);
          col[t] = (p == q) ? v : v * 1.4142135623730951;
        }
      }
      off += nv;
    }
    for (int k = threadIdx.x; k < P.ns; k += NTHREADS) {
      const double w = sqrt(P.x[k] / P.z[k]);
      for (int j = 0; j < m; ++j) B[(int64_t)j * K + off + k] = w * P.Clin[j + (int64_t)k * m];
    }
    __syncthreads();
    // ---- column equilibration (src/qr_schur.jl:73-82)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int bad = 0;
    for (int j = warp; j < m; j += NWARPS) {
      const double* col = B + (int64_t)j * K;
      double s = 0.0;
      for (int t = lane; t < K; t += 32) s = fma(col[t], col[t], s);
      s = sqrt(warp_sum(s));
      if (lane == 0) {
        if (s == 0.0 || !isfinite(s)) bad = 1;
        else P.qrscale[j] = 1.0 / s;
      }
    }
    bad = __syncthreads_or(bad);
    if (bad || K < m) return false;
    for (int64_t t = threadIdx.x; t < (int64_t)K * m; t += NTHREADS) B[t] *= P.qrscale[t / K];
    __syncthreads();
    // ---- Householder QR, reflectors below the diagonal, R above (dgeqr2)
    for (int k = 0; k < m; ++k) {
      double* bk = B + (int64_t)k * K;
      double s = 0.0;
      for (int i = k + 1 + threadIdx.x; i < K; i += NTHREADS) s = fma(bk[i], bk[i], s);
      s = block_sum(s, &sh.rb);
      const double a0 = bk[k];
      double tau = 0.0;
      if (s != 0.0) {
        const double beta = -copysign(sqrt(a0 * a0 + s), a0);
        tau = (beta - a0) / beta;
        const double scal = 1.0 / (a0 - beta);
        for (int i = k + 1 + threadIdx.x; i < K; i += NTHREADS) bk[i] *= scal;
        __syncthreads();
        if (threadIdx.x == 0) bk[k] = beta;
      }
      if (threadIdx.x == 0) P.qrtau[k] = tau;
      __syncthreads();
      if (tau != 0.0) {
        for (int c = k + 1 + warp; c < m; c += NWARPS) {
          double* bc = B + (int64_t)c * K;
          double w = 0.0;
          for (int i = k + 1 + lane; i < K; i += 32) w = fma(bk[i], bc[i], w);
          w = warp_sum(w) + bc[k];
          const double tw = tau * w;
          if (lane == 0) bc[k] -= tw;
          for (int i = k + 1 + lane; i < K; i += 32) bc[i] = fma(-tw, bk[i], bc[i]);
        }
        __syncthreads();
      }
    }
    // rank test: every R_ii nonzero (src/qr_schur.jl:86-87)
    int zero = 0;
    for (int k = threadIdx.x; k < m; k += NTHREADS) zero |= (B[(int64_t)k * K + k] == 0.0);
    zero = __syncthreads_or(zero);
    return !zero;
  }

  // u <- H_k u for k = first..last (step +1 or -1); u length K
  __device__ void qr_apply(double* u, bool transpose) {
    const int m = P.m, K = P.K;
    const double* B = P.qrB;
    for (int it = 0; it < m; ++it) {
      const int k = transpose ? it : m - 1 - it;
      const double tau = P.qrtau[k];
      if (tau == 0.0) continue;
      const double* bk = B + (int64_t)k * K;
      double w = 0.0;
      for (int i = k + 1 + threadIdx.x; i < K; i += NTHREADS) w = fma(bk[i], u[i], w);
      w = block_sum(w, &sh.rb) + u[k];
      const double tw = tau * w;
      for (int i = k + 1 + threadIdx.x; i < K; i += NTHREADS) u[i] = fma(-tw, bk[i], u[i]);
      if (threadIdx.x == 0) u[k] -= tw;
      __syncthreads();
    }
  }

  // solve_directions!(::QRSchurWorkspace, ...) (src/qr_schur.jl:90-160)
  __noinline__ __device__ void qr_solve_directions(double mu, bool corrected) {
    const int m = P.m, K = P.K;
    const double* B = P.qrB;
    double* base = P.qrbase;
    double* u = P.qrdir;
    int64_t off = 0;
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      const int n = b.n;
      const int64_t nv = (int64_t)n * (n + 1) / 2;
      // T = -G' Rd G + diag(mu / D - D) (+ RNT)
      T* rdt = as_T<T>(b.nn, b.Rd, b.W(W_T3));
      cta_gemm<T>(n, 0, 0, 0, 0, (T)1, rdt, b.W(W_G), (T)0, b.W(W_T1), scr());
      cta_gemm<T>(n, 1, 0, 0, 0, (T)-1, b.W(W_G), b.W(W_T1), (T)0, b.W(W_T2), scr());
      const T* Tm = b.W(W_T2);
      const T* D = b.V(WV_D);
      const T* RNT = b.W(W_RNT);
      for (int64_t t = threadIdx.x; t < nv; t += NTHREADS) {
        int q = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
        while ((int64_t)(q + 1) * (q + 2) / 2 <= t) ++q;
        while ((int64_t)q * (q + 1) / 2 > t) --q;
        const int p = (int)(t - (int64_t)q * (q + 1) / 2);
        double v = (double)Tm[p + (int64_t)q * n];
        if (p == q) v += mu / (double)D[p] - (double)D[p];
        if (corrected) v += (double)RNT[p + (int64_t)q * n];
        base[off + t] = (p == q) ? v : 1.4142135623730951 * v;
      }
      __syncthreads();
      off += nv;
    }
    for (int k = threadIdx.x; k < P.ns; k += NTHREADS) {
      const double w = sqrt(P.x[k] / P.z[k]), prod = sqrt(P.x[k] * P.z[k]);
      double v = mu / prod - prod - w * P.Rdlin[k];
      if (corrected) v += P.corrlin[k] / w;
      base[off + k] = v;
    }
    __syncthreads();
    // qbase = Q' base
    for (int t = threadIdx.x; t < K; t += NTHREADS) u[t] = base[t];
    __syncthreads();
    qr_apply(u, true);
    // c = R^-T (scale .* Rp); t = c - qbase[0:m]  (one warp, forward substitution)
    double* cvec = P.wm;
    double* dy = P.dely;
    if ((threadIdx.x >> 5) == 0) {
      const int lane = threadIdx.x & 31;
      for (int j = 0; j < m; ++j) {
        double s = 0.0;
        for (int l = lane; l < j; l += 32) s = fma(B[l + (int64_t)j * K], cvec[l], s);
        s = warp_sum(s);
        if (lane == 0) cvec[j] = (P.qrscale[j] * P.Rp[j] - s) / B[j + (int64_t)j * K];
        __syncwarp();
      }
      for (int j = lane; j < m; j += 32) cvec[j] -= u[j];
      __syncwarp();
      // dy = scale .* (R^-1 t)  (back substitution)
      for (int j = m - 1; j >= 0; --j) {
        double s = 0.0;
        for (int l = j + 1 + lane; l < m; l += 32) s = fma(B[j + (int64_t)l * K], dy[l], s);
        s = warp_sum(s);
        if (lane == 0) dy[j] = (cvec[j] - s) / B[j + (int64_t)j * K];
        __syncwarp();
      }
      for (int j = lane; j < m; j += 32) dy[j] *= P.qrscale[j];
    }
    __syncthreads();
    // direction = base + Q [t; 0]
    for (int t = threadIdx.x; t < K; t += NTHREADS) u[t] = t < m ? cvec[t] : 0.0;
    __syncthreads();
    qr_apply(u, false);
    for (int t = threadIdx.x; t < K; t += NTHREADS) u[t] += base[t];
    __syncthreads();
    off = 0;
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      const int n = b.n;
      const int64_t nv = (int64_t)n * (n + 1) / 2;
      T* Mt = b.W(W_T3);
      for (int64_t k = threadIdx.x; k < b.nn; k += NTHREADS) {
        const int p0 = (int)(k % n), q0 = (int)(k / n);
        const int p = min(p0, q0), q = max(p0, q0);
        const double v = u[off + svec_index(p, q)];
        Mt[k] = (T)(p == q ? v : v / 1.4142135623730951);
      }
      __syncthreads();
      // dX = sym(G M G'), dS = sym(Rd - A*(dy))
      cta_gemm<T>(n, 0, 0, 0, 0, (T)1, b.W(W_G), Mt, (T)0, b.W(W_T1), scr());
      cta_gemm<T>(n, 0, 1, 0, 0, (T)1, b.W(W_T1), b.W(W_G), (T)0, b.W(W_T2), scr());
      const T* dx = b.W(W_T2);
      for (int64_t k = threadIdx.x; k < b.nn; k += NTHREADS) b.dX[k] = (double)dx[k];
      __syncthreads();
      cta_symmetrize<double>(n, b.dX);
      jtprod_combine(b, P.dely, -1.0, b.Rd, nullptr, b.dS);
      cta_symmetrize<double>(n, b.dS);
      off += nv;
    }
    if (P.ns > 0) {
      clin_tmv(P, P.dely, P.Rdlin, -1.0, P.delz);
      for (int k = threadIdx.x; k < P.ns; k += NTHREADS) P.delx[k] = sqrt(P.x[k] / P.z[k]) * u[off + k];
      __syncthreads();
    }
  }

  // ================================================================ DualCentering
  // src/dual_centering.jl: the method carries y, S = C - A*(y) (always
  // feasible) and t; X is an estimate after each predictor step.

  // S = C - A*(y), factor and invert every block (:83-86)
  __noinline__ __device__ bool refresh_slacks() {
    set_dual_slacks();
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      if (!chol_factor<T, double>(b.n, b.S, b.W(W_LS), true, smem, sh)) return false;
      tri_inverse<T>(b.n, b.W(W_LS), b.W(W_LSI), smem);
      cta_gemm<T>(b.n, 1, 0, 1, 1, (T)1, b.W(W_LSI), b.W(W_LSI), (T)0, b.W(W_SI), scr());
      cta_symmetrize<T>(b.n, b.W(W_SI));
    }
    return true;
  }

  // g = A(S^-1) - t b (:89-98); d = H^-1 g, lambda = sqrt(g'd) (:102-110)
  __noinline__ __device__ bool newton_direction() {
    for (int j = threadIdx.x; j < P.m; j += NTHREADS) P.dcgz[j] = 0.0;
    __syncthreads();
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      jprod_add(b, P.m, b.W(W_SI), P.dcgz);
    }
    const double t = P.sc[SC_DC_T];
    for (int j = threadIdx.x; j < P.m; j += NTHREADS) P.dcg[j] = P.dcgz[j] - t * P.b[j];
    __syncthreads();
    if (!factorize_schur()) return false;
    for (int j = threadIdx.x; j < P.m; j += NTHREADS) P.dcd[j] = P.dcg[j];
    __syncthreads();
    schur_solve(P.dcd);
    double gd = 0.0;
    for (int j = threadIdx.x; j < P.m; j += NTHREADS) gd = fma(P.dcg[j], P.dcd[j], gd);
    gd = block_sum(gd, &sh.rb);
    if (threadIdx.x == 0) P.sc[SC_DC_LAM] = sqrt(fmax(gd, 0.0));
    __syncthreads();
    return true;
  }

  // y -= d / (1 + lambda)
  __device__ void damped_newton_step() {
    const double lam = P.sc[SC_DC_LAM];
    for (int j = threadIdx.x; j < P.m; j += NTHREADS) P.y[j] -= P.dcd[j] / (1.0 + lam);
    __syncthreads();
  }

  // initialize_algorithm!(solver, ::DualCentering) (:112-143); returns
  // false where the reference throws ErrorException.
  __noinline__ __device__ bool dc_initialize() {
    const double beta = prm.dc_beta;
    if (threadIdx.x == 0) {
      P.sc[SC_DC_NU] = (double)(nu() - P.ns);
      if (isnan(prm.dc_A)) {
        const double tau = 2.0 * beta / ((1.0 - beta) * (1.0 - beta));
        P.sc[SC_DC_A] = prm.dc_delta + (-tau - log1p(-tau));
      } else {
        P.sc[SC_DC_A] = prm.dc_A;
      }
      P.sc[SC_NNEWTON] = 0.0;
      P.sc[SC_NPRED] = 0.0;
      P.sc[SC_DC_T] = 0.0;
    }
    __syncthreads();
    if (!refresh_slacks()) return false;
    if (!newton_direction()) return false;
    // d = B grad(zeta) (t = 0) and dy = B b
    for (int j = threadIdx.x; j < P.m; j += NTHREADS) P.dcdy[j] = P.b[j];
    __syncthreads();
    schur_solve(P.dcdy);
    double bBb = 0.0, bBg = 0.0;
    for (int j = threadIdx.x; j < P.m; j += NTHREADS) {
      bBb = fma(P.b[j], P.dcdy[j], bBb);
      bBg = fma(P.b[j], P.dcd[j], bBg);
    }
    bBb = fmax(block_sum(bBb, &sh.rb), 2.220446049250313e-16);
    bBg = block_sum(bBg, &sh.rb);
    if (threadIdx.x == 0) P.sc[SC_DC_T] = fmax(bBg / bBb, beta / sqrt(bBb));
    __syncthreads();
    for (int it = 0; it < prm.centering_max_iter; ++it) {
      if (!newton_direction()) return false;
      if (P.sc[SC_DC_LAM] <= beta / 2) break;
      damped_newton_step();
      if (threadIdx.x == 0) { P.sc[SC_ITER] += 1.0; P.sc[SC_NNEWTON] += 1.0; }
      __syncthreads();
      if (!refresh_slacks()) return false;
    }
    if (threadIdx.x == 0) P.sc[SC_MU] = 1.0 / P.sc[SC_DC_T];
    __syncthreads();
    return true;
  }

  // xi(alpha) = sum -log(1 - alpha mu) - log(1 + alpha/(1-alpha) mu) over the
  // proximity eigenvalues of every block (:146-160); one warp.
  __device__ double xi_value(double alpha) {
    const int lane = threadIdx.x & 31;
    double s = 0.0;
    int bad = 0;
    const double b2 = alpha / (1.0 - alpha);
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      const T* ev = b.V(WV_EIG);
      for (int k = lane; k < b.n; k += 32) {
        const double mu = (double)ev[k];
        const double u = 1.0 - alpha * mu, v = 1.0 + b2 * mu;
        if (!(u > 0.0 && v > 0.0)) bad = 1;
        else s -= log(u) + log(v);
      }
    }
    s = warp_sum(s);
    bad = __any_sync(0xffffffffu, bad);
    return bad ? INFINITY : s;
  }

  // bisection on xi(alpha) = A (:163-201); one warp
  __device__ double solve_alpha(double A) {
    const int lane = threadIdx.x & 31;
    double amax = 1.0;
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      const T* ev = b.V(WV_EIG);
      for (int k = lane; k < b.n; k += 32) {
        const double mu = (double)ev[k];
        if (mu > 0.0) amax = fmin(amax, 1.0 / mu);
        if (mu < 0.0) amax = fmin(amax, 1.0 / (1.0 - mu));
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) amax = fmin(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    double hi = amax * 0.99999;
    const double xhi = xi_value(hi);
    if (!isfinite(xhi) || xhi < A) return hi;
    double lo = 0.0;
    for (int it = 0; it < 80; ++it) {
      const double mid = (lo + hi) / 2;
      if (xi_value(mid) < A) lo = mid;
      else hi = mid;
      if (hi - lo <= 2.220446049250313e-16 * fmax(1.0, hi)) break;
    }
    return (lo + hi) / 2;
  }

  // _predictor_step! (:232-264)
  __noinline__ __device__ bool predictor_step() {
    const double t = P.sc[SC_DC_T];
    for (int j = threadIdx.x; j < P.m; j += NTHREADS) {
      P.dcyhat[j] = P.y[j] + P.dcd[j];
      P.dcdy[j] = P.b[j];
    }
    __syncthreads();
    schur_solve(P.dcdy);
    for (int j = threadIdx.x; j < P.m; j += NTHREADS) P.dcdy[j] *= t;
    __syncthreads();
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      const int n = b.n;
      slack(b, P.dcyhat, b.Shat);                       // S_hat = sym(C - A*(y_hat))
      jtprod_combine(b, P.dcdy, 1.0, nullptr, nullptr, b.Dc);
      cta_symmetrize<double>(n, b.Dc);                  // D = sym(A*(dy))
      // eigenvalues of L_hat^-1 D L_hat^-T (:205-215)
      if (!chol_factor<T, double>(n, b.Shat, b.W(W_LX), true, smem, sh)) return false;
      tri_inverse<T>(n, b.W(W_LX), b.W(W_LXI), smem);
      T* dt = as_T<T>(b.nn, b.Dc, b.W(W_DXT));
      cta_gemm<T>(n, 0, 0, 1, 0, (T)1, b.W(W_LXI), dt, (T)0, b.W(W_T1), scr());
      cta_gemm<T>(n, 0, 1, 0, 1, (T)1, b.W(W_T1), b.W(W_LXI), (T)0, b.W(W_T2), scr());
      cta_symmetrize<T>(n, b.W(W_T2));
      if ((threadIdx.x >> 5) == 0)
        warp_lanczos_full<T>(n, b.W(W_T2), b.W(W_Q), b.V(WV_LA), b.V(WV_LB), b.V(WV_LW), b.V(WV_LC));
      __syncthreads();
      T* ev = b.V(WV_EIG);
      for (int k = threadIdx.x; k < n; k += NTHREADS) ev[k] = thread_tridiag_eig<T>(n, b.V(WV_LA), b.V(WV_LB), k);
      __syncthreads();
    }
    // ||s_hat||^2 = sum ||Ls^-1 S_hat Ls^-T||_F^2 (:219-229)
    double shat_n2 = 0.0;
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      T* st = as_T<T>(b.nn, b.Shat, b.W(W_DST));
      cta_gemm<T>(b.n, 0, 0, 1, 0, (T)1, b.W(W_LSI), st, (T)0, b.W(W_T1), scr());
      cta_gemm<T>(b.n, 0, 1, 0, 1, (T)1, b.W(W_T1), b.W(W_LSI), (T)0, b.W(W_T2), scr());
      const T* z = b.W(W_T2);
      double s2 = 0.0;
      for (int64_t k = threadIdx.x; k < b.nn; k += NTHREADS) s2 = fma((double)z[k], (double)z[k], s2);
      shat_n2 += block_sum(s2, &sh.rb);
    }
    if ((threadIdx.x >> 5) == 0) {
      const double alpha = solve_alpha(P.sc[SC_DC_A]);
      if (threadIdx.x == 0) sh.bc[6] = alpha;
    }
    __syncthreads();
    const double alpha = sh.bc[6];
    __syncthreads();
    if (threadIdx.x == 0) { P.sc[SC_ALPHA] = alpha; P.sc[SC_BETA] = alpha; }
    // primal estimate X = (1/t) S^-1 ((1-alpha) S_hat + alpha D) S^-1
    for (int i = 0; i < P.nblocks; ++i) {
      Blk<T> b = blk(i);
      T* buf = b.W(W_T3);
      for (int64_t k = threadIdx.x; k < b.nn; k += NTHREADS) buf[k] = (T)((1.0 - alpha) * b.Shat[k] + alpha * b.Dc[k]);
      __syncthreads();
      cta_gemm<T>(b.n, 0, 0, 0, 0, (T)1, b.W(W_SI), buf, (T)0, b.W(W_T1), scr());
      cta_gemm<T>(b.n, 0, 0, 0, 0, (T)(1.0 / t), b.W(W_T1), b.W(W_SI), (T)0, b.W(W_T2), scr());
      const T* xt = b.W(W_T2);
      for (int64_t k = threadIdx.x; k < b.nn; k += NTHREADS) b.X[k] = (double)xt[k];
      __syncthreads();
      cta_symmetrize<double>(b.n, b.X);
    }
    for (int j = threadIdx.x; j < P.m; j += NTHREADS) P.y[j] = P.dcyhat[j] + alpha * P.dcdy[j];
    __syncthreads();
    if (threadIdx.x == 0) {
      P.sc[SC_DC_T] = P.sc[SC_DC_NU] * t / ((1.0 - alpha) * shat_n2);
      P.sc[SC_NPRED] += 1.0;
    }
    __syncthreads();
    return true;
  }

  // iterate!(solver, ::DualCentering) (:266-289)
  __noinline__ __device__ void dc_iterate() {
    bool ok = newton_direction();
    if (ok) {
      const double lam = P.sc[SC_DC_LAM];
      if (lam > prm.dc_beta) {
        damped_newton_step();
        if (threadIdx.x == 0) {
          P.sc[SC_ALPHA] = P.sc[SC_BETA] = 1.0 / (1.0 + lam);
          P.sc[SC_NNEWTON] += 1.0;
        }
        __syncthreads();
      } else {
        ok = predictor_step();
      }
    }
    if (ok) {
      if (threadIdx.x == 0) P.sc[SC_ITER] += 1.0;
      __syncthreads();
      ok = refresh_slacks();
    }
    if (threadIdx.x == 0) {
      if (!ok) P.sc[SC_STATUS] = (double)MSDP_ERROR_IN_STEP_COMPUTATION;
      else P.sc[SC_MU] = 1.0 / P.sc[SC_DC_T];
    }
    __syncthreads();
  }
};

template <> __device__ __forceinline__ const double* Algo<double>::xt(const Blk<double>& b) const { return b.X; }
template <> __device__ __forceinline__ const float* Algo<float>::xt(const Blk<float>& b) const { return b.W(W_XT); }
template <> __device__ __forceinline__ double* Algo<double>::schur_H() { return P.H64; }
template <> __device__ __forceinline__ double* Algo<double>::schur_L() { return P.H64; }
template <> __device__ __forceinline__ float* Algo<float>::schur_H() { return P.Hf; }
template <> __device__ __forceinline__ float* Algo<float>::schur_L() { return P.Lf; }

// Stage the right-hand side (and the factor when it fits) in shared memory
// and solve with one warp.
template <class T>
__device__ void staged_potrs(int m, const T* L, double* x, unsigned char* smem) {
  const int64_t mm = (int64_t)m * m;
  double* sx = (double*)smem;
  T* sL = (T*)(smem + (((int64_t)m * sizeof(double) + 15) & ~(int64_t)15));
  double* rd = (double*)(smem + MSDP_SMEM_BYTES) - m;  // reciprocal diagonal at the end of the scratch
  const bool stageL = ((int64_t)m * sizeof(double) * 2 + 16 + mm * (int64_t)sizeof(T)) <= MSDP_SMEM_BYTES;
  for (int j = threadIdx.x; j < m; j += NTHREADS) sx[j] = x[j];
  if (stageL)
    for (int64_t k = threadIdx.x; k < mm; k += NTHREADS) sL[k] = L[k];
  __syncthreads();
  if ((threadIdx.x >> 5) == 0) warp_potrs<T, double>(m, stageL ? sL : L, sx, rd);
  __syncthreads();
  for (int j = threadIdx.x; j < m; j += NTHREADS) x[j] = sx[j];
  __syncthreads();
}

template <> __device__ void Algo<double>::schur_solve(double* x) {
  if (prm.schur == MSDP_MADNLP_SCHUR) {
    // MadNLPSchur: Bunch-Kaufman solve (src/kkt.jl:27-32)
    if ((threadIdx.x >> 5) == 0) warp_sytrs_lower<double, double>(P.m, P.H64, P.m, P.piv, x);
    __syncthreads();
    return;
  }
  staged_potrs<double>(P.m, P.H64, x, smem);
}

template <> __device__ void Algo<float>::schur_solve(double* x) {
  // x0 = L^-T L^-1 h in float; then r = h - H x (float64 accumulation of
  // the float matrix) and x += solve(r), twice.
  const int m = P.m;
  double* h = P.wm;   // original right-hand side
  double* r = P.wm2;  // residual / correction
  for (int j = threadIdx.x; j < m; j += NTHREADS) { h[j] = x[j]; r[j] = x[j]; }
  __syncthreads();
  staged_potrs<float>(m, P.Lf, r, smem);
  for (int j = threadIdx.x; j < m; j += NTHREADS) x[j] = r[j];
  __syncthreads();
  for (int it = 0; it < 2; ++it) {
    for (int j = threadIdx.x; j < m; j += NTHREADS) {
      double s = h[j];
      for (int k = 0; k < m; ++k) s -= (double)P.Hf[j + (int64_t)k * m] * x[k];
      r[j] = s;
    }
    __syncthreads();
    staged_potrs<float>(m, P.Lf, r, smem);
    for (int j = threadIdx.x; j < m; j += NTHREADS) x[j] += r[j];
    __syncthreads();
  }
}

}  // namespace
