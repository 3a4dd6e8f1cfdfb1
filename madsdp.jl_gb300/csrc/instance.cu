// Whole-GPU solver for one large SDP (blocks of hundreds to thousands, m in
// the thousands): every step of the interior-point iteration is a sequence
// of device-wide operations on one stream.  Dense products, Cholesky
// factorizations and symmetric eigendecompositions go to cuBLAS/cuSOLVER;
// the Schur-complement assembly of sparse constraints, A(X), A*(y), the
// residuals, the NT scaling arithmetic, the Mehrotra correction and every
// reduction are kernels of this file.  The iteration restates
// src/primal_dual.jl, src/step.jl, src/directions.jl, src/blocks.jl and
// src/solver.jl (file:line at each step) with exact eigenvalues for the
// step lengths.
//
// Constraint storage is chosen per block: coordinate lists (assembly cost
// nnz^2 entry pairs: one-hot, Hankel, sparse) or dense n x n per constraint
// (assembly by GEMMs: H = svec(G'A_jG) svec(G'A_kG)' for NT,
// H_jk = <A_j, S^-1 A_k X> for HKM) when nnz^2 exceeds the dense cost.
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>
#include <atomic>
#include <memory>
#include <new>
#include <thread>

#include "../../include/madsdp_gpu.h"
#include "chol.h"
#include "eigref.h"
#include "la.cuh"
#include "tcgemm.h"
#include "tridiag.h"

struct msdp_context;
extern "C" void* msdp_context_stream(const msdp_context* ctx);

namespace {

constexpr double kEps = 2.220446049250313e-16;
constexpr int kThreads = 256;
constexpr int kRedBlocks = 304;
constexpr int kSlots = 8192;
constexpr int kInfos = 4096;

inline int grid_for(int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + kThreads - 1) / kThreads, 152 * 16));
}
double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// ------------------------------------------------------------------ kernels
enum { RED_DOT = 0, RED_MAXABS, RED_MINRATIO, RED_NONFINITE, RED_SUM, RED_MIN };

__device__ __forceinline__ double red_combine(int op, double a, double b) {
  if (op == RED_MINRATIO || op == RED_MIN) return fmin(a, b);
  if (op == RED_MAXABS) return fmax(a, b);
  return a + b;
}
__device__ __forceinline__ double red_identity(int op) {
  return (op == RED_MINRATIO || op == RED_MIN) ? INFINITY : 0.0;
}

// Block partials of a reduction over a[i * stride] (and b[i]); a fixed grid
// and tree make the result independent of timing.
__global__ void k_reduce(int op, int64_t n, int64_t stride, const double* __restrict__ a,
                         const double* __restrict__ b, double* __restrict__ partial) {
  double acc = red_identity(op);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double va = a[i * stride];
    double v;
    switch (op) {
      case RED_DOT: v = va * b[i]; break;
      case RED_MAXABS: v = fabs(va); break;
      case RED_MINRATIO: { const double d = b[i]; v = d < 0.0 ? -va / d : INFINITY; break; }
      case RED_NONFINITE: v = isfinite(va) ? 0.0 : 1.0; break;
      case RED_MIN: v = isnan(va) ? -INFINITY : va; break;  // NaN counts as not positive
      default: v = va;
    }
    acc = red_combine(op, acc, v);
  }
  __shared__ double sh[kThreads];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = red_combine(op, sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void k_reduce_final(int op, int np, const double* __restrict__ partial, double* __restrict__ out) {
  __shared__ double sh[kThreads];
  double acc = red_identity(op);
  for (int i = threadIdx.x; i < np; i += kThreads) acc = red_combine(op, acc, partial[i]);
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = red_combine(op, sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

// out = a*A + b*B + c*C + d*D + e*E, left to right; absent terms skipped.
// out may be one of the inputs (in-place updates such as X += a dX): no __restrict__
__global__ void k_lin(int64_t N, double* out, double a, const double* A, double b, const double* B,
                      double c, const double* Cc, double d, const double* D, double e, const double* E) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    double v = a * A[i];
    if (B) v = v + b * B[i];
    if (Cc) v = v + c * Cc[i];
    if (D) v = v + d * D[i];
    if (E) v = v + e * E[i];
    out[i] = v;
  }
}

// A = (A + A')/2 in place (src/blocks.jl:77-84).
// one double into device memory by kernel argument (no host source to keep alive)
__global__ void k_put_scalar(double* p, double v) { *p = v; }

__global__ void k_sym(int n, double* A) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < nn; idx += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(idx % n), j = (int)(idx / n);
    if (i > j) {
      const double v = (A[idx] + A[j + (int64_t)i * n]) / 2;
      A[idx] = v;
      A[j + (int64_t)i * n] = v;
    }
  }
}

// out = sym(R - T)
__global__ void k_sym_diff(int n, const double* R, const double* T, double* out) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < nn; idx += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(idx % n), j = (int)(idx / n);
    if (i >= j) {
      const int64_t t = j + (int64_t)i * n;
      const double v = ((R[idx] - T[idx]) + (R[t] - T[t])) / 2;
      out[idx] = v;
      out[t] = v;
    }
  }
}

__global__ void k_lower_to_full(int n, double* A) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < nn; idx += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(idx % n), j = (int)(idx / n);
    if (i < j) A[idx] = A[j + (int64_t)i * n];
  }
}

// Lower Cholesky factor post-processing (src/blocks.jl:101-111): the upper
// triangle is cleared and entries below eps^2 max|L_ii| are flushed to zero.
__global__ void k_chol_post(int n, double* L, const double* maxdiag) {
  const double tol = kEps * kEps * (*maxdiag);
  const int64_t nn = (int64_t)n * n;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < nn; idx += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(idx % n), j = (int)(idx / n);
    if (i < j || fabs(L[idx]) < tol) L[idx] = 0.0;
  }
}

__global__ void k_add_diag(int n, double* A, int64_t lda, double v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) A[i + i * lda] += v;
}

__global__ void k_identity(int n, double* A, double v) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < nn; idx += (int64_t)gridDim.x * blockDim.x)
    A[idx] = (idx % n == idx / n) ? v : 0.0;
}

__global__ void k_fill(int64_t N, double* a, double v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) a[i] = v;
}

// D = sqrt(lambda), sc = sqrt(D) (src/directions.jl:55-60)
__global__ void k_nt_scaling(int n, const double* lam, double* D, double* sc) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    D[i] = sqrt(lam[i]);
    sc[i] = sqrt(D[i]);
  }
}

// G[:, j] /= sc[j]
__global__ void k_div_cols(int n, double* G, const double* sc) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < nn; idx += (int64_t)gridDim.x * blockDim.x)
    G[idx] /= sc[idx / n];
}

// out[i + j n] = Q[j + i n] f[i]: the transpose of Q with its rows scaled
__global__ void k_scaled_transpose(int n, const double* __restrict__ Q, const double* __restrict__ f,
                                   double* __restrict__ out) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < nn; idx += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(idx % n), j = (int)(idx / n);
    out[idx] = Q[j + (int64_t)i * n] * f[i];
  }
}
// f = D^-3/2 = 1 / (D sc)
__global__ void k_gi_scale(int n, const double* __restrict__ D, const double* __restrict__ sc, double* __restrict__ f) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) f[i] = 1.0 / (D[i] * sc[i]);
}
// rows of A scaled: A[i, :] /= sc[i]
__global__ void k_div_rows(int n, double* A, const double* __restrict__ sc) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < nn; idx += (int64_t)gridDim.x * blockDim.x)
    A[idx] /= sc[idx % n];
}

// ---- Lanczos steps with the scalars kept on the device
// out[i] -= sum_j A[i + j lda] v[j]: 32 rows per block of 32 x 32 threads,
// thread (r, g) sums columns g, g + 32, ... (coalesced over r); the 32
// partial sums of a row are added in a fixed order
__global__ void __launch_bounds__(1024) k_gemv_sub(int64_t rows, int cols, const double* __restrict__ A, int64_t lda,
                                                  const double* __restrict__ v, double* __restrict__ out) {
  __shared__ double part[32][33];
  const int r = threadIdx.x & 31, g = threadIdx.x >> 5;
  const int64_t i = (int64_t)blockIdx.x * 32 + r;
  double s = 0.0;
  if (i < rows)
    for (int j = g; j < cols; j += 32) s = fma(A[i + j * lda], v[j], s);
  part[g][r] = s;
  __syncthreads();
  if (g == 0 && i < rows) {
    double t = 0.0;
    for (int q = 0; q < 32; ++q) t += part[q][r];
    out[i] -= t;
  }
}
// ---- one Lanczos step in fewer launches: each reduction leaves per-block
// partial sums, and the kernel that needs the total sums them itself in a
// fixed order (every block the same way), so results do not depend on
// timing and no separate reduction launch is needed.
__device__ __forceinline__ double block_sum256(double v, double* red) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < kThreads / 32; ++w) t += red[w];
  __syncthreads();
  return t;
}
// sum of np partials, identical in every block
__device__ __forceinline__ double sum_partials(const double* __restrict__ part, int np, double* red) {
  double v = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) v += part[i];
  return block_sum256(v, red);
}
// w = Z q (Z symmetric: column dots, one block per column as k_gemv_t) and
// part[b] = sum of q_j w_j over the columns of block b
__global__ void __launch_bounds__(kThreads) k_lz_matvec(int64_t n, const double* __restrict__ Z,
                                                        const double* __restrict__ q, double* __restrict__ w,
                                                        double* __restrict__ part) {
  __shared__ double red[kThreads / 32];
  double acc = 0.0;
  for (int64_t j = blockIdx.x; j < n; j += gridDim.x) {
    const double* a = Z + j * n;
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s = fma(a[i], q[i], s);
    const double t = block_sum256(s, red);
    if (threadIdx.x == 0) w[j] = t;
    acc = fma(q[j], t, acc);
  }
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}
// a = sum of the matvec's partials (stored to *pa by block 0),
// w -= a q + sqrt(*pbb) p (no p at the first step)
__global__ void __launch_bounds__(kThreads) k_lz_update(int64_t n, double* __restrict__ w, const double* __restrict__ q,
                                                        const double* __restrict__ p, const double* __restrict__ part,
                                                        int np, double* __restrict__ pa,
                                                        const double* __restrict__ pbb) {
  __shared__ double red[kThreads / 32];
  const double a = sum_partials(part, np, red);
  if (blockIdx.x == 0 && threadIdx.x == 0) *pa = a;
  const double b = p ? sqrt(*pbb) : 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    w[i] -= a * q[i] + (p ? b * p[i] : 0.0);
}
// k_gemv_sub, and part[b] = sum of the updated out_i^2 over the block's rows
__global__ void __launch_bounds__(1024) k_gemv_sub_dot(int64_t rows, int cols, const double* __restrict__ A,
                                                      int64_t lda, const double* __restrict__ v,
                                                      double* __restrict__ out, double* __restrict__ part) {
  __shared__ double pr[32][33];
  const int r = threadIdx.x & 31, g = threadIdx.x >> 5;
  const int64_t i = (int64_t)blockIdx.x * 32 + r;
  double s = 0.0;
  if (i < rows)
    for (int j = g; j < cols; j += 32) s = fma(A[i + j * lda], v[j], s);
  pr[g][r] = s;
  __syncthreads();
  if (g == 0) {
    double t = 0.0, sq = 0.0;
    if (i < rows) {
      for (int q = 0; q < 32; ++q) t += pr[q][r];
      const double o = out[i] - t;
      out[i] = o;
      sq = o * o;
    }
    for (int o = 16; o; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
    if (r == 0) part[blockIdx.x] = sq;
  }
}
// bb = sum of the partials (stored to *pbb by block 0), out = w / sqrt(bb)
__global__ void __launch_bounds__(kThreads) k_lz_normalize(int64_t n, const double* __restrict__ w,
                                                           const double* __restrict__ part, int np,
                                                           double* __restrict__ pbb, double* __restrict__ out) {
  __shared__ double red[kThreads / 32];
  const double bb = sum_partials(part, np, red);
  if (blockIdx.x == 0 && threadIdx.x == 0) *pbb = bb;
  const double inv = 1.0 / sqrt(bb);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = w[i] * inv;
}
int64_t lanczos_partials(int64_t n) { return std::min<int64_t>(n, 152 * 16) + (n + 31) / 32 + 1; }

// 64-bit copy of sytrf's pivot indices (the solve's format)
__global__ void k_ipiv64(int m, const int* __restrict__ p, int64_t* __restrict__ q) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) q[i] = p[i];
}

// out = -(M + M') ./ (D_i + D_j)  (src/directions.jl:90-100)
__global__ void k_rnt(int n, const double* M, const double* D, double* out) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < nn; idx += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(idx % n), j = (int)(idx / n);
    out[idx] = -(M[idx] + M[j + (int64_t)i * n]) / (D[i] + D[j]);
  }
}

// out[r, c] = A[r, c] * w[c]  (rows x cols, column-major)
__global__ void k_scale_cols(int64_t rows, int64_t cols, const double* A, const double* w, double* out) {
  const int64_t N = rows * cols;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < N; idx += (int64_t)gridDim.x * blockDim.x)
    out[idx] = A[idx] * w[idx / rows];
}

// Scalar block helpers (src/step.jl:63-124, 128-136)
__global__ void k_inv(int ns, const double* z, double* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) out[i] = 1.0 / z[i];
}
__global__ void k_mul(int ns, const double* a, const double* b, double* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) out[i] = a[i] * b[i];
}
// v = x - mu zinv + x zinv Rd_lin [- corr]
__global__ void k_rhs_lin(int ns, double mu, const double* x, const double* zinv, const double* rdl, const double* corr,
                          double* v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
    double t = x[i] - mu * zinv[i] + x[i] * zinv[i] * rdl[i];
    if (corr) t = t - corr[i];
    v[i] = t;
  }
}
// delz = Rd_lin - C'dy ; delx = mu zinv - x - x zinv delz [+ corr]
__global__ void k_dir_lin(int ns, double mu, const double* rdl, const double* ctdy, const double* x, const double* zinv,
                          const double* corr, double* delz, double* delx) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
    const double dz = rdl[i] - ctdy[i];
    double dx = mu * zinv[i] - x[i] - x[i] * zinv[i] * dz;
    if (corr) dx = dx + corr[i];
    delz[i] = dz;
    delx[i] = dx;
  }
}
__global__ void k_corr_lin(int ns, const double* dx, const double* dz, const double* zinv, double* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x)
    out[i] = -dx[i] * dz[i] * zinv[i];
}
// (x + a dx)(z + b dz)
__global__ void k_aff_lin(int ns, double a, double b, const double* x, const double* dx, const double* z,
                          const double* dz, double* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x)
    out[i] = (x[i] + a * dx[i]) * (z[i] + b * dz[i]);
}

// svec of m symmetric n x n matrices (column-major upper triangle,
// off-diagonal entries times sqrt 2): <B_j, B_k> = svec(B_j) . svec(B_k)
// One eigenproblem of a step-length evaluation (n x n basis, 4 (n + 1)
// work entries, result slot).
struct LanczosJob {
  int n;
  const double* Z;
  double* Q;   // n x n basis
  double* ws;  // 4 (n + 1)
  double* out;
};

// lambda_min of formed symmetric Z (n <= 256), one thread block of 256
// threads per matrix: row i of each Lanczos vector on thread i, the basis in
// global memory, full reorthogonalization twice (warp w forms the
// coefficients of basis vectors w, w + 8, ...), and the stopping rule of the
// one-warp routine of la.cuh: the smallest Ritz value of the tridiagonal
// every 4 steps, stop once it moves by at most 64 eps max(1, |theta|) or the
// Krylov space is exhausted.
constexpr int kLanczosCta = 256;
__device__ __forceinline__ double cta_sum256(double x, double* red) {
  x = warp_sum(x);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
  __syncthreads();
  double t = 0.0;
#pragma unroll
  for (int w = 0; w < kLanczosCta / 32; ++w) t += red[w];
  __syncthreads();
  return t;
}
__global__ void __launch_bounds__(kLanczosCta) k_lanczos_cta(const LanczosJob* __restrict__ jobs) {
  const LanczosJob J = jobs[blockIdx.x];
  const int n = J.n, i = threadIdx.x, lane = i & 31, wid = i >> 5;
  __shared__ double qs[kLanczosCta], ws[kLanczosCta], coef[kLanczosCta + 1], red[kLanczosCta / 32];
  __shared__ double theta_s;
  double* a = J.ws;
  double* bb = a + (n + 1);
  double* Q = J.Q;
  const bool own = i < n;
  double v = 0.0;
  if (own) {
    uint32_t h = (uint32_t)(i + 1) * 2654435761u;
    h ^= h >> 15; h *= 2246822519u; h ^= h >> 13;
    v = (double)(h & 0xffffff) / 16777216.0 - 0.5 + 0.01;
  }
  const double nrm = sqrt(cta_sum256(v * v, red));
  if (own) {
    v /= nrm;
    Q[i] = v;
    qs[i] = v;
  }
  if (i == 0) bb[0] = 0.0;
  __syncthreads();
  double theta = 0.0, theta_prev = INFINITY, znorm = 0.0;
  for (int j = 0; j < n; ++j) {
    double w = 0.0, w1 = 0.0;
    if (own) {
      int r = 0;
      for (; r + 1 < n; r += 2) {
        w = fma(J.Z[i + (int64_t)r * n], qs[r], w);
        w1 = fma(J.Z[i + (int64_t)(r + 1) * n], qs[r + 1], w1);
      }
      if (r < n) w = fma(J.Z[i + (int64_t)r * n], qs[r], w);
      w += w1;
    }
    const double aj = cta_sum256(own ? qs[i] * w : 0.0, red);
    const double bj = j > 0 ? bb[j] : 0.0;
    if (own) w -= aj * qs[i] + (j > 0 ? bj * Q[i + (int64_t)(j - 1) * n] : 0.0);
    if (i == 0) a[j] = aj;
    for (int pass = 0; pass < 2; ++pass) {
      if (own) ws[i] = w;
      __syncthreads();
      for (int l = wid; l <= j; l += kLanczosCta / 32) {
        const double* ql = Q + (int64_t)l * n;
        double t = 0.0;
        for (int r = lane; r < n; r += 32) t = fma(ql[r], ws[r], t);
        t = warp_sum(t);
        if (lane == 0) coef[l] = t;
      }
      __syncthreads();
      if (own)
        for (int l = 0; l <= j; ++l) w = fma(-coef[l], Q[i + (int64_t)l * n], w);
    }
    const double bn = sqrt(cta_sum256(own ? w * w : 0.0, red));
    const int k = j + 1;
    znorm = fmax(znorm, fabs(aj) + bn + fabs(bj));
    if (i == 0) bb[j + 1] = bn;
    const bool exhausted = (k == n) || !(bn > 2.220446049250313e-16 * znorm * 4.0);
    if (exhausted || (k >= 4 && (k % 4) == 0)) {
      __syncthreads();
      if (wid == 0) {
        const double th = warp_tridiag_eigmin<double>(k, a, bb);
        if (lane == 0) theta_s = th;
      }
      __syncthreads();
      theta = theta_s;
      const double tolr = 2.220446049250313e-16 * 64.0 * fmax(1.0, fabs(theta));
      if (exhausted || fabs(theta - theta_prev) <= tolr) break;
      theta_prev = theta;
    }
    if (own) {
      const double q = w / bn;
      Q[i + (int64_t)(j + 1) * n] = q;
      qs[i] = q;
    }
    __syncthreads();
  }
  if (i == 0) *J.out = theta;
}

// ---- coordinate-list constraints of one block
// out[j] (+)= sum_{e in j} v_e X[r_e, c_e]
__global__ void k_jprod(int m, const int64_t* __restrict__ conptr, const int32_t* __restrict__ row,
                        const int32_t* __restrict__ col, const double* __restrict__ val, int n,
                        const double* __restrict__ X, double* __restrict__ out, int accumulate) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < m; j += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int64_t q = conptr[j]; q < conptr[j + 1]; ++q) s += val[q] * X[row[q] + (int64_t)col[q] * n];
    out[j] = accumulate ? out[j] + s : s;
  }
}

// out[p] = sum_{e at position p} v_e y[con_e]
__global__ void k_jtprod(int64_t nn, const int64_t* __restrict__ posptr, const int32_t* __restrict__ pcon,
                         const double* __restrict__ pval, const double* __restrict__ y, double* __restrict__ out) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nn; p += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int64_t q = posptr[p]; q < posptr[p + 1]; ++q) s += pval[q] * y[pcon[q]];
    out[p] = s;
  }
}

// ---- dense constraints stored as Aall (n^2 x m, column j = vec(A_j)) and
// the m x ns C_lin: matrix-vector products that stream the matrix once.
// out[i] = sum_j A[i + j lda] v[j]  (i < rows): thread per row, columns in order
__global__ void k_gemv_n(int64_t rows, int cols, const double* __restrict__ A, int64_t lda,
                         const double* __restrict__ v, double* __restrict__ out, int accumulate) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < rows; i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int j = 0; j < cols; ++j) s = fma(A[i + j * lda], v[j], s);
    out[i] = accumulate ? out[i] + s : s;
  }
}
// The same for many columns in two passes: partial sums of kGemvChunks
// column ranges (grid y), then their sum in a fixed order (deterministic).
constexpr int kGemvChunks = 16;
__global__ void k_gemv_n_part(int64_t rows, int cols, const double* __restrict__ A, int64_t lda,
                              const double* __restrict__ v, double* __restrict__ part) {
  const int per = (cols + kGemvChunks - 1) / kGemvChunks;
  const int j0 = blockIdx.y * per, j1 = min(cols, j0 + per);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < rows; i += (int64_t)gridDim.x * blockDim.x) {
    double s0 = 0.0, s1 = 0.0;
    int j = j0;
    for (; j + 1 < j1; j += 2) {
      s0 = fma(A[i + j * lda], v[j], s0);
      s1 = fma(A[i + (j + 1) * lda], v[j + 1], s1);
    }
    if (j < j1) s0 = fma(A[i + j * lda], v[j], s0);
    part[blockIdx.y * rows + i] = s0 + s1;
  }
}
__global__ void k_gemv_n_sum(int64_t rows, const double* __restrict__ part, double* __restrict__ out, int accumulate) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < rows; i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int c = 0; c < kGemvChunks; ++c) s += part[c * rows + i];
    out[i] = accumulate ? out[i] + s : s;
  }
}
// out[j] (+)= sum_i A[i + j lda] v[i]  (j < cols): one block per column,
// fixed reduction tree (deterministic)
__global__ void k_gemv_t(int64_t rows, int cols, const double* __restrict__ A, int64_t lda,
                         const double* __restrict__ v, double* __restrict__ out, int accumulate) {
  __shared__ double red[kThreads / 32];
  for (int j = blockIdx.x; j < cols; j += gridDim.x) {
    const double* a = A + (int64_t)j * lda;
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < rows; i += blockDim.x) s = fma(a[i], v[i], s);
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < kThreads / 32; ++w) t += red[w];
      out[j] = accumulate ? out[j] + t : t;
    }
    __syncthreads();
  }
}

// ---- rank-one constraint blocks: A_j = sg_j v_j v_j' with V = [v_1 ... v_m]
// H[j, k] += sg_j sg_k Q1[j, k] Q2[j, k] for j >= k (NT: Q1 = Q2 = V'WV;
// HKM: Q1 = V'S^-1 V, Q2 = V'XV)
__global__ void k_lowrank_schur(int m, const double* __restrict__ Q1, const double* __restrict__ Q2,
                                const double* __restrict__ sg, double* __restrict__ H) {
  const int64_t mm = (int64_t)m * m;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < mm; idx += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(idx % m), k = (int)(idx / m);
    if (j >= k) H[idx] += sg[j] * sg[k] * Q1[idx] * Q2[idx];
  }
}
// out[j] (+)= sg_j sum_r V[r + j n] P[r + j n]  (one block per column)
__global__ void k_lowrank_dots(int n, int m, const double* __restrict__ V, const double* __restrict__ P,
                               const double* __restrict__ sg, double* __restrict__ out, int accumulate) {
  __shared__ double red[kThreads / 32];
  for (int j = blockIdx.x; j < m; j += gridDim.x) {
    const double* v = V + (int64_t)j * n;
    const double* q = P + (int64_t)j * n;
    double s = 0.0;
    for (int r = threadIdx.x; r < n; r += blockDim.x) s = fma(v[r], q[r], s);
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < kThreads / 32; ++w) t += red[w];
      t *= sg[j];
      out[j] = accumulate ? out[j] + t : t;
    }
    __syncthreads();
  }
}
// Vs[r + j n] = V[r + j n] sg_j y_j
__global__ void k_lowrank_scale(int n, int m, const double* __restrict__ V, const double* __restrict__ sg,
                                const double* __restrict__ y, double* __restrict__ Vs) {
  const int64_t nm = (int64_t)n * m;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < nm; idx += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(idx / n);
    Vs[idx] = V[idx] * sg[j] * y[j];
  }
}

// H[j, k] += <A_j, L A_k R> for j >= k: sum over entry pairs
// v_e v_f L[r_e, r_f] R[c_f, c_e] (the semantics of LowRankOpt's
// schur_complement!, src/solver.jl:30-31,117-118).
__global__ void k_schur_pairs(int m, const int64_t* __restrict__ conptr, const int32_t* __restrict__ row,
                              const int32_t* __restrict__ col, const double* __restrict__ val, int n,
                              const double* __restrict__ L, const double* __restrict__ R, double* __restrict__ H) {
  const int64_t npairs = (int64_t)m * (m + 1) / 2;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < npairs; p += (int64_t)gridDim.x * blockDim.x) {
    int64_t j = (int64_t)((sqrt(8.0 * (double)p + 1.0) - 1.0) / 2.0);
    while (j * (j + 1) / 2 > p) --j;
    while ((j + 1) * (j + 2) / 2 <= p) ++j;
    const int64_t k = p - j * (j + 1) / 2;
    double s = 0.0;
    for (int64_t e = conptr[j]; e < conptr[j + 1]; ++e) {
      const int re = row[e], ce = col[e];
      const double ve = val[e];
      double t = 0.0;
      for (int64_t f = conptr[k]; f < conptr[k + 1]; ++f)
        t += val[f] * L[re + (int64_t)row[f] * n] * R[col[f] + (int64_t)ce * n];
      s += ve * t;
    }
    H[j + k * (int64_t)m] += s;
  }
}

// ------------------------------------------------------------------ host state
struct Blk {
  int n = 0;
  bool dense = false;
  int64_t nnz = 0;
  double cnorm = 0.0;
  bool rd_nonzero = true;
  double *C = nullptr, *X = nullptr, *S = nullptr, *Rd = nullptr, *Ls = nullptr, *Si = nullptr, *Lx = nullptr;
  double *W = nullptr, *G = nullptr, *Gi = nullptr, *dX = nullptr, *dS = nullptr, *corr = nullptr, *ERd = nullptr;
  double *T1 = nullptr, *T2 = nullptr, *T3 = nullptr;
  double *lam = nullptr, *D = nullptr, *sc = nullptr, *w = nullptr;
  int64_t *conptr = nullptr, *posptr = nullptr;
  int32_t *erow = nullptr, *ecol = nullptr, *pcon = nullptr;
  double *eval = nullptr, *pval = nullptr;
  double* Aall = nullptr;  // dense: n x (n m), column j*n.. of A_j
  // rank-one constraints (every A_j = sg_j v_j v_j'): V (n x m), signs,
  // V's columns sliced as rows (K = n) in both precisions, V's rows (K = m),
  // and an n x m temporary
  bool lowrank = false;
  double *V = nullptr, *sg = nullptr, *P = nullptr;
  tcg::Sliced vk[2], vr;
  // NT: Gs = G D^-1/2 and Hx = D^-1/2 Gi for S^-1 = Gs Gs' and the
  // step-length matrices Hx dX Hx', Gs' dS Gs (orthogonally similar to
  // Lx^-1 dX Lx^-T and Ls^-1 dS Ls^-T)
  double *Gs = nullptr, *Hx = nullptr, *gif = nullptr;
  // dense constraints on the tensor cores (sliced once at creation):
  // [A_1; ...; A_m] as rows (j, r) with K = n, in the FP64 (7) and, for the
  // mixed precision, the mixed (3) slicing; HKM also vec(A_j) rows, K = n^2
  tcg::Sliced stk[2], vec[2];
  int2* kmap = nullptr;  // NT: symmetric-vector index -> (row, column), row >= column
};

}  // namespace

struct msdp_solver {
  msdp_context* ctx = nullptr;
  cudaStream_t st = nullptr;
  cublasHandle_t cb = nullptr;
  cusolverDnHandle_t cs = nullptr;
  msdp_components comp{};
  msdp_options opt{};
  int m = 0, ns = 0, nb = 0;
  std::vector<Blk> B;
  std::vector<void*> allocs;
  int64_t bytes = 0;
  double *b = nullptr, *dlin = nullptr, *Clin = nullptr, *Cw = nullptr;
  double *y = nullptr, *dy = nullptr, *Rp = nullptr, *h = nullptr, *acc = nullptr;
  double *x = nullptr, *z = nullptr, *dx = nullptr, *dz = nullptr, *Rdlin = nullptr, *zinv = nullptr;
  double *corrlin = nullptr, *vlin = nullptr, *ctv = nullptr, *wlin = nullptr;
  double *H = nullptr, *H0 = nullptr, *Tb = nullptr, *Bb = nullptr;
  double* gpart = nullptr;  // partial sums of the dense A*(y) (kGemvChunks x n^2)
  double *Q1 = nullptr, *Q2 = nullptr;  // m x m products of the rank-one assembly
  tcg::Sliced tL;                        // operand slices of the rank-one products (n x m or m x n)
  void* tLm = nullptr;
  // tensor-core products: operand slices of the n x n products (tA, tB),
  // the per-iteration operands of the dense assembly (tQ, tS), C_lin and
  // C_lin diag(x/z) (tCl, tCw), the fixed-point workspace and error flag
  tcg::Sliced tA, tB, tQ, tS, tCl[2], tCw;
  void *tAm = nullptr, *tBm = nullptr, *tQm = nullptr, *tSm = nullptr, *tCwm = nullptr;
  long long* tfix = nullptr;
  int64_t tfix_len = 0;
  int* terr = nullptr;
  int64_t tc_products = 0;  // tensor-core products issued
  chol::Work cw, cwH;       // blocked Cholesky: blocks, and the Schur matrix (kept for its solves)
  int* hinfo_dev = nullptr; // status of the Schur factor
  // MadNLPSchur: Bunch-Kaufman LDL' of the Schur matrix (cuSOLVER sytrf /
  // sytrs, whose solve takes 64-bit pivot indices)
  int* ipiv = nullptr;
  int64_t* ipiv64 = nullptr;
  double* sywork = nullptr;
  int sylwork = 0;
  void* sytrs_dev = nullptr;
  size_t sytrs_dev_bytes = 0;
  std::vector<char> sytrs_host;
  // mixed precision: split-precision assembly and FP32-class factor with
  // FP64 iterative refinement while `mixed_on`; FP64 after a stall
  bool mixed_on = false;
  double reg_used = 0.0;
  double *ir_r = nullptr, *ir_d = nullptr, *ir_h = nullptr;
  int n32 = 0, n64 = 0;            // iterations by Schur precision
  int64_t ir_steps = 0, ir_fallbacks = 0;
  double* work = nullptr;
  int lwork = 0;
  // NT eigendecomposition by an FP32 eigensolver and FP64 refinement
  // (eigref.h): FP32 matrix and eigenvalues, its workspace, index workspace
  float *ef32 = nullptr, *ework32 = nullptr;
  int elwork32 = 0;
  int* eibuf = nullptr;
  int64_t eig_refined = 0, eig_dense = 0, eig_steps = 0;
  int64_t lanczos_calls = 0, lanczos_steps = 0, eigmin_dense = 0;  // lambda_min of blocks above 256
  double *lq = nullptr, *lh = nullptr;  // Lanczos basis (n x (kLanczosMax + 1)) and projections
  double* lzp = nullptr;                 // per-block partial sums of the fused Lanczos step
  double *lq2 = nullptr, *lw2 = nullptr;  // bases and work of the batched device Lanczos
  void* ljobs = nullptr;
  int* dinfo = nullptr;
  double *partial = nullptr, *slots = nullptr;
  double* hslots = nullptr;
  int* hinfo = nullptr;
  int nslot = 0, ninfo = 0;
  double bnorm = 0.0, dnorm = 0.0, cmax = 0.0;
  // user initial point
  bool has_ip = false;
  std::vector<std::vector<double>> ipX;
  std::vector<double> ipy, ipx;
  // iteration state
  int status = MSDP_INITIAL, iter = 0;
  double mu = 0, sigma = 0, alpha = 0, beta = 0, inf_pr = 0, inf_du = 0, gap = 0, pobj = 0, dobj = 0;
  double t0 = 0, solve_s = 0;
  std::vector<msdp_iter_record> traj;
  int64_t launches = 0;
  int fail = 0;  // first library/CUDA error seen
  std::string err;
  // per-phase device time: events recorded at phase starts, read after the
  // synchronization that ends each iteration
  cudaEvent_t ev[64] = {};
  int ev_phase[64] = {};
  int nev = 0;
  double phase_s[16] = {};
};

namespace {

using S = msdp_solver;

enum { PH_PREPARE = 0, PH_ASSEMBLY, PH_FACTOR, PH_DIRECTIONS, PH_STEP, PH_CORRECTION, PH_STEP_UPDATE, PH_COUNT };
const char* kPhaseNames[PH_COUNT] = {"prepare", "schur_assembly", "schur_factor", "directions",
                                     "step_lengths", "correction", "take_step_residuals"};

void mark(S* s, int phase) {
  if (s->nev >= 64 || !s->ev[s->nev]) return;
  cudaEventRecord(s->ev[s->nev], s->st);
  s->ev_phase[s->nev] = phase;
  s->nev += 1;
}

// Close the open phase segments (the stream must be idle).
void collect_marks(S* s) {
  if (s->nev == 0) return;
  if (s->nev < 64 && s->ev[s->nev]) {
    cudaEventRecord(s->ev[s->nev], s->st);
    cudaEventSynchronize(s->ev[s->nev]);
    for (int k = 0; k < s->nev; ++k) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, s->ev[k], s->ev[k + 1]) == cudaSuccess) s->phase_s[s->ev_phase[k]] += 1e-3 * ms;
    }
  }
  s->nev = 0;
}

#define LAUNCH(s, kern, n, ...)                                          \
  do {                                                                   \
    kern<<<grid_for(n), kThreads, 0, (s)->st>>>(__VA_ARGS__);            \
    (s)->launches += 1;                                                  \
  } while (0)

void note(S* s, bool ok, const char* what) {
  if (!ok && !s->fail) {
    s->fail = MSDP_ERR_CUDA;
    s->err = what;
  }
}
#define CB(s, call) note(s, (call) == CUBLAS_STATUS_SUCCESS, #call)
#define CS(s, call) note(s, (call) == CUSOLVER_STATUS_SUCCESS, #call)
#define CU(s, call) note(s, (call) == cudaSuccess, #call)

template <class T>
T* dalloc(S* s, int64_t count) {
  void* p = nullptr;
  if (count <= 0) count = 1;
  if (cudaMalloc(&p, sizeof(T) * count) != cudaSuccess) return nullptr;
  s->allocs.push_back(p);
  s->bytes += sizeof(T) * count;
  return (T*)p;
}

// Host data to the device on the solver's stream, complete on return (the
// source may be pageable and short-lived; the legacy default stream is not
// ordered with the solver's non-blocking stream, so no upload goes there).
cudaError_t upload(S* s, void* dst, const void* src, size_t bytes) {
  if (!bytes) return cudaSuccess;
  const cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s->st);
  return e != cudaSuccess ? e : cudaStreamSynchronize(s->st);
}

// ---- reductions into slots
// A fresh device scalar slot; past kSlots the solver fails instead of
// writing beyond the slot arrays.
int next_slot(S* s) {
  if (s->nslot < kSlots) return s->nslot++;
  if (!s->fail) {
    s->fail = MSDP_ERR_CUDA;
    s->err = "device scalar slots exhausted";
  }
  return kSlots - 1;
}

int reduce(S* s, int op, int64_t n, const double* a, const double* b = nullptr, int64_t stride = 1) {
  const int slot = next_slot(s);
  if (n <= 0) {
    LAUNCH(s, k_fill, 1, 1, s->slots + slot, (op == RED_MINRATIO || op == RED_MIN) ? INFINITY : 0.0);
    return slot;
  }
  k_reduce<<<kRedBlocks, kThreads, 0, s->st>>>(op, n, stride, a, b, s->partial);
  k_reduce_final<<<1, kThreads, 0, s->st>>>(op, kRedBlocks, s->partial, s->slots + slot);
  s->launches += 2;
  return slot;
}

int copy_slot(S* s, const double* src) {
  const int slot = next_slot(s);
  CU(s, cudaMemcpyAsync(s->slots + slot, src, sizeof(double), cudaMemcpyDeviceToDevice, s->st));
  return slot;
}

// Bring every slot and info written since the last fetch to the host.
bool fetch(S* s) {
  if (s->nslot) CU(s, cudaMemcpyAsync(s->hslots, s->slots, sizeof(double) * s->nslot, cudaMemcpyDeviceToHost, s->st));
  if (s->ninfo) CU(s, cudaMemcpyAsync(s->hinfo, s->dinfo, sizeof(int) * s->ninfo, cudaMemcpyDeviceToHost, s->st));
  CU(s, cudaStreamSynchronize(s->st));
  return !s->fail;
}
void reset_slots(S* s) { s->nslot = 0; s->ninfo = 0; }
int next_info(S* s) { return s->ninfo < kInfos ? s->ninfo++ : kInfos - 1; }

// ---- tensor-core products (tcgemm.h)
// Bind an operand's slices to rows x K (tensor maps re-encoded only when the
// shape changes; the slicer writes every padded entry, so no clearing).
bool tc_bind(S* s, tcg::Sliced* sl, void* mem, int64_t rows, int64_t K, int ns) {
  if (sl->s && sl->rows == rows && sl->K == K && sl->ns == ns) return true;
  const bool ok = tcg::sliced_init(sl, mem, rows, K, ns, s->st, false) == cudaSuccess;
  note(s, ok, "tcg::sliced_init");
  return ok;
}
void tc_slice(S* s, const tcg::Source& src, tcg::Sliced* sl) {
  note(s, tcg::slice(src, sl, s->st) == cudaSuccess, "tcg::slice");
  s->launches += 2;
}
void tc_product(S* s, const tcg::Sliced& A, const tcg::Sliced& B, tcg::Mode mode, double* C, int64_t ldc, double alpha,
                double beta, bool lower) {
  tcg::Out o;
  o.C = C;
  o.ldc = ldc;
  o.alpha = alpha;
  o.beta = beta;
  o.lower = lower;
  o.fix = s->tfix;
  o.ldfix = A.rows;
  o.err = s->terr;
  if (tcg::needs_fix(A, B, mode, o) && A.rows * B.rows > s->tfix_len) {
    note(s, false, "tensor-core product: fixed-point workspace too small");
    return;
  }
  note(s, tcg::gemm(A, B, mode, o, s->st, &s->launches) == cudaSuccess, "tcg::gemm");
  s->tc_products += 1;
}
// Row operand for op(M): element (r, k) of op(M) (rows x K), M column-major.
tcg::Source op_rows(const double* Mp, int64_t ld, bool trans, int64_t rows, int64_t K) {
  tcg::Source src;
  src.p = Mp;
  src.rows = rows;
  src.K = K;
  src.nr = rows;
  src.bs = 0;
  src.rs = trans ? ld : 1;
  src.ks = trans ? 1 : ld;
  return src;
}

// ---- dense linear algebra
// Products whose dimensions are all at most kSmallGemm are one launch of a
// plain FP64 kernel: at that size the tensor-core path's five launches
// (row exponents and slices of both operands, then the product) cost more
// time than the arithmetic.
constexpr int kSmallGemm = 128;
constexpr int kSgTile = 16;

// C = alpha op(A) op(B) + beta C on CUDA cores (FP64), 16 x 16 output tiles
// with both operand tiles staged in shared memory; lower: only i >= j.
__global__ void __launch_bounds__(kSgTile * kSgTile)
    k_dgemm_small(int m, int n, int k, int ta, int tb, double alpha, const double* __restrict__ A, int lda,
                  const double* __restrict__ B, int ldb, double beta, double* C, int ldc, int lower) {
  __shared__ double As[kSgTile][kSgTile + 1], Bs[kSgTile][kSgTile + 1];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i = blockIdx.x * kSgTile + tx, j = blockIdx.y * kSgTile + ty;
  double acc = 0.0;
  for (int k0 = 0; k0 < k; k0 += kSgTile) {
    // As[r][c] = op(A)(blockrow + r, k0 + c), Bs[r][c] = op(B)(k0 + r, blockcol + c)
    {
      const int r = tx, c = ty, gi = blockIdx.x * kSgTile + r, gk = k0 + c;
      As[r][c] = (gi < m && gk < k) ? (ta ? A[gk + (int64_t)gi * lda] : A[gi + (int64_t)gk * lda]) : 0.0;
      const int gk2 = k0 + tx, gj = blockIdx.y * kSgTile + ty;
      Bs[tx][ty] = (gk2 < k && gj < n) ? (tb ? B[gj + (int64_t)gk2 * ldb] : B[gk2 + (int64_t)gj * ldb]) : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int l = 0; l < kSgTile; ++l) acc = fma(As[tx][l], Bs[l][ty], acc);
    __syncthreads();
  }
  if (i < m && j < n && (!lower || i >= j)) {
    double* c = C + i + (int64_t)j * ldc;
    *c = beta == 0.0 ? alpha * acc : alpha * acc + beta * *c;
  }
}
void small_gemm(S* s, int ta, int tb, int m, int n, int k, double alpha, const double* A, int lda, const double* B,
                int ldb, double beta, double* C, int ldc, bool lower) {
  const dim3 block(kSgTile, kSgTile), grid((m + kSgTile - 1) / kSgTile, (n + kSgTile - 1) / kSgTile);
  k_dgemm_small<<<grid, block, 0, s->st>>>(m, n, k, ta, tb, alpha, A, lda, B, ldb, beta, C, ldc, lower ? 1 : 0);
  s->launches += 1;
}

// C = alpha op(A) op(B) + beta C (FP64-accurate tensor-core product)
void gemm(S* s, cublasOperation_t ta, cublasOperation_t tb, int m, int n, int k, double alpha, const double* A, int lda,
          const double* Bm, int ldb, double beta, double* C, int ldc) {
  if (m <= kSmallGemm && n <= kSmallGemm && k <= kSmallGemm) {
    small_gemm(s, ta != CUBLAS_OP_N, tb != CUBLAS_OP_N, m, n, k, alpha, A, lda, Bm, ldb, beta, C, ldc, false);
    return;
  }
  if (!tc_bind(s, &s->tA, s->tAm, m, k, 7) || !tc_bind(s, &s->tB, s->tBm, n, k, 7)) return;
  tc_slice(s, op_rows(A, lda, ta != CUBLAS_OP_N, m, k), &s->tA);
  tc_slice(s, op_rows(Bm, ldb, tb == CUBLAS_OP_N, n, k), &s->tB);
  tc_product(s, s->tA, s->tB, tcg::kFp64, C, ldc, alpha, beta, false);
}
// lower triangle of C = alpha op(A) op(A)' + beta C, op(A) n x k
void syrk(S* s, bool trans, int n, int k, double alpha, const double* A, int lda, double beta, double* C, int ldc) {
  if (n <= kSmallGemm && k <= kSmallGemm) {
    // op(A) op(A)': op(A) = A' when trans
    small_gemm(s, trans ? 1 : 0, trans ? 0 : 1, n, n, k, alpha, A, lda, A, lda, beta, C, ldc, true);
    return;
  }
  if (!tc_bind(s, &s->tA, s->tAm, n, k, 7)) return;
  tc_slice(s, op_rows(A, lda, trans, n, k), &s->tA);
  tc_product(s, s->tA, s->tA, tcg::kFp64, C, ldc, alpha, beta, true);
}

// potrf of the lower triangle of an n x n block in place (chol.h); returns
// the info index
int potrf(S* s, int n, double* A, int lda) {
  const int k = next_info(s);
  note(s, chol::potrf(s->cw, n, A, lda, s->dinfo + k, tcg::kFp64, s->st, &s->launches) == cudaSuccess,
       "chol::potrf");
  return k;
}

struct CholCheck {
  int info, nonfinite;
};

// Lower Cholesky factor of sym(M) with the flush (src/blocks.jl:94-113);
// success is known after fetch: info == 0 and no non-finite entry.
CholCheck chol_factor(S* s, int n, const double* M, double* L) {
  CU(s, cudaMemcpyAsync(L, M, sizeof(double) * n * n, cudaMemcpyDeviceToDevice, s->st));
  LAUNCH(s, k_sym, (int64_t)n * n, n, L);
  CholCheck c;
  c.nonfinite = reduce(s, RED_NONFINITE, (int64_t)n * n, L);
  c.info = potrf(s, n, L, n);
  const int md = reduce(s, RED_MAXABS, n, L, nullptr, n + 1);
  LAUNCH(s, k_chol_post, (int64_t)n * n, n, L, s->slots + md);
  return c;
}
bool chol_ok(S* s, const CholCheck& c) { return s->hinfo[c.info] == 0 && s->hslots[c.nonfinite] == 0.0; }

// ---- constraint operators of one block
void jprod(S* s, Blk& b, const double* X, double* out, bool accumulate) {
  if (b.lowrank) {
    // A(X)_j = sg_j v_j' X v_j: P = X V on the tensor cores, then column dots
    const int n = b.n;
    if (!tc_bind(s, &s->tA, s->tAm, n, n, 7)) return;
    tc_slice(s, op_rows(X, n, true, n, n), &s->tA);
    tc_product(s, s->tA, b.vk[0], tcg::kFp64, b.P, n, 1.0, 0.0, false);
    k_lowrank_dots<<<std::min(s->m, 152 * 16), kThreads, 0, s->st>>>(n, s->m, b.V, b.P, b.sg, out,
                                                                   accumulate ? 1 : 0);
    s->launches += 1;
  } else if (b.dense) {
    const int64_t nn = (int64_t)b.n * b.n;
    k_gemv_t<<<std::min(s->m, 152 * 16), kThreads, 0, s->st>>>(nn, s->m, b.Aall, nn, X, out, accumulate ? 1 : 0);
    s->launches += 1;
  } else {
    LAUNCH(s, k_jprod, s->m, s->m, b.conptr, b.erow, b.ecol, b.eval, b.n, X, out, accumulate ? 1 : 0);
  }
}

void jtprod(S* s, Blk& b, const double* yv, double* out) {
  const int64_t nn = (int64_t)b.n * b.n;
  if (b.lowrank) {
    // A*(y) = V diag(sg y) V'
    const int n = b.n, m = s->m;
    LAUNCH(s, k_lowrank_scale, (int64_t)n * m, n, m, b.V, b.sg, yv, b.P);
    if (!tc_bind(s, &s->tL, s->tLm, n, m, 7)) return;
    tc_slice(s, op_rows(b.P, n, false, n, m), &s->tL);
    tc_product(s, s->tL, b.vr, tcg::kFp64, out, n, 1.0, 0.0, false);
  } else if (b.dense) {
    // A*(y) streams all of A: columns split over kGemvChunks block rows
    const dim3 grid((unsigned)std::min<int64_t>((nn + kThreads - 1) / kThreads, 152 * 8), kGemvChunks);
    k_gemv_n_part<<<grid, kThreads, 0, s->st>>>(nn, s->m, b.Aall, nn, yv, s->gpart);
    LAUNCH(s, k_gemv_n_sum, nn, nn, s->gpart, out, 0);
    s->launches += 1;
  } else {
    LAUNCH(s, k_jtprod, nn, nn, b.posptr, b.pcon, b.pval, yv, out);
  }
}

bool is_nt(const S* s) { return s->comp.direction == MSDP_NT; }
bool is_madnlp(const S* s) { return s->comp.schur == MSDP_MADNLP_SCHUR; }

// E(M): NT  W M W,  HKM  sym(X M S^-1)  (src/directions.jl:80-84,116-120)
void apply_E(S* s, Blk& b, const double* M, double* out) {
  const int n = b.n;
  if (is_nt(s)) {
    gemm(s, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, 1.0, b.W, n, M, n, 0.0, b.T3, n);
    gemm(s, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, 1.0, b.T3, n, b.W, n, 0.0, out, n);
  } else {
    gemm(s, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, 1.0, b.X, n, M, n, 0.0, b.T3, n);
    gemm(s, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, 1.0, b.T3, n, b.Si, n, 0.0, out, n);
  }
  LAUNCH(s, k_sym, (int64_t)n * n, n, out);
}

// ---- residuals and termination (src/step.jl:12-47, src/primal_dual.jl:123-134)
bool update_residuals(S* s) {
  reset_slots(s);
  const int m = s->m, ns = s->ns;
  if (m) CU(s, cudaMemsetAsync(s->acc, 0, sizeof(double) * m, s->st));
  for (auto& b : s->B) jprod(s, b, b.X, s->acc, true);
  if (ns && m) LAUNCH(s, k_gemv_n, m, m, ns, s->Clin, (int64_t)m, s->x, s->acc, 1);
  if (m) LAUNCH(s, k_lin, m, m, s->Rp, 1.0, s->b, -1.0, s->acc, 0.0, nullptr, 0.0, nullptr, 0.0, nullptr);
  std::vector<int> rmax(s->nb);
  for (int i = 0; i < s->nb; ++i) {
    Blk& b = s->B[i];
    const int64_t nn = (int64_t)b.n * b.n;
    jtprod(s, b, s->y, b.T1);
    LAUNCH(s, k_lin, nn, nn, b.Rd, 1.0, b.C, -1.0, b.S, -1.0, b.T1, 0.0, nullptr, 0.0, nullptr);
    rmax[i] = reduce(s, RED_MAXABS, nn, b.Rd);
  }
  if (ns) {
    if (m) {
      k_gemv_t<<<std::min(ns, 152 * 16), kThreads, 0, s->st>>>(m, ns, s->Clin, m, s->y, s->ctv, 0);
      s->launches += 1;
    } else {
      CU(s, cudaMemsetAsync(s->ctv, 0, sizeof(double) * ns, s->st));
    }
    LAUNCH(s, k_lin, ns, ns, s->Rdlin, 1.0, s->dlin, -1.0, s->z, -1.0, s->ctv, 0.0, nullptr, 0.0, nullptr);
  }
  if (!fetch(s)) return false;
  for (int i = 0; i < s->nb; ++i)
    s->B[i].rd_nonzero = s->hslots[rmax[i]] > 100.0 * kEps * std::max(1.0, s->B[i].cnorm);
  return true;
}

int nu(const S* s) {
  int v = s->ns;
  for (const auto& b : s->B) v += b.n;
  return v;
}

bool total_complementarity(S* s, double* out) {
  reset_slots(s);
  std::vector<int> sl;
  for (auto& b : s->B) sl.push_back(reduce(s, RED_DOT, (int64_t)b.n * b.n, b.X, b.S));
  const int lin = s->ns ? reduce(s, RED_DOT, s->ns, s->x, s->z) : -1;
  if (!fetch(s)) return false;
  double v = 0.0;
  for (int k : sl) v += s->hslots[k];
  if (lin >= 0) v += s->hslots[lin];
  *out = v;
  return true;
}

bool update_termination(S* s) {
  reset_slots(s);
  std::vector<int> cx, rd;
  for (auto& b : s->B) {
    cx.push_back(reduce(s, RED_DOT, (int64_t)b.n * b.n, b.C, b.X));
    rd.push_back(reduce(s, RED_MAXABS, (int64_t)b.n * b.n, b.Rd));
  }
  const int dx = s->ns ? reduce(s, RED_DOT, s->ns, s->dlin, s->x) : -1;
  const int rdl = s->ns ? reduce(s, RED_MAXABS, s->ns, s->Rdlin) : -1;
  const int by = reduce(s, RED_DOT, s->m, s->b, s->y);
  const int rp = reduce(s, RED_MAXABS, s->m, s->Rp);
  if (!fetch(s)) return false;
  double pobj = 0.0;
  for (int k : cx) pobj += s->hslots[k];
  if (dx >= 0) pobj += s->hslots[dx];
  const double dobj = s->hslots[by];
  s->pobj = pobj;
  s->dobj = dobj;
  s->inf_pr = s->hslots[rp] / std::max(1.0, s->bnorm);
  double r = 0.0, cn = s->cmax;
  for (int k : rd) r = std::max(r, s->hslots[k]);
  if (s->ns) {
    r = std::max(r, s->hslots[rdl]);
    cn = std::max(cn, s->dnorm);
  }
  s->inf_du = r / std::max(1.0, cn);
  s->gap = std::fabs(pobj - dobj) / std::max(1.0, std::fabs(pobj) + std::fabs(dobj));
  const bool converged = std::max(std::max(s->inf_pr, s->inf_du), s->gap) <= s->opt.tol;
  if (converged) s->status = MSDP_SOLVE_SUCCEEDED;
  else if (s->iter >= s->opt.max_iter) s->status = MSDP_MAXIMUM_ITERATIONS_EXCEEDED;
  else if (now_s() - s->t0 >= s->opt.max_wall_time) s->status = MSDP_MAXIMUM_WALLTIME_EXCEEDED;
  if (s->status == MSDP_REGULAR && s->mu < s->opt.mu_min) s->status = MSDP_SEARCH_DIRECTION_BECOMES_TOO_SMALL;
  msdp_iter_record rec{};
  rec.iter = s->iter; rec.pobj = pobj; rec.dobj = dobj; rec.inf_pr = s->inf_pr; rec.inf_du = s->inf_du;
  rec.gap = s->gap; rec.mu = s->mu; rec.alpha = s->alpha; rec.beta = s->beta; rec.phase = 1.0;
  s->traj.push_back(rec);
  return true;
}

// ---- NT eigendecomposition N = V diag(lam) V' (src/directions.jl:52-58)
// Orders where cuSOLVER's FP32 eigensolver plus the refinement beat its
// FP64 one on GB300 (measured: n = 100: 4.5 ms FP64 against 2.1 ms FP32;
// n = 2000: 100 ms against 25 ms; n = 400: no gain).
bool eig_refinable(int n) { return n >= 8 && (n <= 256 || n >= 600); }
constexpr int kEigRefineMax = 8;
// first-order corrections up to this size are taken; larger ones make
// clusters.  cuSOLVER's FP32 eigenvectors at n = 2000 are orthogonal only
// to about 2e-6 (measured on GB300; LAPACK's to 8e-9), and 1e-3 made
// clusters of 70-210 vectors on max-cut iterates where 3e-2 makes at most 8
// and converges in 4-5 steps.
constexpr double kEigCouple = 3e-2;

// FP32 eigenvectors (cuSOLVER's FP32 eigensolver on the shifted N; a
// one-block FP32 Jacobi start measured slower at n = 100) refined to FP64
// accuracy (eigref.h: Ogita-Aishima steps
// with exact rotations inside clusters of close eigenvalues), every product
// an FP64-accurate tensor-core product.  In: N's lower triangle in b.T2.
// Out: V in b.T2, lam in b.lam (Rayleigh quotients, not sorted).  Returns
// false when it did not converge or the FP32 solver failed; b.T2 then holds
// N's lower triangle again.  The refinement works on N shifted by its mean
// eigenvalue.  Scratch: b.G (N), b.W (shifted N, full), b.Gs, b.Si, b.Hx,
// b.Gi, b.T3.
bool nt_eig_refined(S* s, Blk& b) {
  const int n = b.n;
  const int64_t nn = (int64_t)n * n;
  CU(s, cudaMemcpyAsync(b.G, b.T2, sizeof(double) * nn, cudaMemcpyDeviceToDevice, s->st));  // N, for a fallback
  CU(s, cudaMemcpyAsync(b.W, b.T2, sizeof(double) * nn, cudaMemcpyDeviceToDevice, s->st));
  LAUNCH(s, k_lower_to_full, nn, n, b.W);
  // W = N - (trace N / n) I: same eigenvectors, eigenvalues shifted by the mean
  const int tr = reduce(s, RED_SUM, n, b.W, nullptr, (int64_t)n + 1);
  CU(s, eigref::shift_diag(n, b.W, s->slots + tr, -1.0 / n, s->st));
  const int ke = next_info(s);
  CU(s, eigref::to_float(nn, b.W, s->ef32, s->st));
  CS(s, cusolverDnSsyevd(s->cs, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, s->ef32, n, s->ef32 + nn,
                         s->ework32, s->elwork32, s->dinfo + ke));
  CU(s, eigref::to_double(nn, s->ef32, b.T2, s->st));
  s->launches += 3;
  bool conv = false, ok = true;
  for (int it = 0; it < kEigRefineMax && ok && !conv; ++it) {
    gemm(s, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, 1.0, b.W, n, b.T2, n, 0.0, b.Gs, n);   // N V
    gemm(s, CUBLAS_OP_T, CUBLAS_OP_N, n, n, n, 1.0, b.T2, n, b.Gs, n, 0.0, b.Si, n);  // S = V'NV
    syrk(s, true, n, n, 1.0, b.T2, n, 0.0, b.Hx, n);                                  // R = V'V
    // three consecutive slots for the residual measures of V
    const int se = next_slot(s);
    next_slot(s);
    next_slot(s);
    const int kf = next_info(s);
    CU(s, cudaMemsetAsync(s->dinfo + kf, 0, sizeof(int), s->st));
    CU(s, eigref::step(n, b.Si, b.Hx, kEigCouple, b.lam, b.Gi, s->eibuf, (unsigned long long*)(s->slots + se),
                       s->dinfo + kf, s->st, &s->launches));
    gemm(s, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, 1.0, b.T2, n, b.Gi, n, 0.0, b.T3, n);  // V (I + E)
    CU(s, cudaMemcpyAsync(b.T2, b.T3, sizeof(double) * nn, cudaMemcpyDeviceToDevice, s->st));
    s->eig_steps += 1;
    if (!fetch(s)) return false;
    ok = s->hinfo[ke] == 0 && s->hinfo[kf] == 0 && se + 2 < kSlots;
    // the basis this step started from was accurate to 1e-12 (off-diagonal
    // residual relative to max |lam|, and orthogonality): after the step
    // what remains is second order
    const double lmax = s->hslots[se + 2];
    const double off = lmax > 0.0 ? s->hslots[se] / lmax : (s->hslots[se] == 0.0 ? 0.0 : INFINITY);
    const double res = std::max(off, s->hslots[se + 1]);
    conv = ok && res <= 1e-12;
  }
  if (!conv) {
    CU(s, cudaMemcpyAsync(b.T2, b.G, sizeof(double) * nn, cudaMemcpyDeviceToDevice, s->st));
    return false;
  }
  CU(s, eigref::shift_vec(n, b.lam, s->slots + tr, 1.0 / n, s->st));  // eigenvalues of N
  s->launches += 3;
  return true;
}

// ---- prepare (src/primal_dual.jl:29-37, src/directions.jl:45-75, src/blocks.jl:94-130)
bool prepare(S* s, bool* ok) {
  reset_slots(s);
  const bool need_lx = is_nt(s) || s->comp.step == MSDP_EIGEN_STEP;
  std::vector<CholCheck> cs_, cx_;
  std::vector<int> lam0;
  for (auto& b : s->B) {
    const int n = b.n;
    const int64_t nn = (int64_t)n * n;
    cs_.push_back(chol_factor(s, n, b.S, b.Ls));
    if (!is_nt(s)) {
      // S^-1 from the factor (potri on a copy, lower to full); NT forms it
      // from the scaling below
      CU(s, cudaMemcpyAsync(b.Si, b.Ls, sizeof(double) * nn, cudaMemcpyDeviceToDevice, s->st));
      const int k = next_info(s);
      CS(s, cusolverDnDpotri(s->cs, CUBLAS_FILL_MODE_LOWER, n, b.Si, n, s->work, s->lwork, s->dinfo + k));
      LAUNCH(s, k_lower_to_full, nn, n, b.Si);
    }
    if (need_lx) cx_.push_back(chol_factor(s, n, b.X, b.Lx));
    if (is_nt(s)) {
      // M = Ls' Lx ; N = M'M ; eig(N) = V diag(lam) V'
      gemm(s, CUBLAS_OP_T, CUBLAS_OP_N, n, n, n, 1.0, b.Ls, n, b.Lx, n, 0.0, b.T1, n);
      syrk(s, true, n, n, 1.0, b.T1, n, 0.0, b.T2, n);
      if (s->ef32 && eig_refinable(n) && nt_eig_refined(s, b)) {
        s->eig_refined += 1;
      } else {
        const int ke = next_info(s);
        CS(s, cusolverDnDsyevd(s->cs, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, b.T2, n, b.lam, s->work,
                               s->lwork, s->dinfo + ke));
        s->eig_dense += 1;
      }
      lam0.push_back(reduce(s, RED_MIN, n, b.lam));
      LAUNCH(s, k_nt_scaling, n, n, b.lam, b.D, b.sc);
      // G = Lx V D^-1/2 and W = G G'.  From M V = U D (U orthogonal):
      // Gi = G^-1 = D^-3/2 (M V)' Ls' (no triangular solve) and
      // S^-1 = G D^-1 G' = Gs Gs' with Gs = G D^-1/2
      gemm(s, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, 1.0, b.Lx, n, b.T2, n, 0.0, b.G, n);
      LAUNCH(s, k_div_cols, nn, n, b.G, b.sc);
      gemm(s, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, 1.0, b.T1, n, b.T2, n, 0.0, b.T3, n);   // M V
      gemm(s, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, 1.0, b.Ls, n, b.T3, n, 0.0, b.T1, n);   // Ls M V
      LAUNCH(s, k_gi_scale, n, n, b.D, b.sc, b.gif);
      LAUNCH(s, k_scaled_transpose, nn, n, b.T1, b.gif, b.Gi);
      syrk(s, false, n, n, 1.0, b.G, n, 0.0, b.W, n);
      LAUNCH(s, k_lower_to_full, nn, n, b.W);
      CU(s, cudaMemcpyAsync(b.Gs, b.G, sizeof(double) * nn, cudaMemcpyDeviceToDevice, s->st));
      LAUNCH(s, k_div_cols, nn, n, b.Gs, b.sc);
      syrk(s, false, n, n, 1.0, b.Gs, n, 0.0, b.Si, n);
      LAUNCH(s, k_lower_to_full, nn, n, b.Si);
      CU(s, cudaMemcpyAsync(b.Hx, b.Gi, sizeof(double) * nn, cudaMemcpyDeviceToDevice, s->st));
      LAUNCH(s, k_div_rows, nn, n, b.Hx, b.sc);
    }
  }
  if (s->ns) LAUNCH(s, k_inv, s->ns, s->ns, s->z, s->zinv);
  if (!fetch(s)) return false;
  *ok = true;
  for (size_t i = 0; i < cs_.size(); ++i) *ok = *ok && chol_ok(s, cs_[i]);
  for (size_t i = 0; i < cx_.size(); ++i) *ok = *ok && chol_ok(s, cx_[i]);
  for (int k : lam0) *ok = *ok && s->hslots[k] > 0.0;
  if (*ok) {
    // E(Rd) is fixed for the iteration: computed once for rhs and directions
    for (auto& b : s->B)
      if (b.rd_nonzero) apply_E(s, b, b.Rd, b.ERd);
  }
  return !s->fail;
}

// H = sum_i <A_ij, L_i A_ik R_i> + C_lin diag(x/z) C_lin' (lower triangle).
// Dense constraint blocks and the scalar block are products on the tensor
// cores (tcgemm.h), in the FP64 slicing or, for the mixed precision, the
// split-precision one; coordinate lists use the entry-pair kernel.
void schur_complement(S* s, double* H, tcg::Mode mode) {
  const int m = s->m;
  const int nsl = tcg::slices_of(mode), mi = mode == tcg::kMixed ? 1 : 0;
  CU(s, cudaMemsetAsync(H, 0, sizeof(double) * m * m, s->st));
  for (auto& b : s->B) {
    const int n = b.n;
    const double* L = is_nt(s) ? b.W : b.Si;
    const double* R = is_nt(s) ? b.W : b.X;
    const int64_t mn = (int64_t)m * n;
    if (b.lowrank) {
      // NT: Q = V'WV, H += sg sg' o Q o Q; HKM: H += sg sg' o (V'S^-1 V) o (V'XV)
      for (int side = 0; side < (is_nt(s) ? 1 : 2); ++side) {
        const double* Lm = side ? R : L;
        if (!tc_bind(s, &s->tA, s->tAm, n, n, nsl) || !tc_bind(s, &s->tL, s->tLm, m, n, nsl)) return;
        tc_slice(s, op_rows(Lm, n, true, n, n), &s->tA);
        tc_product(s, s->tA, b.vk[mi], mode, b.P, n, 1.0, 0.0, false);            // P = Lm V
        tc_slice(s, op_rows(b.P, n, true, m, n), &s->tL);                        // rows: columns of P
        tc_product(s, b.vk[mi], s->tL, mode, side ? s->Q2 : s->Q1, m, 1.0, 0.0, true);  // V' P (lower)
      }
      LAUNCH(s, k_lowrank_schur, (int64_t)m * m, m, s->Q1, is_nt(s) ? s->Q1 : s->Q2, b.sg, H);
    } else if (!b.dense) {
      LAUNCH(s, k_schur_pairs, (int64_t)m * (m + 1) / 2, m, b.conptr, b.erow, b.ecol, b.eval, n, L, R, H);
    } else if (is_nt(s)) {
      // P = [A_1; ...; A_m] G (rows (j, r)), then B_j = (A_j G)' G, then
      // H += svec(B)' svec(B) over K = n(n+1)/2 (off-diagonals x sqrt 2)
      if (!tc_bind(s, &s->tB, s->tBm, n, n, nsl) || !tc_bind(s, &s->tQ, s->tQm, mn, n, nsl)) return;
      tc_slice(s, op_rows(b.G, n, true, n, n), &s->tB);
      tc_product(s, b.stk[mi], s->tB, mode, s->Tb, mn, 1.0, 0.0, false);
      tcg::Source q;
      q.p = s->Tb; q.rows = mn; q.K = n; q.nr = n; q.bs = n; q.rs = mn; q.ks = 1;
      tc_slice(s, q, &s->tQ);
      tc_product(s, s->tQ, s->tB, mode, s->Bb, mn, 1.0, 0.0, false);
      const int64_t K = (int64_t)n * (n + 1) / 2;
      if (!tc_bind(s, &s->tS, s->tSm, m, K, nsl)) return;
      tcg::Source v;
      v.p = s->Bb; v.rows = m; v.K = K; v.nr = 1; v.bs = n; v.rs = 1; v.ks = mn; v.kmap = b.kmap;
      tc_slice(s, v, &s->tS);
      tc_product(s, s->tS, s->tS, mode, H, m, 1.0, 1.0, true);
    } else {
      // P_k = A_k X (rows (k, r)), T_k = S^-1 P_k (side by side), H_jk += <A_j, T_k>
      if (!tc_bind(s, &s->tB, s->tBm, n, n, nsl) || !tc_bind(s, &s->tA, s->tAm, n, n, nsl) ||
          !tc_bind(s, &s->tQ, s->tQm, mn, n, nsl))
        return;
      tc_slice(s, op_rows(b.X, n, true, n, n), &s->tB);
      tc_product(s, b.stk[mi], s->tB, mode, s->Tb, mn, 1.0, 0.0, false);
      tc_slice(s, op_rows(b.Si, n, true, n, n), &s->tA);  // S^-1 is symmetric: rows read contiguously
      tcg::Source q;
      q.p = s->Tb; q.rows = mn; q.K = n; q.nr = n; q.bs = n; q.rs = mn; q.ks = 1;
      tc_slice(s, q, &s->tQ);
      tc_product(s, s->tA, s->tQ, mode, s->Bb, n, 1.0, 0.0, false);
      const int64_t nn = (int64_t)n * n;
      if (!tc_bind(s, &s->tS, s->tSm, m, nn, nsl)) return;
      tcg::Source t;
      t.p = s->Bb; t.rows = m; t.K = nn; t.nr = 1; t.bs = nn; t.rs = 0; t.ks = 1;
      tc_slice(s, t, &s->tS);
      tc_product(s, b.vec[mi], s->tS, mode, H, m, 1.0, 1.0, true);
    }
  }
  if (s->ns && m) {
    LAUNCH(s, k_mul, s->ns, s->ns, s->x, s->zinv, s->wlin);
    LAUNCH(s, k_scale_cols, (int64_t)m * s->ns, m, s->ns, s->Clin, s->wlin, s->Cw);
    if (!tc_bind(s, &s->tCw, s->tCwm, m, s->ns, nsl)) return;
    tc_slice(s, op_rows(s->Cw, m, false, m, s->ns), &s->tCw);
    tc_product(s, s->tCl[mi], s->tCw, mode, H, m, 1.0, 1.0, true);
  }
}

// Regularization retry loop (src/solver.jl:299-314, src/schur_solvers.jl:15-19).
// kMixed: split-precision assembly and an FP32-class factor (the solve is
// refined in FP64, solve_schur); when that factorization breaks down, the
// FP64 Schur matrix is used from then on.
bool factorize_schur(S* s, bool* ok, tcg::Mode mode) {
  const int m = s->m;
  *ok = false;
  if (m == 0) { *ok = true; return true; }
  mark(s, PH_ASSEMBLY);
  schur_complement(s, s->H0, mode);
  mark(s, PH_FACTOR);
  double reg = s->opt.regularize_schur;
  for (int t = 0; t < s->opt.max_schur_reg; ++t) {
    reset_slots(s);
    CU(s, cudaMemcpyAsync(s->H, s->H0, sizeof(double) * m * m, cudaMemcpyDeviceToDevice, s->st));
    if (reg > 0) LAUNCH(s, k_add_diag, m, m, s->H, (int64_t)m, reg);
    const int nf = reduce(s, RED_NONFINITE, (int64_t)m * m, s->H);
    const int k = next_info(s);
    if (is_madnlp(s)) {
      // MadNLPSchur (src/schur_solvers.jl:23-39, src/kkt.jl:7-32): Bunch-Kaufman
      // LDL' of the lower triangle; fails on an exactly singular pivot
      CS(s, cusolverDnDsytrf(s->cs, CUBLAS_FILL_MODE_LOWER, m, s->H, m, s->ipiv, s->sywork, s->sylwork,
                             s->dinfo + k));
      LAUNCH(s, k_ipiv64, m, m, s->ipiv, s->ipiv64);
    } else {
      note(s, chol::potrf(s->cwH, m, s->H, m, s->hinfo_dev, mode, s->st, &s->launches) == cudaSuccess,
           "chol::potrf");
      CU(s, cudaMemcpyAsync(s->dinfo + k, s->hinfo_dev, sizeof(int), cudaMemcpyDeviceToDevice, s->st));
    }
    if (!fetch(s)) return false;
    if (s->hinfo[k] == 0 && s->hslots[nf] == 0.0) {
      s->reg_used = reg;
      *ok = true;
      return true;
    }
    if (mode == tcg::kMixed) {
      s->mixed_on = false;
      s->ir_fallbacks += 1;
      return factorize_schur(s, ok, tcg::kFp64);
    }
    reg = reg == 0.0 ? 1e-12 : 10.0 * reg;
  }
  return true;
}
bool factorize_schur(S* s, bool* ok) { return factorize_schur(s, ok, s->mixed_on ? tcg::kMixed : tcg::kFp64); }

// out = L^-T L^-1 v with the Cholesky factor in H (chol.h)
void chol_solve(S* s, const double* v, double* out) {
  const int m = s->m;
  if (out != v) CU(s, cudaMemcpyAsync(out, v, sizeof(double) * m, cudaMemcpyDeviceToDevice, s->st));
  if (is_madnlp(s)) {
    CS(s, cusolverDnXsytrs(s->cs, CUBLAS_FILL_MODE_LOWER, m, 1, CUDA_R_64F, s->H, m, s->ipiv64, CUDA_R_64F, out, m,
                           s->sytrs_dev, s->sytrs_dev_bytes, s->sytrs_host.empty() ? nullptr : s->sytrs_host.data(),
                           s->sytrs_host.size(), s->hinfo_dev));
    return;
  }
  note(s, chol::solve(s->cwH, m, s->H, m, out, s->hinfo_dev, s->st, &s->launches) == cudaSuccess, "chol::solve");
}

// out = (H + reg I) v in FP64 without forming H: sum over blocks of
// A(E(A*(v))) plus C_lin diag(x/z) C_lin' v (the definition of the Schur
// complement, src/solver.jl:30-31,117-118; NT, where H is symmetric).
// The blocks' T1/T2 temporaries are free between the rhs and the directions.
void schur_apply(S* s, const double* v, double* out) {
  const int m = s->m, ns = s->ns;
  CU(s, cudaMemsetAsync(out, 0, sizeof(double) * m, s->st));
  for (auto& b : s->B) {
    jtprod(s, b, v, b.T1);
    apply_E(s, b, b.T1, b.T2);
    jprod(s, b, b.T2, out, true);
  }
  if (ns) {
    k_gemv_t<<<std::min(ns, 152 * 16), kThreads, 0, s->st>>>(m, ns, s->Clin, m, v, s->ctv, 0);
    s->launches += 1;
    LAUNCH(s, k_mul, ns, ns, s->ctv, s->wlin, s->vlin);
    LAUNCH(s, k_gemv_n, m, m, ns, s->Clin, (int64_t)m, s->vlin, out, 1);
  }
  if (s->reg_used > 0.0) LAUNCH(s, k_lin, m, m, out, 1.0, out, s->reg_used, v, 0.0, nullptr, 0.0, nullptr, 0.0, nullptr);
}

constexpr int kMaxRefine = 10;

// dy = (H + reg I)^-1 h.  FP64: two triangular solves with the factor.
// Mixed: the FP32-class factor's solution refined with FP64 residuals
// h - (H + reg I) dy of the matrix-free operator until the residual is
// below 1e-12 |h| or stops halving; if it then exceeds 1e-11 |h|, the Schur
// matrix is assembled
// and factored in FP64 for this and every later iteration.
bool solve_schur(S* s, bool* ok) {
  const int m = s->m;
  *ok = true;
  chol_solve(s, s->h, s->dy);
  if (!s->mixed_on) return !s->fail;
  CU(s, cudaMemcpyAsync(s->ir_h, s->h, sizeof(double) * m, cudaMemcpyDeviceToDevice, s->st));
  reset_slots(s);
  const int hs = reduce(s, RED_MAXABS, m, s->ir_h);
  if (!fetch(s)) return false;
  const double hn = std::max(s->hslots[hs], 1e-300);
  double prev = INFINITY, rn = INFINITY;
  int it = 0;
  for (; it < kMaxRefine; ++it) {
    schur_apply(s, s->dy, s->ir_r);
    LAUNCH(s, k_lin, m, m, s->ir_r, 1.0, s->ir_h, -1.0, s->ir_r, 0.0, nullptr, 0.0, nullptr, 0.0, nullptr);
    reset_slots(s);
    const int rs = reduce(s, RED_MAXABS, m, s->ir_r);
    if (!fetch(s)) return false;
    rn = s->hslots[rs];
    if (!(rn <= 1e-12 * hn) && rn < 0.5 * prev) {
      prev = rn;
      chol_solve(s, s->ir_r, s->ir_d);
      LAUNCH(s, k_lin, m, m, s->dy, 1.0, s->dy, 1.0, s->ir_d, 0.0, nullptr, 0.0, nullptr, 0.0, nullptr);
      continue;
    }
    break;
  }
  s->ir_steps += it;
  if (std::isfinite(rn) && rn <= 1e-11 * hn) return true;
  // refinement stalled: FP64 Schur matrix from now on
  s->mixed_on = false;
  s->ir_fallbacks += 1;
  bool f = false;
  if (!factorize_schur(s, &f, tcg::kFp64)) return false;
  if (!f) {
    *ok = false;
    return true;
  }
  chol_solve(s, s->ir_h, s->dy);
  CU(s, cudaMemcpyAsync(s->h, s->ir_h, sizeof(double) * m, cudaMemcpyDeviceToDevice, s->st));
  return !s->fail;
}

// ---- directions (src/step.jl:63-124); false on a CUDA/library failure
bool solve_directions(S* s, double mu, bool corrected) {
  const int m = s->m, ns = s->ns;
  // rhs
  if (m) CU(s, cudaMemcpyAsync(s->h, s->Rp, sizeof(double) * m, cudaMemcpyDeviceToDevice, s->st));
  for (auto& b : s->B) {
    const int64_t nn = (int64_t)b.n * b.n;
    LAUNCH(s, k_lin, nn, nn, b.T1, 1.0, b.X, -mu, b.Si, 1.0, b.rd_nonzero ? b.ERd : nullptr, -1.0,
           corrected ? b.corr : nullptr, 0.0, nullptr);
    jprod(s, b, b.T1, s->h, true);
  }
  if (ns && m) {
    LAUNCH(s, k_rhs_lin, ns, ns, mu, s->x, s->zinv, s->Rdlin, corrected ? s->corrlin : nullptr, s->vlin);
    LAUNCH(s, k_gemv_n, m, m, ns, s->Clin, (int64_t)m, s->vlin, s->h, 1);
  }
  // dely = H^-1 h
  if (m) {
    bool ok = true;
    if (!solve_schur(s, &ok)) return false;
    if (!ok) {
      s->status = MSDP_ERROR_IN_STEP_COMPUTATION;
      return true;
    }
  }
  // directions
  for (auto& b : s->B) {
    const int64_t nn = (int64_t)b.n * b.n;
    jtprod(s, b, s->dy, b.T1);
    LAUNCH(s, k_sym_diff, nn, b.n, b.Rd, b.T1, b.dS);
    apply_E(s, b, b.T1, b.T2);
    LAUNCH(s, k_lin, nn, nn, b.dX, mu, b.Si, -1.0, b.X, 1.0, b.T2, -1.0, b.rd_nonzero ? b.ERd : nullptr, 1.0,
           corrected ? b.corr : nullptr);
    LAUNCH(s, k_sym, nn, b.n, b.dX);
  }
  if (ns) {
    if (m) {
      k_gemv_t<<<std::min(ns, 152 * 16), kThreads, 0, s->st>>>(m, ns, s->Clin, m, s->dy, s->ctv, 0);
      s->launches += 1;
    } else {
      CU(s, cudaMemsetAsync(s->ctv, 0, sizeof(double) * ns, s->st));
    }
    LAUNCH(s, k_dir_lin, ns, ns, mu, s->Rdlin, s->ctv, s->x, s->zinv, corrected ? s->corrlin : nullptr, s->dz, s->dx);
  }
  return !s->fail;
}

// ---- Mehrotra correction (src/step.jl:128-136, src/directions.jl:90-100,123-127)
void correction(S* s) {
  for (auto& b : s->B) {
    const int n = b.n;
    const int64_t nn = (int64_t)n * n;
    if (is_nt(s)) {
      gemm(s, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, 1.0, b.Gi, n, b.dX, n, 0.0, b.T1, n);
      gemm(s, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, 1.0, b.T1, n, b.dS, n, 0.0, b.T2, n);
      gemm(s, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, 1.0, b.T2, n, b.G, n, 0.0, b.T1, n);
      LAUNCH(s, k_rnt, nn, n, b.T1, b.D, b.T2);
      gemm(s, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, 1.0, b.G, n, b.T2, n, 0.0, b.T1, n);
      gemm(s, CUBLAS_OP_N, CUBLAS_OP_T, n, n, n, 1.0, b.T1, n, b.G, n, 0.0, b.corr, n);
    } else {
      gemm(s, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, 1.0, b.dX, n, b.dS, n, 0.0, b.T1, n);
      gemm(s, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, -1.0, b.T1, n, b.Si, n, 0.0, b.corr, n);
    }
    LAUNCH(s, k_sym, nn, n, b.corr);
  }
  if (s->ns) LAUNCH(s, k_corr_lin, s->ns, s->ns, s->dx, s->dz, s->zinv, s->corrlin);
}

// ---- Lanczos for lambda_min of a formed symmetric Z (blocks above
// kLanczosWarpMax, 256).  Full reorthogonalization (twice); the step's scalars
// stay on the device and the host reads them every kLanczosBatch steps to
// apply the stopping rule at each step in order: the smallest Ritz value of
// the first step whose Ritz residual |beta_k s_k| is below 1e-12 ||Z||, or
// of step n.  Gives up at kLanczosMax (the caller then uses the dense
// eigensolver).
constexpr int kLanczosMin = 257;
constexpr int kLanczosMax = 320;
constexpr int kLanczosBatch = 8;
constexpr int kLanczosWarpMax = kLanczosCta;  // batched one-block device Lanczos up to this size

bool lanczos_eigmin(S* s, int n, const double* Z, double* out) {
  double* Q = s->lq;
  // fixed pseudo-random start vector (xorshift), normalized
  std::vector<double> q0(n);
  uint64_t st = 0x9E3779B97F4A7C15ull ^ (uint64_t)n;
  double nrm = 0.0;
  for (int i = 0; i < n; ++i) {
    st ^= st << 13; st ^= st >> 7; st ^= st << 17;
    q0[i] = (double)(st >> 11) * (1.0 / 9007199254740992.0) - 0.5;
    nrm += q0[i] * q0[i];
  }
  nrm = std::sqrt(nrm);
  for (auto& v : q0) v /= nrm;
  CU(s, cudaMemcpyAsync(Q, q0.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s->st));
  std::vector<double> al, be;
  std::vector<int> aslot, bslot;
  const int kmax = std::min(n, kLanczosMax);
  const int ga = std::min(n, 152 * 16);
  for (int k0 = 0; k0 < kmax; k0 += kLanczosBatch) {
    const int k1 = std::min(kmax, k0 + kLanczosBatch);
    for (int k = k0; k < k1; ++k) {
      const double* q = Q + (int64_t)k * n;
      double* w = Q + (int64_t)(k + 1) * n;
      // seven launches per step: matvec with the a partials, update (sums
      // them), two reorthogonalization passes (the second leaving the w'w
      // partials), normalization (sums those)
      double* pa_part = s->lzp;
      double* pb_part = s->lzp + ga;
      const int gsub = (n + 31) / 32;
      const int sa = next_slot(s);
      const int sb = next_slot(s);
      aslot.push_back(sa);
      k_lz_matvec<<<ga, kThreads, 0, s->st>>>((int64_t)n, Z, q, w, pa_part);
      k_lz_update<<<grid_for(n), kThreads, 0, s->st>>>((int64_t)n, w, q, k ? Q + (int64_t)(k - 1) * n : nullptr,
                                                        pa_part, ga, s->slots + sa,
                                                        k ? s->slots + bslot.back() : s->slots + sa);
      for (int r = 0; r < 2; ++r) {
        k_gemv_t<<<std::min(k + 1, 152 * 16), kThreads, 0, s->st>>>(n, k + 1, Q, n, w, s->lh, 0);
        if (r == 0)
          k_gemv_sub<<<gsub, 1024, 0, s->st>>>((int64_t)n, k + 1, Q, (int64_t)n, s->lh, w);
        else
          k_gemv_sub_dot<<<gsub, 1024, 0, s->st>>>((int64_t)n, k + 1, Q, (int64_t)n, s->lh, w, pb_part);
      }
      bslot.push_back(sb);
      k_lz_normalize<<<grid_for(n), kThreads, 0, s->st>>>((int64_t)n, w, pb_part, gsub, s->slots + sb, w);
      s->launches += 7;
      CU(s, cudaGetLastError());
    }
    if (!fetch(s)) return false;
    s->lanczos_steps += k1 - k0;
    for (int k = k0; k < k1; ++k) {
      al.push_back(s->hslots[aslot[k]]);
      const double beta = std::sqrt(std::max(s->hslots[bslot[k]], 0.0));
      double znorm = 0.0;
      const double theta = tridiag_min(al, be, k + 1, &znorm);
      if (k + 1 == n || beta <= 1e-300) { *out = theta; return true; }
      const double resid = beta * tridiag_last_component(al, be, k + 1, theta, znorm);
      if (resid <= 1e-12 * std::max(znorm, 1e-300)) { *out = theta; return true; }
      be.push_back(beta);
    }
  }
  return false;
}

// ---- step lengths (src/step.jl:148-228)
// slot of lambda_min(L^-1 D L^-T) (src/step.jl:150-163)
// Z = sym(L^-1 D L^-T) into Z (src/step.jl:150-163)
void form_congruence(S* s, int n, const double* L, const double* D, double* Z) {
  const double one = 1.0;
  CU(s, cudaMemcpyAsync(Z, D, sizeof(double) * n * n, cudaMemcpyDeviceToDevice, s->st));
  CB(s, cublasDtrsm(s->cb, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, n, n, &one, L, n,
                    Z, n));
  CB(s, cublasDtrsm(s->cb, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, CUBLAS_DIAG_NON_UNIT, n, n, &one, L,
                    n, Z, n));
  LAUNCH(s, k_sym, (int64_t)n * n, n, Z);
}

// slot of lambda_min(Z) for n > kLanczosWarpMax: host-driven Lanczos from
// kLanczosMin on, else (or when it does not converge) the dense eigensolver
int eigmin_large(S* s, Blk& b, double* Z) {
  const int n = b.n;
  if (n >= kLanczosMin) {
    double lam = 0.0;
    s->lanczos_calls += 1;
    if (lanczos_eigmin(s, n, Z, &lam)) {
      const int slot = next_slot(s);
      k_put_scalar<<<1, 1, 0, s->st>>>(s->slots + slot, lam);
      s->launches += 1;
      return slot;
    }
  }
  const int k = next_info(s);
  CS(s, cusolverDnDsyevd(s->cs, CUSOLVER_EIG_MODE_NOVECTOR, CUBLAS_FILL_MODE_LOWER, n, Z, n, b.w, s->work, s->lwork,
                         s->dinfo + k));
  s->eigmin_dense += 1;
  return copy_slot(s, b.w);
}

double eigen_step(double lam, double tau) { return lam > -std::sqrt(kEps) ? 1.0 : std::min(1.0, -tau / lam); }



// CholeskyBacktrack (src/step.jl:202-221)
bool backtrack(S* s, bool primal, double* out) {
  double a = 1.0;
  const double shrink = s->comp.shrink, boundary = s->comp.boundary;
  for (auto& b : s->B) {
    const int64_t nn = (int64_t)b.n * b.n;
    const double* Xv = primal ? b.X : b.S;
    const double* dXv = primal ? b.dX : b.dS;
    for (;;) {
      reset_slots(s);
      LAUNCH(s, k_lin, nn, nn, b.T1, 1.0, Xv, a, dXv, 0.0, nullptr, 0.0, nullptr, 0.0, nullptr);
      const int nf = reduce(s, RED_NONFINITE, nn, b.T1);
      const int k = potrf(s, b.n, b.T1, b.n);
      if (!fetch(s)) return false;
      if (s->hinfo[k] == 0 && s->hslots[nf] == 0.0) break;
      a *= shrink;
      if (a < kEps) { *out = 0.0; return true; }
    }
  }
  if (a != 1.0) a *= boundary;
  if (s->ns) {
    reset_slots(s);
    const int r = primal ? reduce(s, RED_MINRATIO, s->ns, s->x, s->dx) : reduce(s, RED_MINRATIO, s->ns, s->z, s->dz);
    if (!fetch(s)) return false;
    a = std::min(a, boundary * s->hslots[r]);
  }
  *out = a;
  return true;
}

bool step_lengths(S* s, double* a_out, double* b_out) {
  if (s->comp.step == MSDP_CHOLESKY_BACKTRACK)
    return backtrack(s, true, a_out) && backtrack(s, false, b_out);
  reset_slots(s);
  std::vector<int> lx, ls;
  std::vector<LanczosJob> jobs;
  int64_t qoff = 0, woff = 0;
  for (auto& b : s->B) {
    const int n = b.n;
    // Z_X ~ Lx^-1 dX Lx^-T in T1, Z_S ~ Ls^-1 dS Ls^-T in T2: NT by the
    // orthogonally similar Hx dX Hx' and Gs' dS Gs (products only)
    if (is_nt(s)) {
      gemm(s, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, 1.0, b.Hx, n, b.dX, n, 0.0, b.T3, n);
      gemm(s, CUBLAS_OP_N, CUBLAS_OP_T, n, n, n, 1.0, b.T3, n, b.Hx, n, 0.0, b.T1, n);
      LAUNCH(s, k_sym, (int64_t)n * n, n, b.T1);
      gemm(s, CUBLAS_OP_T, CUBLAS_OP_N, n, n, n, 1.0, b.Gs, n, b.dS, n, 0.0, b.T3, n);
      gemm(s, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, 1.0, b.T3, n, b.Gs, n, 0.0, b.T2, n);
      LAUNCH(s, k_sym, (int64_t)n * n, n, b.T2);
    } else {
      form_congruence(s, n, b.Lx, b.dX, b.T1);
      form_congruence(s, n, b.Ls, b.dS, b.T2);
    }
    if (n <= kLanczosWarpMax) {
      for (int side = 0; side < 2; ++side) {
        const int slot = next_slot(s);
        jobs.push_back(LanczosJob{n, side ? b.T2 : b.T1, s->lq2 + qoff, s->lw2 + woff, s->slots + slot});
        qoff += (int64_t)n * n;
        woff += 4 * (int64_t)(n + 1);
        (side ? ls : lx).push_back(slot);
      }
    } else {
      lx.push_back(eigmin_large(s, b, b.T1));
      ls.push_back(eigmin_large(s, b, b.T2));
    }
  }
  if (!jobs.empty()) {
    CU(s, cudaMemcpyAsync(s->ljobs, jobs.data(), sizeof(LanczosJob) * jobs.size(), cudaMemcpyHostToDevice, s->st));
    k_lanczos_cta<<<(unsigned)jobs.size(), kLanczosCta, 0, s->st>>>((const LanczosJob*)s->ljobs);
    s->launches += 1;
  }
  const int rx = s->ns ? reduce(s, RED_MINRATIO, s->ns, s->x, s->dx) : -1;
  const int rz = s->ns ? reduce(s, RED_MINRATIO, s->ns, s->z, s->dz) : -1;
  if (!fetch(s)) return false;
  double a = 1.0, bt = 1.0;
  const double tau = s->comp.tau;
  for (size_t i = 0; i < lx.size(); ++i) {
    a = std::min(a, eigen_step(s->hslots[lx[i]], tau));
    bt = std::min(bt, eigen_step(s->hslots[ls[i]], tau));
  }
  if (s->ns) {
    a = std::min(a, tau * s->hslots[rx]);
    bt = std::min(bt, tau * s->hslots[rz]);
  }
  *a_out = a;
  *b_out = bt;
  return true;
}

// src/step.jl:231-243
bool affine_complementarity(S* s, double a, double bt, double* out) {
  reset_slots(s);
  std::vector<int> sl;
  for (auto& b : s->B) {
    const int64_t nn = (int64_t)b.n * b.n;
    sl.push_back(reduce(s, RED_DOT, nn, b.X, b.S));
    sl.push_back(reduce(s, RED_DOT, nn, b.X, b.dS));
    sl.push_back(reduce(s, RED_DOT, nn, b.dX, b.S));
    sl.push_back(reduce(s, RED_DOT, nn, b.dX, b.dS));
  }
  int lin = -1;
  if (s->ns) {
    LAUNCH(s, k_aff_lin, s->ns, s->ns, a, bt, s->x, s->dx, s->z, s->dz, s->vlin);
    lin = reduce(s, RED_SUM, s->ns, s->vlin);
  }
  if (!fetch(s)) return false;
  double v = 0.0;
  for (size_t i = 0; i < sl.size(); i += 4) {
    v += s->hslots[sl[i]];
    v += bt * s->hslots[sl[i + 1]];
    v += a * s->hslots[sl[i + 2]];
    v += a * bt * s->hslots[sl[i + 3]];
  }
  if (lin >= 0) v += s->hslots[lin];
  *out = v / std::max(nu(s), 1);
  return true;
}

// src/primal_dual.jl:56-72
bool take_step(S* s, double a, double bt) {
  s->alpha = a;
  s->beta = bt;
  for (auto& b : s->B) {
    const int64_t nn = (int64_t)b.n * b.n;
    LAUNCH(s, k_lin, nn, nn, b.X, 1.0, b.X, a, b.dX, 0.0, nullptr, 0.0, nullptr, 0.0, nullptr);
    LAUNCH(s, k_lin, nn, nn, b.S, 1.0, b.S, bt, b.dS, 0.0, nullptr, 0.0, nullptr, 0.0, nullptr);
  }
  if (s->m) LAUNCH(s, k_lin, s->m, s->m, s->y, 1.0, s->y, bt, s->dy, 0.0, nullptr, 0.0, nullptr, 0.0, nullptr);
  if (s->ns) {
    LAUNCH(s, k_lin, s->ns, s->ns, s->x, 1.0, s->x, a, s->dx, 0.0, nullptr, 0.0, nullptr, 0.0, nullptr);
    LAUNCH(s, k_lin, s->ns, s->ns, s->z, 1.0, s->z, bt, s->dz, 0.0, nullptr, 0.0, nullptr, 0.0, nullptr);
  }
  s->iter += 1;
  return update_residuals(s);
}

bool start_iteration(S* s, bool* ok) {
  bool p = false, f = false;
  s->nev = 0;
  mark(s, PH_PREPARE);
  if (!prepare(s, &p)) return false;
  if (p && !factorize_schur(s, &f)) return false;
  *ok = p && f;
  if (!*ok) s->status = MSDP_ERROR_IN_STEP_COMPUTATION;
  return true;
}

// src/primal_dual.jl:85-101
bool iterate_mehrotra(S* s) {
  bool ok = false;
  if (!start_iteration(s, &ok)) return false;
  if (!ok) return true;
  double tc = 0.0;
  if (!total_complementarity(s, &tc)) return false;
  const double mu = tc / std::max(nu(s), 1);
  s->mu = mu;
  mark(s, PH_DIRECTIONS);
  if (!solve_directions(s, 0.0, false)) return false;
  if (s->status != MSDP_REGULAR) return true;
  double aa = 0, ba = 0, mua = 0;
  mark(s, PH_STEP);
  if (!step_lengths(s, &aa, &ba) || !affine_complementarity(s, aa, ba, &mua)) return false;
  const double sigma = std::min(std::max(std::pow(mua / std::max(mu, kEps), s->comp.sigma_exponent), 1e-8), 1.0);
  s->sigma = sigma;
  mark(s, PH_CORRECTION);
  correction(s);
  mark(s, PH_DIRECTIONS);
  if (!solve_directions(s, sigma * mu, true)) return false;
  if (s->status != MSDP_REGULAR) return true;
  double a = 0, bt = 0;
  mark(s, PH_STEP);
  if (!step_lengths(s, &a, &bt)) return false;
  mark(s, PH_STEP_UPDATE);
  const bool r = take_step(s, a, bt);
  (s->mixed_on ? s->n32 : s->n64) += 1;
  collect_marks(s);
  return r;
}

// src/primal_dual.jl:104-121
bool iterate_adaptive(S* s) {
  bool ok = false;
  if (!start_iteration(s, &ok)) return false;
  if (!ok) return true;
  if (!solve_directions(s, s->mu, false)) return false;
  if (s->status != MSDP_REGULAR) return true;
  double a = 0, bt = 0;
  if (!step_lengths(s, &a, &bt) || !take_step(s, a, bt)) return false;
  (s->mixed_on ? s->n32 : s->n64) += 1;
  double tc = 0.0;
  if (!total_complementarity(s, &tc)) return false;
  double mu = s->comp.ratio * tc / std::max(nu(s), 1);
  if (std::min(a, bt) < 0.5) mu *= 1.5;
  if (a + bt > 1.6) mu *= 0.75;
  if (a + bt > 1.9) mu /= 1.0 + 0.1 * s->iter;
  s->mu = mu;
  collect_marks(s);
  return true;
}

// S_i = sym(C_i - A_i*(y)), z = d_lin - C_lin'y (src/solver.jl:192-211)
void set_dual_slacks(S* s) {
  for (auto& b : s->B) {
    const int64_t nn = (int64_t)b.n * b.n;
    jtprod(s, b, s->y, b.T1);
    LAUNCH(s, k_lin, nn, nn, b.S, 1.0, b.C, -1.0, b.T1, 0.0, nullptr, 0.0, nullptr, 0.0, nullptr);
    LAUNCH(s, k_sym, nn, b.n, b.S);
  }
  if (s->ns) {
    if (s->m) {
      k_gemv_t<<<std::min(s->ns, 152 * 16), kThreads, 0, s->st>>>(s->m, s->ns, s->Clin, s->m, s->y, s->ctv, 0);
      s->launches += 1;
    } else {
      CU(s, cudaMemsetAsync(s->ctv, 0, sizeof(double) * s->ns, s->st));
    }
    LAUNCH(s, k_lin, s->ns, s->ns, s->z, 1.0, s->dlin, -1.0, s->ctv, 0.0, nullptr, 0.0, nullptr, 0.0, nullptr);
  }
}

// Initial points (src/solver.jl:213-284); returns MSDP_ERR_INITIAL_POINT
// when DualShift finds no interior point.
int initial_point(S* s) {
  const int ip = s->comp.initial_point;
  if (ip == MSDP_SCALED_IDENTITY) {
    double beta;
    if (s->comp.scale > 0.0) {
      beta = s->comp.scale;
    } else {
      double cs = s->cmax;
      if (s->ns) cs = std::max(cs, s->dnorm);
      beta = std::max(10.0, std::sqrt(std::max(s->bnorm, 1.0) * std::max(cs, 1.0)) * std::sqrt((double)nu(s)));
    }
    for (auto& b : s->B) {
      LAUNCH(s, k_identity, (int64_t)b.n * b.n, b.n, b.X, beta);
      LAUNCH(s, k_identity, (int64_t)b.n * b.n, b.n, b.S, beta);
    }
    if (s->m) CU(s, cudaMemsetAsync(s->y, 0, sizeof(double) * s->m, s->st));
    if (s->ns) {
      LAUNCH(s, k_fill, s->ns, s->ns, s->x, beta);
      LAUNCH(s, k_fill, s->ns, s->ns, s->z, beta);
    }
    return MSDP_OK;
  }
  if (ip == MSDP_INITIAL_POINT) {
    if (!s->has_ip) return MSDP_ERR_INVALID_ARGUMENT;
    if (s->m) CU(s, cudaMemcpyAsync(s->y, s->ipy.data(), 8 * s->m, cudaMemcpyHostToDevice, s->st));
    for (int i = 0; i < s->nb; ++i)
      CU(s, cudaMemcpyAsync(s->B[i].X, s->ipX[i].data(), 8 * s->ipX[i].size(), cudaMemcpyHostToDevice, s->st));
    if (s->ns) CU(s, cudaMemcpyAsync(s->x, s->ipx.data(), 8 * s->ns, cudaMemcpyHostToDevice, s->st));
    set_dual_slacks(s);
    CU(s, cudaStreamSynchronize(s->st));
    return MSDP_OK;
  }
  // DualShift
  for (auto& b : s->B) LAUNCH(s, k_identity, (int64_t)b.n * b.n, b.n, b.X, 1.0);
  if (s->ns) LAUNCH(s, k_fill, s->ns, s->ns, s->x, 1.0);
  double rho = 0.0;
  while (rho <= s->comp.max_shift) {
    if (s->m) LAUNCH(s, k_fill, s->m, s->m, s->y, -rho);
    set_dual_slacks(s);
    reset_slots(s);
    std::vector<CholCheck> cc;
    for (auto& b : s->B) cc.push_back(chol_factor(s, b.n, b.S, b.Ls));
    const int zmin = s->ns ? reduce(s, RED_MIN, s->ns, s->z) : -1;
    if (!fetch(s)) return s->fail;
    bool interior = true;
    for (auto& c : cc) interior = interior && chol_ok(s, c);
    if (s->ns) interior = interior && s->hslots[zmin] > 0.0;
    if (interior) {
      if (rho != 0.0) {
        if (s->m) LAUNCH(s, k_fill, s->m, s->m, s->y, -2.0 * rho);
        set_dual_slacks(s);
      }
      return MSDP_OK;
    }
    rho = rho == 0.0 ? s->comp.initial_shift : 2.0 * rho;
  }
  return MSDP_ERR_INITIAL_POINT;
}

int initialize(S* s) {
  const int rc = initial_point(s);
  if (rc) return rc;
  s->iter = 0;
  s->status = MSDP_REGULAR;
  s->alpha = s->beta = s->sigma = 0.0;
  s->traj.clear();
  s->t0 = now_s();
  if (!update_residuals(s)) return MSDP_ERR_CUDA;
  double tc = 0.0;
  if (!total_complementarity(s, &tc)) return MSDP_ERR_CUDA;
  const double mu = tc / std::max(nu(s), 1);
  s->mu = s->comp.centering == MSDP_ADAPTIVE_MU ? s->comp.initial_ratio * mu : mu;
  return MSDP_OK;
}

// Tensor-core workspaces, and the slices of the constant constraint data
// (dense blocks: [A_1; ...; A_m] rows, HKM also vec(A_j) rows; C_lin),
// made once; nonzero on failure.
int tc_setup(S* s, bool mixed) {
  const int m = s->m, ns = s->ns;
  int nmax = 1, nd = 0;
  for (auto& b : s->B) {
    nmax = std::max(nmax, b.n);
    if (b.dense) nd = std::max(nd, b.n);
  }
  auto tcalloc = [&](int64_t bytes) -> void* {
    void* p = nullptr;
    if (cudaMalloc(&p, (size_t)std::max<int64_t>(bytes, 256)) != cudaSuccess) return nullptr;
    s->allocs.push_back(p);
    s->bytes += bytes;
    return p;
  };
  s->tAm = tcalloc(tcg::sliced_bytes(nmax, nmax, 7));
  s->tBm = tcalloc(tcg::sliced_bytes(nmax, nmax, 7));
  int64_t fixn = std::max<int64_t>((int64_t)nmax * nmax, (int64_t)m * m);
  if (nd) {
    const int64_t mn = (int64_t)m * nd;
    s->tQm = tcalloc(tcg::sliced_bytes(mn, nd, 7));
    s->tSm = tcalloc(tcg::sliced_bytes(m, is_nt(s) ? (int64_t)nd * (nd + 1) / 2 : (int64_t)nd * nd, 7));
    if (!s->tQm || !s->tSm) return 1;
    fixn = std::max(fixn, mn * nd);  // split-K operands of the assembly's first two products
  }
  if (ns && m) {
    s->tCwm = tcalloc(tcg::sliced_bytes(m, ns, 7));
    if (!s->tCwm) return 1;
  }
  s->tfix = (long long*)tcalloc(8 * fixn);
  s->tfix_len = fixn;
  s->terr = (int*)tcalloc(sizeof(int));
  void* cwm = tcalloc(chol::work_bytes(nmax));
  void* cwh = tcalloc(chol::work_bytes(std::max(m, 1)));
  s->hinfo_dev = (int*)tcalloc(sizeof(int));
  if (!s->tAm || !s->tBm || !s->tfix || !s->terr || !cwm || !cwh || !s->hinfo_dev) return 1;
  CU(s, chol::init(&s->cw, cwm, nmax, s->terr, s->st));
  CU(s, chol::init(&s->cwH, cwh, std::max(m, 1), s->terr, s->st));
  CU(s, cudaMemsetAsync(s->hinfo_dev, 0, sizeof(int), s->st));
  CU(s, cudaMemsetAsync(s->terr, 0, sizeof(int), s->st));
  const int nmodes = mixed ? 2 : 1;
  for (auto& b : s->B) {
    if (!b.dense) continue;
    const int n = b.n;
    const int64_t mn = (int64_t)m * n, nn = (int64_t)n * n;
    for (int mi = 0; mi < nmodes; ++mi) {
      const int nsl = mi ? 3 : 7;
      void* mem = tcalloc(tcg::sliced_bytes(mn, n, nsl));
      if (!mem) return 1;
      CU(s, tcg::sliced_init(&b.stk[mi], mem, mn, n, nsl, s->st));
      // row (j, r), column k: A_j(r, k) = A_j(k, r) = Aall[j n^2 + k + r n]
      tcg::Source a;
      a.p = b.Aall; a.rows = mn; a.K = n; a.nr = n; a.bs = nn; a.rs = n; a.ks = 1;
      tc_slice(s, a, &b.stk[mi]);
      if (!is_nt(s)) {
        void* vm = tcalloc(tcg::sliced_bytes(m, nn, nsl));
        if (!vm) return 1;
        CU(s, tcg::sliced_init(&b.vec[mi], vm, m, nn, nsl, s->st));
        tcg::Source v;
        v.p = b.Aall; v.rows = m; v.K = nn; v.nr = 1; v.bs = nn; v.rs = 0; v.ks = 1;
        tc_slice(s, v, &b.vec[mi]);
      }
    }
    if (is_nt(s)) {
      // symmetric-vector order: column c, then rows r >= c
      std::vector<int2> km;
      km.reserve((size_t)(nn + n) / 2);
      for (int c = 0; c < n; ++c)
        for (int r = c; r < n; ++r) km.push_back(make_int2(r, c));
      b.kmap = (int2*)tcalloc((int64_t)sizeof(int2) * km.size());
      if (!b.kmap) return 1;
      CU(s, upload(s, b.kmap, km.data(), sizeof(int2) * km.size()));
    }
  }
  int64_t lr_bytes = 0;
  for (auto& b : s->B) {
    if (!b.lowrank) continue;
    const int n = b.n;
    lr_bytes = std::max(lr_bytes, std::max(tcg::sliced_bytes(n, m, 7), tcg::sliced_bytes(m, n, 7)));
    for (int mi = 0; mi < nmodes; ++mi) {
      const int nsl = mi ? 3 : 7;
      void* mem = tcalloc(tcg::sliced_bytes(m, n, nsl));
      if (!mem) return 1;
      CU(s, tcg::sliced_init(&b.vk[mi], mem, m, n, nsl, s->st));
      tc_slice(s, op_rows(b.V, n, true, m, n), &b.vk[mi]);  // row j = v_j
    }
    void* mem = tcalloc(tcg::sliced_bytes(n, m, 7));
    if (!mem) return 1;
    CU(s, tcg::sliced_init(&b.vr, mem, n, m, 7, s->st));
    tc_slice(s, op_rows(b.V, n, false, n, m), &b.vr);  // row r = (v_1r ... v_mr)
  }
  if (lr_bytes) {
    s->tLm = tcalloc(lr_bytes);
    if (!s->tLm) return 1;
  }
  if (ns && m) {
    for (int mi = 0; mi < nmodes; ++mi) {
      const int nsl = mi ? 3 : 7;
      void* mem = tcalloc(tcg::sliced_bytes(m, ns, nsl));
      if (!mem) return 1;
      CU(s, tcg::sliced_init(&s->tCl[mi], mem, m, ns, nsl, s->st));
      tc_slice(s, op_rows(s->Clin, m, false, m, ns), &s->tCl[mi]);
    }
  }
  CU(s, cudaStreamSynchronize(s->st));
  return s->fail ? 1 : 0;
}

// Every constraint of the block is sg_j v_j v_j' (or zero): fills V
// (n x m, column-major) and sg from the coordinate lists (v_j from the
// column of the largest diagonal entry); false when any entry differs from
// sg_j v_rj v_cj by more than 8 eps of the constraint's largest entry, or
// when an entry of the outer product is missing.
// f(lo, hi) over the chunks of [0, count) on the host's threads (at most 32;
// one when count is below `grain` per extra thread)
template <class F>
void host_parallel(int64_t count, F f, int64_t grain = (int64_t)1 << 20) {
  const int64_t hw = std::max<int64_t>(1, (int64_t)std::thread::hardware_concurrency());
  const int64_t T = std::max<int64_t>(1, std::min<int64_t>(std::min<int64_t>(hw, 32), count / std::max<int64_t>(grain, 1)));
  if (T <= 1) {
    f((int64_t)0, count);
    return;
  }
  std::vector<std::thread> pool;
  pool.reserve((size_t)T);
  for (int64_t t = 0; t < T; ++t) pool.emplace_back(f, count * t / T, count * (t + 1) / T);
  for (auto& th : pool) th.join();
}

// Whether the entries q in [e0, e1) (entry ord[q], or q without ord) of one
// constraint are s v v' (every entry within 8 eps of s v_r v_c and no entry
// of the outer product missing); v into w (length n) when w is given.
bool rank_one_group(int n, int64_t e0, int64_t e1, const int64_t* ord, const int32_t* row, const int32_t* col,
                    const double* val, double* w, double* sgn_out) {
  auto at = [&](int64_t q) { return ord ? ord[q] : q; };
  int p = -1;
  double dmax = 0.0, amax = 0.0;
  for (int64_t q = e0; q < e1; ++q) {
    const int64_t e = at(q);
    if (row[e] < 0 || row[e] >= n || col[e] < 0 || col[e] >= n) return false;
    amax = std::max(amax, std::fabs(val[e]));
    if (row[e] == col[e] && std::fabs(val[e]) > dmax) { dmax = std::fabs(val[e]); p = row[e]; }
  }
  if (p < 0 || !(dmax > 0.0) || !std::isfinite(amax)) return false;
  double dp = 0.0;
  for (int64_t q = e0; q < e1; ++q) {
    const int64_t e = at(q);
    if (row[e] == p && col[e] == p) dp = val[e];
  }
  const double scale = std::sqrt(std::fabs(dp)), sgn = dp > 0 ? 1.0 : -1.0;
  std::vector<double> v(n, 0.0);
  for (int64_t q = e0; q < e1; ++q) {
    const int64_t e = at(q);
    if (col[e] == p) v[row[e]] = val[e] / scale;
  }
  int64_t k = 0;
  for (double x : v) k += x != 0.0;
  if (e1 - e0 != k * k) return false;
  for (int64_t q = e0; q < e1; ++q) {
    const int64_t e = at(q);
    const double wr = v[row[e]], wc = v[col[e]];
    if (wr == 0.0 || wc == 0.0 || std::fabs(sgn * wr * wc - val[e]) > 8.0 * kEps * amax) return false;
  }
  if (w) std::copy(v.begin(), v.end(), w);
  if (sgn_out) *sgn_out = sgn;
  return true;
}

bool detect_rank_one(int n, int m, int64_t nnz, const int32_t* con, const int32_t* row, const int32_t* col,
                     const double* val, std::vector<double>* V, std::vector<double>* sg) {
  // cheap rejection first: the leading run of entries of one constraint
  // (grouped input) must itself be rank one, so dense or sparse general
  // constraints are turned down without a pass over all entries (input
  // whose constraints are not grouped may then miss the low-rank form and
  // take the general paths, which give the same results)
  if (nnz > 0 && con[0] >= 0 && con[0] < m) {
    int64_t e1 = 0;
    while (e1 < nnz && con[e1] == con[0]) ++e1;
    if (!rank_one_group(n, 0, e1, nullptr, row, col, val, nullptr, nullptr)) return false;
  }
  std::vector<int64_t> start(m + 2, 0);
  bool grouped = true;  // entries already in constraint order (the usual input): no permutation
  for (int64_t e = 0; e < nnz; ++e) {
    if (con[e] < 0 || con[e] >= m || row[e] < 0 || row[e] >= n || col[e] < 0 || col[e] >= n) return false;
    start[con[e] + 2] += 1;
    grouped = grouped && (e == 0 || con[e] >= con[e - 1]);
  }
  for (int j = 0; j < m; ++j) start[j + 2] += start[j + 1];
  std::vector<int64_t> ord;
  if (grouped) {
    for (int j = 0; j <= m; ++j) start[j] = start[j + 1];
  } else {
    ord.resize(nnz);
    for (int64_t e = 0; e < nnz; ++e) ord[start[con[e] + 1]++] = e;
  }
  V->assign((size_t)n * m, 0.0);
  sg->assign(m, 1.0);
  for (int j = 0; j < m; ++j) {
    const int64_t e0 = start[j], e1 = start[j + 1];
    if (e0 == e1) continue;
    double sgn = 1.0;
    if (!rank_one_group(n, e0, e1, grouped ? nullptr : ord.data(), row, col, val, V->data() + (int64_t)j * n, &sgn))
      return false;
    (*sg)[j] = sgn;
  }
  return true;
}

void release(S* s) {
  if (s->st) cudaStreamSynchronize(s->st);
  for (auto& e : s->ev)
    if (e) cudaEventDestroy(e);
  for (void* p : s->allocs) cudaFree(p);
  s->allocs.clear();
  if (s->hslots) cudaFreeHost(s->hslots);
  if (s->hinfo) cudaFreeHost(s->hinfo);
  if (s->cb) cublasDestroy(s->cb);
  if (s->cs) cusolverDnDestroy(s->cs);
}

}  // namespace

extern "C" {

int msdp_solver_create(msdp_context* ctx, const msdp_problem_desc* d, const msdp_components* comp,
                       const msdp_options* opt, msdp_solver** out) {
  if (!ctx || !d || !out) return MSDP_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  msdp_components c;
  msdp_options o;
  if (comp) c = *comp; else msdp_default_components(&c);
  if (opt) o = *opt; else msdp_default_options(&o);
  if (d->nblocks < 0 || d->m < 0 || d->ns < 0 || (d->nblocks == 0 && d->ns == 0)) return MSDP_ERR_INVALID_ARGUMENT;
  if (c.algorithm != MSDP_PRIMAL_DUAL || (c.schur != MSDP_DENSE_CHOLESKY && c.schur != MSDP_MADNLP_SCHUR) ||
      (c.precision != MSDP_FP64 && c.precision != MSDP_FP64_TENSOR && c.precision != MSDP_MIXED))
    return MSDP_ERR_UNSUPPORTED;
  // MadNLPSchur factors in FP64 only (no split-precision factor for it)
  if (c.schur == MSDP_MADNLP_SCHUR && c.precision == MSDP_MIXED) return MSDP_ERR_UNSUPPORTED;
  // mixed: the refinement applies H matrix-free, which equals the factored
  // lower-triangle matrix only when H is symmetric (NT)
  if (c.precision == MSDP_MIXED && c.direction != MSDP_NT) return MSDP_ERR_UNSUPPORTED;
  if (!(c.tau > 0.0) || !(c.shrink > 0.0 && c.shrink < 1.0) || !(c.boundary > 0.0 && c.boundary <= 1.0) ||
      o.max_iter < 0 || (c.initial_point == MSDP_DUAL_SHIFT && !(c.initial_shift > 0.0)))
    return MSDP_ERR_INVALID_ARGUMENT;
  auto s = new msdp_solver();
  s->ctx = ctx;
  s->st = (cudaStream_t)msdp_context_stream(ctx);
  s->comp = c;
  s->opt = o;
  s->m = d->m;
  s->ns = d->ns;
  s->nb = d->nblocks;
  const int m = d->m, ns = d->ns;
  auto bail = [&](int code) {
    release(s);
    delete s;
    return code;
  };
  if (cublasCreate(&s->cb) != CUBLAS_STATUS_SUCCESS || cusolverDnCreate(&s->cs) != CUSOLVER_STATUS_SUCCESS)
    return bail(MSDP_ERR_CUDA);
  cublasSetStream(s->cb, s->st);
  cusolverDnSetStream(s->cs, s->st);
  if (c.precision == MSDP_FP64_TENSOR) {
    // double-precision products by fixed-point emulation on tensor cores
    // (cuBLAS picks the mantissa width for FP64 accuracy)
    if (cublasSetMathMode(s->cb, CUBLAS_FP64_EMULATED_FIXEDPOINT_MATH) != CUBLAS_STATUS_SUCCESS ||
        cublasSetEmulationStrategy(s->cb, CUBLAS_EMULATION_STRATEGY_EAGER) != CUBLAS_STATUS_SUCCESS)
      return bail(MSDP_ERR_UNSUPPORTED);
  }
  for (auto& e : s->ev)
    if (cudaEventCreate(&e) != cudaSuccess) e = nullptr;
  // ---- host staging of the constraints
  s->B.resize(s->nb);
  double cmax = 0.0;
  int64_t dense_ws = 0;
  std::vector<std::vector<double>> lrV(s->nb), lrS(s->nb);
  bool any_lowrank = false;
  for (int i = 0; i < s->nb; ++i) {
    Blk& b = s->B[i];
    b.n = d->sides[i];
    b.nnz = d->A_nnz[i];
    if (b.n <= 0 || b.nnz < 0) return bail(MSDP_ERR_INVALID_ARGUMENT);
    const double n = b.n;
    const double pair_cost = (double)b.nnz * (double)b.nnz;
    const double dense_cost = 4.0 * n * n * n * m + 2.0 * (double)m * m * n * n;
    // rank-one constraints (LowRankOpt's low-rank format): products with
    // V = [v_1 ... v_m] when cheaper than entry pairs and dense products
    const double lowrank_cost = 4.0 * n * n * m + 2.0 * (double)m * m * n;
    b.lowrank = m > 0 && lowrank_cost < std::min(pair_cost, dense_cost) &&
                detect_rank_one(b.n, m, b.nnz, d->A_con[i], d->A_row[i], d->A_col[i], d->A_val[i], &lrV[i], &lrS[i]);
    any_lowrank = any_lowrank || b.lowrank;
    b.dense = !b.lowrank && m > 0 && pair_cost > dense_cost && n * n * m * 8.0 * 3.0 < 96e9;
    if (b.dense) dense_ws = std::max<int64_t>(dense_ws, (int64_t)b.n * b.n * m);
  }
  // ---- device allocations
  auto vec = [&](int64_t k) { return dalloc<double>(s, k); };
  s->b = vec(m); s->dlin = vec(ns); s->Clin = vec((int64_t)m * ns); s->Cw = vec((int64_t)m * ns);
  s->y = vec(m); s->dy = vec(m); s->Rp = vec(m); s->h = vec(m); s->acc = vec(m);
  s->x = vec(ns); s->z = vec(ns); s->dx = vec(ns); s->dz = vec(ns); s->Rdlin = vec(ns); s->zinv = vec(ns);
  s->corrlin = vec(ns); s->vlin = vec(ns); s->ctv = vec(ns); s->wlin = vec(ns);
  s->H = vec((int64_t)m * m); s->H0 = vec((int64_t)m * m);
  s->ir_r = vec(m); s->ir_d = vec(m); s->ir_h = vec(m);
  if (any_lowrank) {
    s->Q1 = vec((int64_t)m * m); s->Q2 = vec((int64_t)m * m);
    if (!s->Q1 || !s->Q2) return bail(MSDP_ERR_OUT_OF_MEMORY);
  }
  if (dense_ws) { s->Tb = vec(dense_ws); s->Bb = vec(dense_ws); }
  {
    int64_t nn_dense = 0;
    for (auto& b : s->B)
      if (b.dense) nn_dense = std::max<int64_t>(nn_dense, (int64_t)b.n * b.n);
    if (nn_dense) {
      s->gpart = vec(nn_dense * kGemvChunks);
      if (!s->gpart) return bail(MSDP_ERR_OUT_OF_MEMORY);
    }
  }
  s->partial = vec(kRedBlocks); s->slots = vec(kSlots);
  s->dinfo = dalloc<int>(s, kInfos);
  bool okalloc = s->b && s->dlin && s->Clin && s->Cw && s->y && s->dy && s->Rp && s->h && s->acc && s->x && s->z &&
                 s->dx && s->dz && s->Rdlin && s->zinv && s->corrlin && s->vlin && s->ctv && s->wlin && s->H &&
                 s->H0 && s->partial && s->slots && s->dinfo && (!dense_ws || (s->Tb && s->Bb)) && s->ir_r &&
                 s->ir_d && s->ir_h;
  if (!okalloc) return bail(MSDP_ERR_OUT_OF_MEMORY);
  if (cudaMallocHost((void**)&s->hslots, sizeof(double) * kSlots) != cudaSuccess ||
      cudaMallocHost((void**)&s->hinfo, sizeof(int) * kInfos) != cudaSuccess)
    return bail(MSDP_ERR_OUT_OF_MEMORY);
  int lwork = 0;
  for (int i = 0; i < s->nb; ++i) {
    Blk& b = s->B[i];
    const int n = b.n;
    const int64_t nn = (int64_t)n * n;
    double** mats[] = {&b.C, &b.X, &b.S, &b.Rd, &b.Ls, &b.Si, &b.Lx, &b.W, &b.G, &b.Gi,
                       &b.dX, &b.dS, &b.corr, &b.ERd, &b.T1, &b.T2, &b.T3, &b.Gs, &b.Hx};
    for (double** p : mats) {
      *p = vec(nn);
      if (!*p) return bail(MSDP_ERR_OUT_OF_MEMORY);
    }
    b.lam = vec(n); b.D = vec(n); b.sc = vec(n); b.w = vec(n); b.gif = vec(n);
    if (!b.lam || !b.D || !b.sc || !b.w || !b.gif) return bail(MSDP_ERR_OUT_OF_MEMORY);
    int lw = 0;
    cusolverDnDpotrf_bufferSize(s->cs, CUBLAS_FILL_MODE_LOWER, n, b.X, n, &lw); lwork = std::max(lwork, lw);
    cusolverDnDpotri_bufferSize(s->cs, CUBLAS_FILL_MODE_LOWER, n, b.X, n, &lw); lwork = std::max(lwork, lw);
    cusolverDnDsyevd_bufferSize(s->cs, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, b.X, n, b.lam, &lw);
    lwork = std::max(lwork, lw);
    // constraints: range check on the host threads (tens of millions of
    // entries for dense constraints), noting whether they come grouped by
    // constraint
    const int32_t *con = d->A_con[i], *row = d->A_row[i], *col = d->A_col[i];
    const double* val = d->A_val[i];
    bool grouped = true;
    {
      std::atomic<bool> bad{false}, unordered{false};
      host_parallel(b.nnz, [&](int64_t lo, int64_t hi) {
        for (int64_t e = lo; e < hi; ++e) {
          if (con[e] < 0 || con[e] >= m || row[e] < 0 || row[e] >= n || col[e] < 0 || col[e] >= n) {
            bad = true;
            return;
          }
          if (e > 0 && con[e] < con[e - 1]) unordered = true;
        }
      });
      if (bad) return bail(MSDP_ERR_INVALID_ARGUMENT);
      grouped = !unordered;
    }
    double cn = 0.0;
    for (int64_t k = 0; k < nn; ++k) cn = std::max(cn, std::fabs(d->C[i][k]));
    b.cnorm = cn;
    cmax = std::max(cmax, cn);
    CU(s, upload(s, b.C, d->C[i], 8 * nn));
    if (b.lowrank) {
      b.V = vec((int64_t)n * m); b.sg = vec(m); b.P = vec((int64_t)n * m);
      if (!b.V || !b.sg || !b.P) return bail(MSDP_ERR_OUT_OF_MEMORY);
      CU(s, upload(s, b.V, lrV[i].data(), 8 * lrV[i].size()));
      CU(s, upload(s, b.sg, lrS[i].data(), 8 * lrS[i].size()));
    } else if (b.dense) {
      // A_j at [j n^2, (j+1) n^2); entries grouped by constraint are
      // scattered by the host threads, each owning a range of constraints
      // (so no two write the same A_j), else by one thread
      const int64_t total = nn * m;
      std::unique_ptr<double[]> Ad(new (std::nothrow) double[(size_t)std::max<int64_t>(total, 1)]);
      if (!Ad) return bail(MSDP_ERR_OUT_OF_MEMORY);
      auto scatter = [&](int c0, int c1) {
        std::fill(Ad.get() + (int64_t)c0 * nn, Ad.get() + (int64_t)c1 * nn, 0.0);
        const int64_t e0 = std::lower_bound(con, con + b.nnz, c0) - con;
        const int64_t e1 = std::lower_bound(con, con + b.nnz, c1) - con;
        for (int64_t e = e0; e < e1; ++e) Ad[(size_t)con[e] * nn + row[e] + (int64_t)col[e] * n] += val[e];
      };
      if (grouped) {
        host_parallel(m, [&](int64_t lo, int64_t hi) { scatter((int)lo, (int)hi); }, 1);
      } else {
        host_parallel(total, [&](int64_t lo, int64_t hi) { std::fill(Ad.get() + lo, Ad.get() + hi, 0.0); });
        for (int64_t e = 0; e < b.nnz; ++e) Ad[(size_t)con[e] * nn + row[e] + (int64_t)col[e] * n] += val[e];
      }
      b.Aall = vec(nn * m);
      if (!b.Aall) return bail(MSDP_ERR_OUT_OF_MEMORY);
      CU(s, upload(s, b.Aall, Ad.get(), 8 * (size_t)total));
    } else {
      const int64_t nnz = b.nnz;
      std::vector<int64_t> idx(nnz);
      std::iota(idx.begin(), idx.end(), 0);
      std::stable_sort(idx.begin(), idx.end(), [&](int64_t a1, int64_t a2) {
        if (con[a1] != con[a2]) return con[a1] < con[a2];
        if (col[a1] != col[a2]) return col[a1] < col[a2];
        return row[a1] < row[a2];
      });
      std::vector<int64_t> cptr(m + 1, 0), pptr(nn + 1, 0);
      std::vector<int32_t> er(nnz), ec(nnz), pc(nnz);
      std::vector<double> ev(nnz), pv(nnz);
      for (int64_t e = 0; e < nnz; ++e) {
        const int64_t q = idx[e];
        er[e] = row[q]; ec[e] = col[q]; ev[e] = val[q];
        cptr[con[q] + 1] += 1;
        pptr[row[q] + (int64_t)col[q] * n + 1] += 1;
      }
      for (int j = 0; j < m; ++j) cptr[j + 1] += cptr[j];
      for (int64_t k = 0; k < nn; ++k) pptr[k + 1] += pptr[k];
      std::vector<int64_t> fill(pptr.begin(), pptr.end() - 1);
      for (int64_t e = 0; e < nnz; ++e) {
        const int64_t q = idx[e];
        const int64_t p = fill[row[q] + (int64_t)col[q] * n]++;
        pc[p] = con[q]; pv[p] = val[q];
      }
      b.conptr = dalloc<int64_t>(s, m + 1); b.posptr = dalloc<int64_t>(s, nn + 1);
      b.erow = dalloc<int32_t>(s, nnz); b.ecol = dalloc<int32_t>(s, nnz); b.pcon = dalloc<int32_t>(s, nnz);
      b.eval = vec(nnz); b.pval = vec(nnz);
      if (!b.conptr || !b.posptr || !b.erow || !b.ecol || !b.pcon || !b.eval || !b.pval)
        return bail(MSDP_ERR_OUT_OF_MEMORY);
      CU(s, upload(s, b.conptr, cptr.data(), 8 * (m + 1)));
      CU(s, upload(s, b.posptr, pptr.data(), 8 * (nn + 1)));
      if (nnz) {
        CU(s, upload(s, b.erow, er.data(), 4 * nnz));
        CU(s, upload(s, b.ecol, ec.data(), 4 * nnz));
        CU(s, upload(s, b.pcon, pc.data(), 4 * nnz));
        CU(s, upload(s, b.eval, ev.data(), 8 * nnz));
        CU(s, upload(s, b.pval, pv.data(), 8 * nnz));
      }
    }
  }
  if (m) {
    int lw = 0;
    cusolverDnDpotrf_bufferSize(s->cs, CUBLAS_FILL_MODE_LOWER, m, s->H, m, &lw);
    lwork = std::max(lwork, lw);
  }
  if (m && c.schur == MSDP_MADNLP_SCHUR) {
    int lw = 0;
    if (cusolverDnDsytrf_bufferSize(s->cs, m, s->H, m, &lw) != CUSOLVER_STATUS_SUCCESS) return bail(MSDP_ERR_CUDA);
    s->sylwork = std::max(lw, 1);
    s->sywork = vec(s->sylwork);
    s->ipiv = dalloc<int>(s, m);
    s->ipiv64 = dalloc<int64_t>(s, m);
    size_t dev = 0, host = 0;
    if (cusolverDnXsytrs_bufferSize(s->cs, CUBLAS_FILL_MODE_LOWER, m, 1, CUDA_R_64F, s->H, m, s->ipiv64, CUDA_R_64F,
                                    s->dy, m, &dev, &host) != CUSOLVER_STATUS_SUCCESS)
      return bail(MSDP_ERR_CUDA);
    s->sytrs_dev_bytes = std::max<size_t>(dev, 1);
    s->sytrs_dev = dalloc<unsigned char>(s, (int64_t)s->sytrs_dev_bytes);
    s->sytrs_host.assign(host, 0);
    if (!s->sywork || !s->ipiv || !s->ipiv64 || !s->sytrs_dev) return bail(MSDP_ERR_OUT_OF_MEMORY);
  }
  s->lwork = std::max(lwork, 1);
  s->work = vec(s->lwork);
  if (!s->work) return bail(MSDP_ERR_OUT_OF_MEMORY);
  if (is_nt(s)) {
    // FP32 eigensolver and refinement workspace of the NT eigendecomposition
    int nref = 0, lw32 = 1;
    for (auto& b : s->B) {
      if (!eig_refinable(b.n)) continue;
      nref = std::max(nref, b.n);
      int lw = 0;
      cusolverDnSsyevd_bufferSize(s->cs, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, b.n, nullptr, b.n,
                                  nullptr, &lw);
      lw32 = std::max(lw32, lw);
    }
    if (nref) {
      s->ef32 = dalloc<float>(s, (int64_t)nref * nref + nref);  // FP32 matrix and eigenvalues
      s->ework32 = dalloc<float>(s, lw32);
      s->elwork32 = lw32;
      s->eibuf = dalloc<int>(s, eigref::ibuf_ints(nref));
      if (!s->ef32 || !s->ework32 || !s->eibuf) return bail(MSDP_ERR_OUT_OF_MEMORY);
    }
  }
  int nmax = 0;
  for (auto& b : s->B) nmax = std::max(nmax, b.n);
  if (nmax >= kLanczosMin) {
    s->lq = vec((int64_t)nmax * (std::min(nmax, kLanczosMax) + 1));
    s->lh = vec(kLanczosMax + 1);
    s->lzp = vec(lanczos_partials(nmax));
    if (!s->lzp) return bail(MSDP_ERR_OUT_OF_MEMORY);
    if (!s->lq || !s->lh) return bail(MSDP_ERR_OUT_OF_MEMORY);
  }
  {
    // batched device Lanczos: two bases (X and S side) per small block
    int64_t q = 0, w = 0, nj = 0;
    for (auto& b : s->B)
      if (b.n <= kLanczosWarpMax) { q += 2 * (int64_t)b.n * b.n; w += 8 * (int64_t)(b.n + 1); nj += 2; }
    if (nj) {
      s->lq2 = vec(q);
      s->lw2 = vec(w);
      s->ljobs = dalloc<unsigned char>(s, (int64_t)sizeof(LanczosJob) * nj);
      if (!s->lq2 || !s->lw2 || !s->ljobs) return bail(MSDP_ERR_OUT_OF_MEMORY);
    }
  }
  double bn = 0.0, dn = 0.0;
  for (int j = 0; j < m; ++j) bn = std::max(bn, std::fabs(d->b[j]));
  for (int k = 0; k < ns; ++k) dn = std::max(dn, std::fabs(d->d_lin[k]));
  s->bnorm = bn; s->dnorm = dn; s->cmax = cmax;
  if (m) CU(s, upload(s, s->b, d->b, 8 * m));
  if (ns) CU(s, upload(s, s->dlin, d->d_lin, 8 * ns));
  if (ns && m) CU(s, upload(s, s->Clin, d->C_lin, 8 * (int64_t)m * ns));
  if (s->fail) return bail(s->fail);
  if (tc_setup(s, c.precision == MSDP_MIXED)) return bail(s->fail ? s->fail : MSDP_ERR_OUT_OF_MEMORY);
  *out = s;
  return MSDP_OK;
}

int msdp_solver_destroy(msdp_solver* s) {
  if (!s) return MSDP_OK;
  release(s);
  delete s;
  return MSDP_OK;
}

int msdp_solver_set_initial_point(msdp_solver* s, const double* const* X, const double* y, const double* x) {
  if (!s || (s->m && !y) || (s->nb && !X)) return MSDP_ERR_INVALID_ARGUMENT;
  s->ipX.assign(s->nb, {});
  for (int i = 0; i < s->nb; ++i) {
    const int64_t nn = (int64_t)s->B[i].n * s->B[i].n;
    if (!X[i]) return MSDP_ERR_INVALID_ARGUMENT;
    s->ipX[i].assign(X[i], X[i] + nn);
  }
  s->ipy.assign(y, y + s->m);
  if (x) s->ipx.assign(x, x + s->ns); else s->ipx.assign(s->ns, 1.0);
  s->has_ip = true;
  return MSDP_OK;
}

int msdp_solver_solve(msdp_solver* s) {
  if (!s) return MSDP_ERR_INVALID_ARGUMENT;
  s->fail = 0;
  for (auto& v : s->phase_s) v = 0.0;
  s->mixed_on = s->comp.precision == MSDP_MIXED;
  s->n32 = s->n64 = 0;
  s->ir_steps = s->ir_fallbacks = 0;
  s->eig_refined = s->eig_dense = s->eig_steps = 0;
  s->lanczos_calls = s->lanczos_steps = s->eigmin_dense = 0;
  s->reg_used = 0.0;
  const double t0 = now_s();
  int rc = initialize(s);
  if (rc) return rc;
  if (!update_termination(s)) return s->fail ? s->fail : MSDP_ERR_CUDA;
  while (s->status == MSDP_REGULAR) {
    const bool ok = s->comp.centering == MSDP_ADAPTIVE_MU ? iterate_adaptive(s) : iterate_mehrotra(s);
    if (!ok) return s->fail ? s->fail : MSDP_ERR_CUDA;
    if (s->status != MSDP_REGULAR) break;
    if (!update_termination(s)) return s->fail ? s->fail : MSDP_ERR_CUDA;
  }
  s->solve_s = now_s() - t0;
  return MSDP_OK;
}

int msdp_solver_get_stats(const msdp_solver* s, msdp_stats* o) {
  if (!s || !o) return MSDP_ERR_INVALID_ARGUMENT;
  std::memset(o, 0, sizeof(*o));
  o->status = s->status; o->iter = s->iter; o->iter_fp64 = s->n64; o->iter_fp32 = s->n32;
  o->pobj = s->pobj; o->dobj = s->dobj; o->inf_pr = s->inf_pr; o->inf_du = s->inf_du; o->gap = s->gap;
  o->mu = s->mu; o->sigma = s->sigma; o->alpha = s->alpha; o->beta = s->beta; o->solve_ns = s->solve_s * 1e9;
  return MSDP_OK;
}

int msdp_solver_get_solution(msdp_solver* s, double* const* X, double* y, double* x, double* z) {
  if (!s) return MSDP_ERR_INVALID_ARGUMENT;
  s->fail = 0;
  for (int i = 0; X && i < s->nb; ++i)
    if (X[i]) CU(s, cudaMemcpyAsync(X[i], s->B[i].X, 8 * (int64_t)s->B[i].n * s->B[i].n, cudaMemcpyDeviceToHost, s->st));
  if (y && s->m) CU(s, cudaMemcpyAsync(y, s->y, 8 * s->m, cudaMemcpyDeviceToHost, s->st));
  if (x && s->ns) CU(s, cudaMemcpyAsync(x, s->x, 8 * s->ns, cudaMemcpyDeviceToHost, s->st));
  if (z && s->ns) CU(s, cudaMemcpyAsync(z, s->z, 8 * s->ns, cudaMemcpyDeviceToHost, s->st));
  CU(s, cudaStreamSynchronize(s->st));
  return s->fail;
}

// ---- component-granular calls (one GPU component beside CPU components)
int msdp_solver_set_iterate(msdp_solver* s, const double* const* X, const double* const* Sm, const double* y,
                            const double* x, const double* z) {
  if (!s || (s->nb && (!X || !Sm)) || (s->m && !y) || (s->ns && (!x || !z))) return MSDP_ERR_INVALID_ARGUMENT;
  s->fail = 0;
  for (int i = 0; i < s->nb; ++i) {
    if (!X[i] || !Sm[i]) return MSDP_ERR_INVALID_ARGUMENT;
    const int64_t nn = (int64_t)s->B[i].n * s->B[i].n;
    CU(s, cudaMemcpyAsync(s->B[i].X, X[i], 8 * nn, cudaMemcpyHostToDevice, s->st));
    CU(s, cudaMemcpyAsync(s->B[i].S, Sm[i], 8 * nn, cudaMemcpyHostToDevice, s->st));
  }
  if (s->m) CU(s, cudaMemcpyAsync(s->y, y, 8 * s->m, cudaMemcpyHostToDevice, s->st));
  if (s->ns) {
    CU(s, cudaMemcpyAsync(s->x, x, 8 * s->ns, cudaMemcpyHostToDevice, s->st));
    CU(s, cudaMemcpyAsync(s->z, z, 8 * s->ns, cudaMemcpyHostToDevice, s->st));
  }
  CU(s, cudaStreamSynchronize(s->st));  // the caller's buffers are free again on return
  s->status = MSDP_REGULAR;
  if (!update_residuals(s)) return s->fail ? s->fail : MSDP_ERR_CUDA;
  return s->fail;
}

int msdp_solver_prepare(msdp_solver* s, int32_t* ok) {
  if (!s || !ok) return MSDP_ERR_INVALID_ARGUMENT;
  s->fail = 0;
  bool p = false;
  if (!prepare(s, &p)) return s->fail ? s->fail : MSDP_ERR_CUDA;
  *ok = p ? 1 : 0;
  return MSDP_OK;
}

int msdp_solver_schur_assemble(msdp_solver* s, int32_t precision, double* H) {
  if (!s || (s->m && !H) || (precision != MSDP_FP64 && precision != MSDP_MIXED)) return MSDP_ERR_INVALID_ARGUMENT;
  if (precision == MSDP_MIXED && !is_nt(s)) return MSDP_ERR_UNSUPPORTED;
  if (precision == MSDP_MIXED &&
      std::any_of(s->B.begin(), s->B.end(),
                  [](const Blk& b) { return (b.dense && !b.stk[1].s) || (b.lowrank && !b.vk[1].s); }))
    return MSDP_ERR_UNSUPPORTED;  // split-precision slices are made for mixed-precision solvers only
  s->fail = 0;
  if (!s->m) return MSDP_OK;
  schur_complement(s, s->H0, precision == MSDP_MIXED ? tcg::kMixed : tcg::kFp64);
  CU(s, cudaMemcpyAsync(H, s->H0, 8 * (int64_t)s->m * s->m, cudaMemcpyDeviceToHost, s->st));
  CU(s, cudaStreamSynchronize(s->st));
  return s->fail;
}

int msdp_solver_get_block_matrix(msdp_solver* s, int32_t block, int32_t which, double* out) {
  if (!s || !out || block < 0 || block >= s->nb) return MSDP_ERR_INVALID_ARGUMENT;
  Blk& b = s->B[block];
  const double* src = nullptr;
  int64_t len = (int64_t)b.n * b.n;
  switch (which) {
    case MSDP_SMAT_W: src = b.W; break;
    case MSDP_SMAT_G: src = b.G; break;
    case MSDP_SMAT_SINV: src = b.Si; break;
    case MSDP_SMAT_LS: src = b.Ls; break;
    case MSDP_SMAT_LX: src = b.Lx; break;
    case MSDP_SMAT_D: src = b.D; len = b.n; break;
    default: return MSDP_ERR_INVALID_ARGUMENT;
  }
  s->fail = 0;
  CU(s, cudaMemcpyAsync(out, src, 8 * len, cudaMemcpyDeviceToHost, s->st));
  CU(s, cudaStreamSynchronize(s->st));
  return s->fail;
}

int msdp_solver_step_eig(msdp_solver* s, int32_t block, const double* L, const double* D, double* lambda_min) {
  if (!s || !L || !D || !lambda_min || block < 0 || block >= s->nb) return MSDP_ERR_INVALID_ARGUMENT;
  Blk& b = s->B[block];
  const int n = b.n;
  const int64_t nn = (int64_t)n * n;
  s->fail = 0;
  reset_slots(s);
  CU(s, cudaMemcpyAsync(b.T3, L, 8 * nn, cudaMemcpyHostToDevice, s->st));
  CU(s, cudaMemcpyAsync(b.T2, D, 8 * nn, cudaMemcpyHostToDevice, s->st));
  form_congruence(s, n, b.T3, b.T2, b.T1);
  int slot;
  LanczosJob job{};  // the copy's source: alive until fetch() below has synchronized
  if (n <= kLanczosWarpMax) {
    slot = next_slot(s);
    job = LanczosJob{n, b.T1, s->lq2, s->lw2, s->slots + slot};
    CU(s, cudaMemcpyAsync(s->ljobs, &job, sizeof(job), cudaMemcpyHostToDevice, s->st));
    k_lanczos_cta<<<1, kLanczosCta, 0, s->st>>>((const LanczosJob*)s->ljobs);
    s->launches += 1;
  } else {
    slot = eigmin_large(s, b, b.T1);
  }
  if (!fetch(s)) return s->fail ? s->fail : MSDP_ERR_CUDA;
  *lambda_min = s->hslots[slot];
  return MSDP_OK;
}

int msdp_solver_get_trajectory(const msdp_solver* s, msdp_iter_record* out, int32_t capacity, int32_t* count) {
  if (!s || !count) return MSDP_ERR_INVALID_ARGUMENT;
  *count = (int32_t)s->traj.size();
  for (int32_t k = 0; out && k < capacity && k < *count; ++k) out[k] = s->traj[k];
  return MSDP_OK;
}

int msdp_solver_get_profile(const msdp_solver* s, double* seconds, int32_t capacity) {
  if (!s || !seconds) return MSDP_ERR_INVALID_ARGUMENT;
  const int n = std::min<int>(capacity, PH_COUNT);
  for (int k = 0; k < n; ++k) seconds[k] = s->phase_s[k];
  return n;
}

const char* msdp_solver_profile_field_name(int32_t i) { return (i >= 0 && i < PH_COUNT) ? kPhaseNames[i] : nullptr; }

namespace {
const char* kCounterNames[] = {"refinement_steps", "refinement_fallbacks", "eig_refined", "eig_dense",
                               "eig_refinement_steps", "tensor_core_products", "lanczos_calls", "lanczos_steps",
                               "eigmin_dense"};
constexpr int kCounters = (int)(sizeof(kCounterNames) / sizeof(kCounterNames[0]));
}  // namespace

int msdp_solver_get_counters(const msdp_solver* s, int64_t* out, int32_t capacity) {
  if (!s || !out) return MSDP_ERR_INVALID_ARGUMENT;
  const int64_t v[kCounters] = {s->ir_steps,    s->ir_fallbacks,  s->eig_refined,   s->eig_dense,   s->eig_steps,
                                s->tc_products, s->lanczos_calls, s->lanczos_steps, s->eigmin_dense};
  const int n = std::min<int>(capacity, kCounters);
  for (int k = 0; k < n; ++k) out[k] = v[k];
  return n;
}

const char* msdp_solver_counter_name(int32_t i) { return (i >= 0 && i < kCounters) ? kCounterNames[i] : nullptr; }

int64_t msdp_solver_device_bytes(const msdp_solver* s) { return s ? s->bytes : 0; }
int64_t msdp_solver_launch_count(const msdp_solver* s) { return s ? s->launches : 0; }
const char* msdp_solver_last_error(const msdp_solver* s) { return s ? s->err.c_str() : "no solver"; }

}  // extern "C"
