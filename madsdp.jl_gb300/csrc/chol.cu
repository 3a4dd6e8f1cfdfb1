// Blocked Cholesky factorization with tensor-core trailing updates; see chol.h.
#include "chol.h"

#include <algorithm>

namespace chol {
namespace {

constexpr int NB = 32;    // block column width (= K of the trailing update)
constexpr int ROWS = 64;  // panel rows per thread block, one per thread

template <class T>
__device__ __forceinline__ T sqrt_t(T x);
template <>
__device__ __forceinline__ double sqrt_t<double>(double x) { return sqrt(x); }
template <>
__device__ __forceinline__ float sqrt_t<float>(float x) { return sqrtf(x); }

// Block column k0: factor the diagonal block, solve the panel rows of this
// thread block, write both back and the panel's slices for the update.
// The factored diagonal block goes to `diag` (NB x NB per block column), not
// to A: other thread blocks of the same launch may still be reading it.
template <class T, int NS>
__global__ void __launch_bounds__(ROWS) k_panel(int n, int k0, double* __restrict__ A, int64_t lda,
                                               int* __restrict__ info, __nv_bfloat16* __restrict__ sl,
                                               int32_t* __restrict__ ex, int64_t Rpad, double* __restrict__ diag) {
  __shared__ T L[NB][NB + 1];
  __shared__ T rdiag[NB];
  __shared__ int bad;
  if (*(volatile int*)info != 0) return;  // an earlier block column failed
  const int kb = min(NB, n - k0);
  const int tid = threadIdx.x;
  for (int idx = tid; idx < NB * NB; idx += ROWS) {
    const int r = idx % NB, c = idx / NB;
    T v = (T)0;
    if (r < kb && c < kb) {
      if (r >= c) v = (T)A[(k0 + r) + (int64_t)(k0 + c) * lda];
    } else if (r == c) {
      v = (T)1;
    }
    L[r][c] = v;
  }
  if (tid == 0) bad = 0;
  __syncthreads();
  for (int j = 0; j < kb; ++j) {
    if (tid == 0) {
      const T d = L[j][j];
      if (!(d > (T)0) || !isfinite(d)) {
        bad = k0 + j + 1;
      } else {
        const T sq = sqrt_t<T>(d);
        L[j][j] = sq;
        rdiag[j] = (T)1 / sq;
      }
    }
    __syncthreads();
    if (bad) break;
    if (tid > j && tid < kb) L[tid][j] *= rdiag[j];
    __syncthreads();
    if (tid > j && tid < kb) {
      const T lij = L[tid][j];
      for (int c = j + 1; c <= tid; ++c) L[tid][c] -= lij * L[c][j];
    }
    __syncthreads();
  }
  if (bad) {
    if (blockIdx.x == 0 && tid == 0) atomicCAS(info, 0, bad);
    return;
  }
  if (blockIdx.x == 0)
    for (int idx = tid; idx < NB * NB; idx += ROWS) diag[(int64_t)k0 * NB + idx] = (double)L[idx % NB][idx / NB];
  // panel rows exist only below a full diagonal block (k0 + NB < n)
  const int64_t i = (int64_t)k0 + NB + (int64_t)blockIdx.x * ROWS + tid;
  if (kb < NB || i >= n) return;
  T x[NB];
#pragma unroll
  for (int c = 0; c < NB; ++c) x[c] = (T)A[i + (int64_t)(k0 + c) * lda];
  // x <- x L11^-T, column by column (each solved entry updates the later ones)
#pragma unroll
  for (int c = 0; c < NB; ++c) {
    x[c] *= rdiag[c];
#pragma unroll
    for (int k = c + 1; k < NB; ++k) x[k] -= x[c] * L[k][c];
  }
  int mx = 0;
#pragma unroll
  for (int c = 0; c < NB; ++c) {
    const double v = (double)x[c];
    A[i + (int64_t)(k0 + c) * lda] = v;
    mx = max(mx, tcg::exp_field(v));
  }
  const int e = tcg::row_exp(mx);
  const int64_t R = i - (k0 + NB);
  ex[R] = e;
#pragma unroll
  for (int c = 0; c < NB; ++c) tcg::write_slices<NS>((double)x[c], e, sl + R * NB + c, Rpad * NB);
}

// Lower triangles of the factored diagonal blocks into A (after the last
// block column; the info check skips a failed factorization).
__global__ void k_put_diag(int n, double* __restrict__ A, int64_t lda, const double* __restrict__ diag,
                           const int* __restrict__ info) {
  if (*info != 0) return;
  const int64_t total = (int64_t)((n + NB - 1) / NB) * NB * NB;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k0 = idx / (NB * NB) * NB;
    const int q = (int)(idx % (NB * NB)), r = q % NB, c = q / NB;
    if (r >= c && k0 + r < n) A[(k0 + r) + (k0 + c) * lda] = diag[idx];
  }
}

// Inverse of each factored diagonal block (one thread block of NB warps per
// block; warp c forms column c row by row with a warp sum).
__global__ void __launch_bounds__(NB * 32) k_diag_inverse(int n, const double* __restrict__ diag,
                                                          double* __restrict__ dinv, const int* __restrict__ info) {
  if (*info != 0) return;
  __shared__ double Ls[NB][NB + 1], inv[NB][NB + 1];
  const int64_t k0 = (int64_t)blockIdx.x * NB;
  const int kb = (int)min((int64_t)NB, (int64_t)n - k0);
  const int t = threadIdx.x, lane = t & 31, c = t >> 5;
  {
    const int r = t % NB, cc = t / NB;
    Ls[r][cc] = diag[k0 * NB + t];  // column-major NB x NB block
    inv[r][cc] = 0.0;
  }
  __syncthreads();
  for (int r = 0; r < kb; ++r) {
    double term = (lane >= c && lane < r) ? Ls[r][lane] * inv[lane][c] : 0.0;
    for (int o = 16; o; o >>= 1) term += __shfl_xor_sync(0xffffffffu, term, o);
    if (lane == 0 && c <= r) inv[r][c] = ((r == c ? 1.0 : 0.0) - term) / Ls[r][r];
    __syncthreads();
  }
  {
    const int r = t % NB, cc = t / NB;
    dinv[k0 * NB + t] = (r < kb && cc < kb) ? inv[r][cc] : 0.0;
  }
}

// x <- L^-T L^-1 x with the factor in L (lower) and the inverses of its
// diagonal blocks; one thread block, block row by block row.  The sums over
// the solved part read NB consecutive entries per column (coalesced), four
// independent accumulators per thread.
__global__ void __launch_bounds__(1024) k_chol_solve(int n, const double* __restrict__ L, int64_t ld,
                                                     const double* __restrict__ dinv, double* x,
                                                     const int* __restrict__ info) {
  if (*info != 0) return;
  __shared__ double red[32][33];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int nbk = (n + NB - 1) / NB;
  // forward: L y = x
  for (int b = 0; b < nbk; ++b) {
    const int r0 = b * NB, rows = min(NB, n - r0);
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    if (lane < rows) {
      const double* Lr = L + r0 + lane;
      int c = w;
      for (; c + 96 < r0; c += 128) {
        a0 = fma(Lr[(int64_t)c * ld], x[c], a0);
        a1 = fma(Lr[(int64_t)(c + 32) * ld], x[c + 32], a1);
        a2 = fma(Lr[(int64_t)(c + 64) * ld], x[c + 64], a2);
        a3 = fma(Lr[(int64_t)(c + 96) * ld], x[c + 96], a3);
      }
      for (; c < r0; c += 32) a0 = fma(Lr[(int64_t)c * ld], x[c], a0);
    }
    red[w][lane] = (a0 + a1) + (a2 + a3);
    __syncthreads();
    if (w == 0) {
      double sum = 0.0;
      for (int g = 0; g < 32; ++g) sum += red[g][lane];
      const double v = lane < rows ? x[r0 + lane] - sum : 0.0;
      const double* Di = dinv + (int64_t)b * NB * NB;
      double y = 0.0;
      for (int c = 0; c < NB; ++c) y = fma(Di[lane + c * NB], __shfl_sync(0xffffffffu, v, c), y);
      if (lane < rows) x[r0 + lane] = y;
    }
    __syncthreads();
  }
  // backward: L' z = y
  for (int b = nbk - 1; b >= 0; --b) {
    const int r0 = b * NB, rows = min(NB, n - r0);
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    if (w < rows) {
      const double* Lc = L + (int64_t)(r0 + w) * ld;
      int j = r0 + NB + lane;
      for (; j + 96 < n; j += 128) {
        a0 = fma(Lc[j], x[j], a0);
        a1 = fma(Lc[j + 32], x[j + 32], a1);
        a2 = fma(Lc[j + 64], x[j + 64], a2);
        a3 = fma(Lc[j + 96], x[j + 96], a3);
      }
      for (; j < n; j += 32) a0 = fma(Lc[j], x[j], a0);
    }
    double a = (a0 + a1) + (a2 + a3);
    for (int o = 16; o; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0) red[0][w] = a;
    __syncthreads();
    if (w == 0) {
      const double v = lane < rows ? x[r0 + lane] - red[0][lane] : 0.0;
      const double* Di = dinv + (int64_t)b * NB * NB;
      double y = 0.0;
      for (int c = 0; c < NB; ++c) y = fma(Di[c + lane * NB], __shfl_sync(0xffffffffu, v, c), y);
      if (lane < rows) x[r0 + lane] = y;
    }
    __syncthreads();
  }
}

int64_t panel_bytes(int64_t nmax) { return tcg::sliced_bytes(nmax, NB, 7); }

}  // namespace

int64_t work_bytes(int64_t nmax) {
  nmax = std::max<int64_t>(nmax, 1);
  return panel_bytes(nmax) + 2 * (nmax + NB) * NB * 8;
}

cudaError_t init(Work* w, void* mem, int64_t nmax, int* err, cudaStream_t st) {
  w->mem = mem;
  w->nmax = std::max<int64_t>(nmax, 1);
  w->err = err;
  w->diag = (double*)((char*)mem + panel_bytes(w->nmax));
  w->dinv = w->diag + (w->nmax + NB) * NB;
  return tcg::sliced_init(&w->panel, mem, w->nmax, NB, 7, st);
}

cudaError_t solve(const Work& w, int n, const double* L, int64_t ld, double* x, const int* info, cudaStream_t st,
                  int64_t* launches) {
  if (n <= 0) return cudaSuccess;
  if (n > w.nmax) return cudaErrorInvalidValue;
  k_chol_solve<<<1, 1024, 0, st>>>(n, L, ld, w.dinv, x, info);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t potrf(Work& w, int n, double* A, int64_t lda, int* info, tcg::Mode mode, cudaStream_t st,
                  int64_t* launches) {
  if (n < 0 || n > w.nmax || lda < std::max(n, 1)) return cudaErrorInvalidValue;
  const int ns = tcg::slices_of(mode);
  cudaError_t e = cudaSuccess;
  if (w.panel.ns != ns) {
    e = tcg::sliced_init(&w.panel, w.mem, w.nmax, NB, ns, st, false);
    if (e != cudaSuccess) return e;
  }
  e = cudaMemsetAsync(info, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  for (int k0 = 0; k0 < n; k0 += NB) {
    const int kb = std::min(NB, n - k0);
    const int64_t nr = n - k0 - kb;
    const unsigned grid = (unsigned)std::max<int64_t>(1, (nr + ROWS - 1) / ROWS);
    if (mode == tcg::kMixed)
      k_panel<float, 3><<<grid, ROWS, 0, st>>>(n, k0, A, lda, info, w.panel.s, w.panel.ex, w.panel.Rpad, w.diag);
    else
      k_panel<double, 7><<<grid, ROWS, 0, st>>>(n, k0, A, lda, info, w.panel.s, w.panel.ex, w.panel.Rpad, w.diag);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (launches) *launches += 1;
    if (nr > 0) {
      w.panel.rows = nr;
      tcg::Out o;
      o.C = A + (k0 + kb) + (int64_t)(k0 + kb) * lda;
      o.ldc = lda;
      o.alpha = -1.0;
      o.beta = 1.0;
      o.lower = true;
      o.err = w.err;
      e = tcg::gemm(w.panel, w.panel, mode, o, st, launches);
      if (e != cudaSuccess) return e;
    }
  }
  if (n > 0) {
    const int64_t total = (int64_t)((n + NB - 1) / NB) * NB * NB;
    k_put_diag<<<(unsigned)std::min<int64_t>((total + 255) / 256, 1024), 256, 0, st>>>(n, A, lda, w.diag, info);
    k_diag_inverse<<<(unsigned)((n + NB - 1) / NB), NB * 32, 0, st>>>(n, w.diag, w.dinv, info);
    if (launches) *launches += 2;
    e = cudaGetLastError();
  }
  return e;
}

}  // namespace chol

// ---------------------------------------------------------------- C ABI
// DenseCholesky's factorize! (src/schur_solvers.jl:15-19) for one dense
// matrix on the device (include/madsdp_gpu.h).
#include "../../include/madsdp_gpu.h"

extern "C" int msdp_dense_cholesky(int32_t precision, int32_t n, double* A, int64_t lda, int32_t* info,
                                   void* stream) {
  if (n < 0 || !info || (n && !A) || lda < std::max(n, 1)) return MSDP_ERR_INVALID_ARGUMENT;
  if (precision != MSDP_FP64 && precision != MSDP_MIXED) return MSDP_ERR_INVALID_ARGUMENT;
  *info = 0;
  if (n == 0) return MSDP_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t wb = chol::work_bytes(n);
  char* mem = nullptr;
  if (cudaMalloc(&mem, (size_t)(wb + 512)) != cudaSuccess) return MSDP_ERR_OUT_OF_MEMORY;
  int* dinfo = (int*)(mem + wb);
  int* derr = dinfo + 1;
  chol::Work w;
  cudaError_t e = cudaMemsetAsync(derr, 0, sizeof(int), st);
  if (e == cudaSuccess) e = chol::init(&w, mem, n, derr, st);
  if (e == cudaSuccess)
    e = chol::potrf(w, n, A, lda, dinfo, precision == MSDP_MIXED ? tcg::kMixed : tcg::kFp64, st, nullptr);
  int h[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, dinfo, 2 * sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(mem);
  if (e != cudaSuccess || h[1]) return MSDP_ERR_CUDA;
  *info = h[0];
  return MSDP_OK;
}
