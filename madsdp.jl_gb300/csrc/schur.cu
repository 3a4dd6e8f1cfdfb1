// Device workspace of one m x m Schur system for the reference's
// AbstractSchurSolver contract (src/components.jl:253-266,
// src/schur_solvers.jl:10-21): the host assembles H (as MadSDP's driver
// does), factorize! runs the blocked Cholesky of chol.h on the GPU and
// schur_solve! the two triangular solves.  With MSDP_MIXED the factor is
// FP32-class and each solve is refined against H in FP64 (residual
// h - H x from the stored lower triangle) until the residual stops
// shrinking; a solve whose residual then exceeds 1e-11 |h| refactors H in
// FP64, which stays in use until the next factorize.  When the FP32-class
// factorization itself breaks down, factorize! falls back to FP64 at once.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "../../include/madsdp_gpu.h"
#include "chol.h"

struct msdp_context;
extern "C" void* msdp_context_stream(const msdp_context* ctx);

struct msdp_schur {
  cudaStream_t st = nullptr;
  int m = 0;
  bool mixed = false, fp64_now = false;
  double *H = nullptr, *L = nullptr, *x = nullptr, *r = nullptr, *d = nullptr, *b = nullptr;
  double* red = nullptr;   // partial maxima of |r| and |b|
  int* info = nullptr;
  int* err = nullptr;
  double* hmax = nullptr;  // pinned host copy of the partial maxima
  void* wmem = nullptr;
  chol::Work w;
  bool factored = false;
};

namespace {

constexpr int kThreads = 256;
constexpr int kRedBlocks = 128;

// y = Hsym x with Hsym(i, j) = H(max(i, j), min(i, j)) (lower triangle):
// the j <= i part by rows (coalesced over i), then the j > i part by columns.
__global__ void k_symv_lower_rows(int m, const double* __restrict__ H, const double* __restrict__ x,
                                  double* __restrict__ y) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int j = 0; j <= i; ++j) s = fma(H[i + (int64_t)j * m], x[j], s);
    y[i] = s;
  }
}
__global__ void k_symv_lower_cols(int m, const double* __restrict__ H, const double* __restrict__ x,
                                  double* __restrict__ y) {
  __shared__ double red[kThreads / 32];
  for (int i = blockIdx.x; i < m; i += gridDim.x) {
    const double* col = H + (int64_t)i * m;
    double s = 0.0;
    for (int j = i + 1 + threadIdx.x; j < m; j += blockDim.x) s = fma(col[j], x[j], s);
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < kThreads / 32; ++w) t += red[w];
      y[i] += t;
    }
    __syncthreads();
  }
}
// r = b - r; partial maxima of |r| and |b| per block
__global__ void k_residual(int m, const double* __restrict__ b, double* __restrict__ r, double* __restrict__ part) {
  __shared__ double rr[kThreads / 32], bb[kThreads / 32];
  double mr = 0.0, mb = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    const double v = b[i] - r[i];
    r[i] = v;
    mr = fmax(mr, fabs(v));
    mb = fmax(mb, fabs(b[i]));
  }
  for (int o = 16; o; o >>= 1) {
    mr = fmax(mr, __shfl_xor_sync(0xffffffffu, mr, o));
    mb = fmax(mb, __shfl_xor_sync(0xffffffffu, mb, o));
  }
  if ((threadIdx.x & 31) == 0) {
    rr[threadIdx.x >> 5] = mr;
    bb[threadIdx.x >> 5] = mb;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, c = 0.0;
    for (int w = 0; w < kThreads / 32; ++w) {
      a = fmax(a, rr[w]);
      c = fmax(c, bb[w]);
    }
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = c;
  }
}
__global__ void k_axpy1(int m, double* __restrict__ x, const double* __restrict__ d) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) x[i] += d[i];
}

int factor(msdp_schur* ws, tcg::Mode mode, int32_t* success) {
  const int m = ws->m;
  if (cudaMemcpyAsync(ws->L, ws->H, sizeof(double) * m * m, cudaMemcpyDeviceToDevice, ws->st) != cudaSuccess ||
      chol::potrf(ws->w, m, ws->L, m, ws->info, mode, ws->st, nullptr) != cudaSuccess)
    return MSDP_ERR_CUDA;
  int h[2] = {0, 0};
  if (cudaMemcpyAsync(h, ws->info, sizeof(int), cudaMemcpyDeviceToHost, ws->st) != cudaSuccess ||
      cudaMemcpyAsync(h + 1, ws->err, sizeof(int), cudaMemcpyDeviceToHost, ws->st) != cudaSuccess ||
      cudaStreamSynchronize(ws->st) != cudaSuccess || h[1])
    return MSDP_ERR_CUDA;
  *success = h[0] == 0 ? 1 : 0;
  ws->factored = h[0] == 0;
  return MSDP_OK;
}

// ws->r = b - H x; the largest |r| and |b| through the pinned partials
bool residual(msdp_schur* ws, double* rn, double* bn) {
  const int m = ws->m;
  const unsigned g = (unsigned)std::min((m + kThreads - 1) / kThreads, 152 * 8);
  k_symv_lower_rows<<<g, kThreads, 0, ws->st>>>(m, ws->H, ws->x, ws->r);
  k_symv_lower_cols<<<(unsigned)std::min(m, 152 * 8), kThreads, 0, ws->st>>>(m, ws->H, ws->x, ws->r);
  k_residual<<<kRedBlocks, kThreads, 0, ws->st>>>(m, ws->b, ws->r, ws->red);
  if (cudaMemcpyAsync(ws->hmax, ws->red, sizeof(double) * 2 * kRedBlocks, cudaMemcpyDeviceToHost, ws->st) !=
          cudaSuccess ||
      cudaStreamSynchronize(ws->st) != cudaSuccess)
    return false;
  double a = 0.0, c = 0.0;
  for (int k = 0; k < kRedBlocks; ++k) {
    a = std::max(a, ws->hmax[2 * k]);
    c = std::max(c, ws->hmax[2 * k + 1]);
  }
  *rn = a;
  *bn = c;
  return true;
}

}  // namespace

extern "C" {

int msdp_schur_create(msdp_context* ctx, int32_t m, int32_t precision, msdp_schur** out) {
  if (!ctx || !out || m < 0 || (precision != MSDP_FP64 && precision != MSDP_MIXED)) return MSDP_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  auto ws = new msdp_schur();
  ws->st = (cudaStream_t)msdp_context_stream(ctx);
  ws->m = m;
  ws->mixed = precision == MSDP_MIXED;
  const int64_t mm = std::max<int64_t>((int64_t)m * m, 1), mv = std::max(m, 1);
  const int64_t wb = chol::work_bytes(mv);
  const size_t bytes = sizeof(double) * (2 * mm + 4 * mv + 2 * kRedBlocks) + 256 + wb;
  char* p = nullptr;
  if (cudaMalloc(&p, bytes) != cudaSuccess) {
    delete ws;
    return MSDP_ERR_OUT_OF_MEMORY;
  }
  ws->wmem = p;
  double* q = (double*)(p + wb);
  ws->H = q; q += mm;
  ws->L = q; q += mm;
  ws->x = q; q += mv;
  ws->r = q; q += mv;
  ws->d = q; q += mv;
  ws->b = q; q += mv;
  ws->red = q; q += 2 * kRedBlocks;
  ws->info = (int*)q;
  ws->err = ws->info + 1;
  if (cudaMallocHost((void**)&ws->hmax, sizeof(double) * 2 * kRedBlocks) != cudaSuccess ||
      cudaMemsetAsync(ws->info, 0, 2 * sizeof(int), ws->st) != cudaSuccess ||
      chol::init(&ws->w, p, mv, ws->err, ws->st) != cudaSuccess) {
    msdp_schur_destroy(ws);
    return MSDP_ERR_CUDA;
  }
  *out = ws;
  return MSDP_OK;
}

int msdp_schur_destroy(msdp_schur* ws) {
  if (!ws) return MSDP_OK;
  if (ws->st) cudaStreamSynchronize(ws->st);
  if (ws->wmem) cudaFree(ws->wmem);
  if (ws->hmax) cudaFreeHost(ws->hmax);
  delete ws;
  return MSDP_OK;
}

int msdp_schur_factorize(msdp_schur* ws, const double* H, int32_t* success) {
  if (!ws || !H || !success) return MSDP_ERR_INVALID_ARGUMENT;
  *success = 0;
  if (ws->m == 0) {
    *success = 1;
    ws->factored = true;
    return MSDP_OK;
  }
  if (cudaMemcpyAsync(ws->H, H, sizeof(double) * ws->m * ws->m, cudaMemcpyHostToDevice, ws->st) != cudaSuccess)
    return MSDP_ERR_CUDA;
  ws->fp64_now = !ws->mixed;
  const int rc = factor(ws, ws->mixed ? tcg::kMixed : tcg::kFp64, success);
  if (rc || *success || !ws->mixed) return rc;
  // the FP32-class factorization broke down (H too ill-conditioned for it):
  // the FP64 factor decides issuccess, as DenseCholesky's does
  ws->fp64_now = true;
  return factor(ws, tcg::kFp64, success);
}

int msdp_schur_solve(msdp_schur* ws, double* rhs) {
  if (!ws || (!rhs && ws->m)) return MSDP_ERR_INVALID_ARGUMENT;
  if (!ws->factored) return MSDP_ERR_INVALID_ARGUMENT;
  const int m = ws->m;
  if (m == 0) return MSDP_OK;
  cudaStream_t st = ws->st;
  if (cudaMemcpyAsync(ws->b, rhs, sizeof(double) * m, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(ws->x, ws->b, sizeof(double) * m, cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
      chol::solve(ws->w, m, ws->L, m, ws->x, ws->info, st, nullptr) != cudaSuccess)
    return MSDP_ERR_CUDA;
  if (!ws->fp64_now) {
    double prev = INFINITY, rn = INFINITY, bn = 0.0;
    for (int it = 0; it < 10; ++it) {
      if (!residual(ws, &rn, &bn)) return MSDP_ERR_CUDA;
      if (rn <= 1e-14 * bn || !(rn < 0.5 * prev)) break;
      prev = rn;
      if (cudaMemcpyAsync(ws->d, ws->r, sizeof(double) * m, cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
          chol::solve(ws->w, m, ws->L, m, ws->d, ws->info, st, nullptr) != cudaSuccess)
        return MSDP_ERR_CUDA;
      k_axpy1<<<(unsigned)std::min((m + kThreads - 1) / kThreads, 152 * 8), kThreads, 0, st>>>(m, ws->x, ws->d);
    }
    if (!(std::isfinite(rn) && rn <= 1e-11 * std::max(bn, 1e-300))) {
      // refinement stalled: FP64 factor from here on
      int32_t ok = 0;
      const int rc = factor(ws, tcg::kFp64, &ok);
      if (rc) return rc;
      if (!ok) return MSDP_ERR_CUDA;
      ws->fp64_now = true;
      if (cudaMemcpyAsync(ws->x, ws->b, sizeof(double) * m, cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
          chol::solve(ws->w, m, ws->L, m, ws->x, ws->info, st, nullptr) != cudaSuccess)
        return MSDP_ERR_CUDA;
    }
  }
  if (cudaMemcpyAsync(rhs, ws->x, sizeof(double) * m, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return MSDP_ERR_CUDA;
  return MSDP_OK;
}

int msdp_schur_fp64_active(const msdp_schur* ws) { return ws && ws->fp64_now ? 1 : 0; }

}  // extern "C"
