// Elementwise and cluster parts of one eigendecomposition refinement step
// (eigref.h).
#include "eigref.h"

#include <algorithm>
#include <cmath>
#include <mutex>

namespace eigref {
namespace {

constexpr int kThreads = 256;
constexpr int kLd = kMaxCluster + 1;  // padded row stride of the cluster blocks in shared memory
constexpr int kClusterThreads = 1024;
constexpr int kClusterSmem = 3 * kMaxCluster * kLd * (int)sizeof(double);

__device__ __forceinline__ double lower(const double* A, int n, int i, int j) {
  return i >= j ? A[i + (int64_t)j * n] : A[j + (int64_t)i * n];
}
__device__ __forceinline__ void max_bits(unsigned long long* p, double v) {
  atomicMax(p, (unsigned long long)__double_as_longlong(v));
}

__global__ void k_f2(int64_t count, const double* __restrict__ src, float* __restrict__ dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (float)src[i];
}
__global__ void k_d2(int64_t count, const float* __restrict__ src, double* __restrict__ dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (double)src[i];
}

// reach[i] = i, no clusters, residual measures 0
__global__ void k_init(int n, int* ibuf, unsigned long long* res) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) ibuf[i] = i;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ibuf[3 * n] = 0;
    res[0] = res[1] = res[2] = 0ull;
  }
}

// Rayleigh quotients lam_i = S_ii / R_ii; res[2] = max |lam_i|
__global__ void k_lambda(int n, const double* __restrict__ S, const double* __restrict__ R, double* lam,
                         unsigned long long* res, int* flag) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double v = S[i + (int64_t)i * n] / R[i + (int64_t)i * n];
    lam[i] = v;
    if (isfinite(v)) max_bits(res + 2, fabs(v));
    else *flag = 1;
  }
}

// First-order corrections of the separated pairs; coupled pairs widen
// their row's reach (the cluster solve writes their entries).
__global__ void __launch_bounds__(kThreads) k_pairs(int n, const double* __restrict__ S, const double* __restrict__ R,
                                                    const double* __restrict__ lam, double tau, double* E1,
                                                    int* reach, unsigned long long* res, int* flag) {
  const int64_t total = (int64_t)n * n;
  double mnum = 0.0, mrt = 0.0;
  bool bad = false;
  // an off-diagonal residual at rounding level of max |lam| (res[2], set by
  // k_lambda) needs no rotation, however close the two eigenvalues are
  const double negligible = 64.0 * 2.220446049250313e-16 * __longlong_as_double((long long)res[2]);
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(idx % n), j = (int)(idx / n);
    const double rij = lower(R, n, i, j);
    if (i == j) {
      E1[idx] = 1.0 + 0.5 * (1.0 - rij);
      mrt = fmax(mrt, fabs(1.0 - rij));
      continue;
    }
    const double s = lower(S, n, i, j);
    const double rt = -rij;                      // (I - R)_ij
    const double li = lam[i], lj = lam[j];
    const double num_ij = s + lj * rt, num_ji = s + li * rt;
    const double gap = lj - li;
    const double num = fmax(fabs(num_ij), fabs(num_ji));
    mnum = fmax(mnum, num);
    mrt = fmax(mrt, fabs(rt));
    if (!isfinite(num)) bad = true;
    if (num <= negligible) {
      E1[idx] = 0.5 * rt;  // already diagonal to rounding: orthonormalize only
    } else if (gap != 0.0 && num <= tau * fabs(gap)) {
      E1[idx] = num_ij / gap;
    } else {
      E1[idx] = 0.0;
      atomicMax(&reach[min(i, j)], max(i, j));
    }
  }
  // block maxima, one atomic each per block
  __shared__ double red[2][kThreads / 32];
  for (int o = 16; o > 0; o >>= 1) {
    mnum = fmax(mnum, __shfl_xor_sync(0xffffffffu, mnum, o));
    mrt = fmax(mrt, __shfl_xor_sync(0xffffffffu, mrt, o));
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = mnum;
    red[1][threadIdx.x >> 5] = mrt;
  }
  bad = __syncthreads_or(bad);
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < kThreads / 32; ++w) {
      a = fmax(a, red[0][w]);
      b = fmax(b, red[1][w]);
    }
    max_bits(res, a);
    max_bits(res + 1, b);
    if (bad) *flag = 1;
  }
}

// Clusters: maximal index ranges closed under the coupled pairs' reach
// (one thread; n steps).  list[2c], list[2c+1] = start and size of the
// c-th cluster of size >= 2; count at ibuf[3n].
__global__ void k_clusters(int n, int* ibuf, int* flag) {
  if (threadIdx.x != 0 || blockIdx.x != 0 || n <= 0) return;
  const int* reach = ibuf;
  int* list = ibuf + n;
  int count = 0, a = 0, end = reach[0];
  for (int i = 1; i <= n; ++i) {
    if (i == n || i > end) {
      const int k = end - a + 1;
      if (k >= 2) {
        list[2 * count] = a;
        list[2 * count + 1] = k;
        ++count;
        if (k > kMaxCluster) *flag = 1;
      }
      if (i == n) break;
      a = i;
      end = reach[i];
    } else {
      end = max(end, reach[i]);
    }
  }
  ibuf[3 * n] = count;
}

// Each cluster [a, a+k): its block of I + E becomes O = I + R~_cc/2
// (first-order orthonormalization), C = O S_cc O is diagonalized by cyclic
// Jacobi with the parallel (round-robin) pair order, one warp per pair, and
// the cluster's columns of I + E (all n rows) are multiplied by the
// rotation Q, in row chunks staged in shared memory.
__global__ void __launch_bounds__(kClusterThreads) k_cluster_solve(int n, const double* __restrict__ S,
                                                                   const double* __restrict__ R, const int* ibuf,
                                                                   double* E1) {
  extern __shared__ double sm[];
  double* C = sm;                       // [k][kLd], C[i * kLd + j] = C_ij
  double* Q = C + kMaxCluster * kLd;
  double* O = Q + kMaxCluster * kLd;
  const int count = ibuf[3 * n];
  const int* list = ibuf + n;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int c = blockIdx.x; c < count; c += gridDim.x) {
    const int a = list[2 * c], k = list[2 * c + 1];
    if (k > kMaxCluster) continue;  // flagged by k_clusters
    // O = I + (I - R_cc)/2 (also the block of I + E); Q = S_cc
    for (int t = threadIdx.x; t < k * k; t += blockDim.x) {
      const int i = t % k, j = t / k;
      const double o = (i == j ? 1.0 : 0.0) + 0.5 * ((i == j ? 1.0 : 0.0) - lower(R, n, a + i, a + j));
      O[i * kLd + j] = o;
      E1[(a + i) + (int64_t)(a + j) * n] = o;
      Q[i * kLd + j] = lower(S, n, a + i, a + j);
    }
    __syncthreads();
    // C = S_cc O, then Q = O C (symmetric), then C = Q and Q = I
    for (int t = threadIdx.x; t < k * k; t += blockDim.x) {
      const int i = t % k, j = t / k;
      double acc = 0.0;
      for (int l = 0; l < k; ++l) acc = fma(Q[i * kLd + l], O[l * kLd + j], acc);
      C[i * kLd + j] = acc;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < k * k; t += blockDim.x) {
      const int i = t % k, j = t / k;
      double acc = 0.0;
      for (int l = 0; l < k; ++l) acc = fma(O[i * kLd + l], C[l * kLd + j], acc);
      Q[i * kLd + j] = acc;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < k * k; t += blockDim.x) {
      const int i = t % k, j = t / k;
      C[i * kLd + j] = 0.5 * (Q[i * kLd + j] + Q[j * kLd + i]);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < k * k; t += blockDim.x) {
      const int i = t % k, j = t / k;
      Q[i * kLd + j] = i == j ? 1.0 : 0.0;
    }
    __syncthreads();
    const int K = k + (k & 1);
    for (int sweep = 0; sweep < 40; ++sweep) {
      int rotated = 0;
      for (int r = 0; r < K - 1; ++r) {
        int p = -1, q = -1;
        if (warp < K / 2) {
          if (warp == 0) { p = K - 1; q = r; }
          else { p = (r + warp) % (K - 1); q = (r - warp + (K - 1)) % (K - 1); }
          if (p >= k || q >= k) p = q = -1;
        }
        double cs = 1.0, sn = 0.0;
        if (p >= 0) {
          const double app = C[p * kLd + p], aqq = C[q * kLd + q], apq = C[p * kLd + q];
          if (fabs(apq) > 1e-15 * sqrt(fabs(app * aqq)) && fabs(apq) > 1e-300) {
            const double z = (aqq - app) / (2.0 * apq);
            const double t = (z >= 0.0 ? 1.0 : -1.0) / (fabs(z) + sqrt(1.0 + z * z));
            cs = 1.0 / sqrt(1.0 + t * t);
            sn = t * cs;
            rotated = 1;
          } else {
            p = q = -1;
          }
        }
        __syncthreads();
        // rows p, q of C
        if (p >= 0)
          for (int l = lane; l < k; l += 32) {
            const double x = C[p * kLd + l], y = C[q * kLd + l];
            C[p * kLd + l] = cs * x - sn * y;
            C[q * kLd + l] = sn * x + cs * y;
          }
        __syncthreads();
        // columns p, q of C and of Q
        if (p >= 0)
          for (int l = lane; l < k; l += 32) {
            const double x = C[l * kLd + p], y = C[l * kLd + q];
            C[l * kLd + p] = cs * x - sn * y;
            C[l * kLd + q] = sn * x + cs * y;
            const double u = Q[l * kLd + p], v = Q[l * kLd + q];
            Q[l * kLd + p] = cs * u - sn * v;
            Q[l * kLd + q] = sn * u + cs * v;
          }
        __syncthreads();
      }
      if (!__syncthreads_or(rotated)) break;
    }
    // columns a..a+k of I + E times Q, P rows at a time (C: input chunk,
    // O: output chunk; both free now)
    const int P = (kMaxCluster * kLd) / k;
    for (int p0 = 0; p0 < n; p0 += P) {
      const int rows = min(P, n - p0);
      for (int t = threadIdx.x; t < rows * k; t += blockDim.x) {
        const int r = t % rows, l = t / rows;
        C[r * k + l] = E1[(p0 + r) + (int64_t)(a + l) * n];
      }
      __syncthreads();
      for (int t = threadIdx.x; t < rows * k; t += blockDim.x) {
        const int r = t % rows, j = t / rows;
        double acc = 0.0;
        for (int l = 0; l < k; ++l) acc = fma(C[r * k + l], Q[l * kLd + j], acc);
        O[r * k + j] = acc;
      }
      __syncthreads();
      for (int t = threadIdx.x; t < rows * k; t += blockDim.x) {
        const int r = t % rows, j = t / rows;
        E1[(p0 + r) + (int64_t)(a + j) * n] = O[r * k + j];
      }
      __syncthreads();
    }
  }
}

// A_ii += f * (*t) (the diagonal shift by a device scalar)
__global__ void k_shift_diag(int n, double* A, const double* t, double f) {
  const double sh = f * *t;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) A[i + (int64_t)i * n] += sh;
}
__global__ void k_shift_vec(int n, double* v, const double* t, double f) {
  const double sh = f * *t;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] += sh;
}

unsigned grid_for(int64_t count) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((count + kThreads - 1) / kThreads, 152 * 8));
}

}  // namespace

cudaError_t to_float(int64_t count, const double* src, float* dst, cudaStream_t st) {
  k_f2<<<grid_for(count), kThreads, 0, st>>>(count, src, dst);
  return cudaGetLastError();
}
cudaError_t to_double(int64_t count, const float* src, double* dst, cudaStream_t st) {
  k_d2<<<grid_for(count), kThreads, 0, st>>>(count, src, dst);
  return cudaGetLastError();
}

cudaError_t shift_diag(int n, double* A, const double* t, double f, cudaStream_t st) {
  k_shift_diag<<<grid_for(n), kThreads, 0, st>>>(n, A, t, f);
  return cudaGetLastError();
}
cudaError_t shift_vec(int n, double* v, const double* t, double f, cudaStream_t st) {
  k_shift_vec<<<grid_for(n), kThreads, 0, st>>>(n, v, t, f);
  return cudaGetLastError();
}

cudaError_t step(int n, const double* S, const double* R, double tau, double* lam, double* E1, int* ibuf,
                 unsigned long long* res, int* flag, cudaStream_t st, int64_t* launches) {
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [] {
    attr = cudaFuncSetAttribute(k_cluster_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, kClusterSmem);
  });
  if (attr != cudaSuccess) return attr;
  if (n <= 0) return cudaSuccess;
  k_init<<<grid_for(n), kThreads, 0, st>>>(n, ibuf, res);
  k_lambda<<<grid_for(n), kThreads, 0, st>>>(n, S, R, lam, res, flag);
  k_pairs<<<grid_for((int64_t)n * n), kThreads, 0, st>>>(n, S, R, lam, tau, E1, ibuf, res, flag);
  k_clusters<<<1, 32, 0, st>>>(n, ibuf, flag);
  k_cluster_solve<<<(unsigned)std::max(1, std::min(n / 2, 304)), kClusterThreads, kClusterSmem, st>>>(n, S, R, ibuf,
                                                                                                      E1);
  if (launches) *launches += 5;
  return cudaGetLastError();
}

}  // namespace eigref
