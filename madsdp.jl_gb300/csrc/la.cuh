// CTA-cooperative dense linear algebra for the per-problem IPM kernel.
//
// Every routine is called by all NTHREADS threads of one CTA and ends with a
// __syncthreads(), so results are visible to the whole CTA on return.
// Matrices are column-major with leading dimension n (A(i,j) = A[i + j*n]);
// pointers may address global or shared memory (generic addressing).
// T is the compute type (double for the FP64 path, float for the FP32
// phase of the mixed path).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#ifndef NTHREADS
#define NTHREADS 128
#endif
#define NWARPS (NTHREADS / 32)

template <class T> struct Num;
template <> struct Num<double> {
  static __device__ __forceinline__ double eps() { return 2.220446049250313e-16; }
  static __device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
  static __device__ __forceinline__ double rsqrt_(double x) { return rsqrt(x); }
  static __device__ __forceinline__ bool finite(double x) { return isfinite(x); }
};
template <> struct Num<float> {
  static __device__ __forceinline__ float eps() { return 1.1920928955078125e-7f; }
  static __device__ __forceinline__ float sqrt_(float x) { return sqrtf(x); }
  static __device__ __forceinline__ float rsqrt_(float x) { return rsqrtf(x); }
  static __device__ __forceinline__ bool finite(float x) { return isfinite(x); }
};

// ---------------------------------------------------------------- reductions
template <class T> __device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
template <class T> __device__ __forceinline__ T warp_max(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Scratch for block reductions (NWARPS doubles + result).
struct RedBuf { double v[NWARPS + 1]; };

__device__ __forceinline__ double block_sum(double v, RedBuf* rb) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_sum(v);
  if (lane == 0) rb->v[warp] = v;
  __syncthreads();
  if (warp == 0) {
    double r = lane < NWARPS ? rb->v[lane] : 0.0;
    r = warp_sum(r);
    if (lane == 0) rb->v[NWARPS] = r;
  }
  __syncthreads();
  double r = rb->v[NWARPS];
  __syncthreads();
  return r;
}

__device__ __forceinline__ double block_max(double v, RedBuf* rb) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_max(v);
  if (lane == 0) rb->v[warp] = v;
  __syncthreads();
  if (warp == 0) {
    double r = lane < NWARPS ? rb->v[lane] : -INFINITY;
    r = warp_max(r);
    if (lane == 0) rb->v[NWARPS] = r;
  }
  __syncthreads();
  double r = rb->v[NWARPS];
  __syncthreads();
  return r;
}

// ---------------------------------------------------------------- elementwise
template <class T, class U>
__device__ void cta_convert(int64_t len, T* __restrict__ dst, const U* __restrict__ src) {
  for (int64_t k = threadIdx.x; k < len; k += NTHREADS) dst[k] = (T)src[k];
  __syncthreads();
}
template <class T> __device__ void cta_fill(int64_t len, T* dst, T v) {
  for (int64_t k = threadIdx.x; k < len; k += NTHREADS) dst[k] = v;
  __syncthreads();
}
// A = (A + A') / 2 in place (src/blocks.jl:77-84).  Each unordered pair is
// owned by one thread.
template <class T> __device__ void cta_symmetrize(int n, T* A) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t k = threadIdx.x; k < nn; k += NTHREADS) {
    int i = (int)(k % n), j = (int)(k / n);
    if (i > j) {
      T v = (A[i + (int64_t)j * n] + A[j + (int64_t)i * n]) / (T)2;
      A[i + (int64_t)j * n] = v;
      A[j + (int64_t)i * n] = v;
    }
  }
  __syncthreads();
}
// Upper triangle := lower triangle (after a lower-only symmetric product).
template <class T> __device__ void cta_lower_to_full(int n, T* A) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t k = threadIdx.x; k < nn; k += NTHREADS) {
    const int i = (int)(k % n), j = (int)(k / n);
    if (i < j) A[k] = A[j + (int64_t)i * n];
  }
  __syncthreads();
}
// dst = sym(src) into another buffer.
template <class T, class U> __device__ void cta_sym_copy(int n, T* dst, const U* src) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t k = threadIdx.x; k < nn; k += NTHREADS) {
    int i = (int)(k % n), j = (int)(k / n);
    dst[k] = (T)((src[i + (int64_t)j * n] + src[j + (int64_t)i * n]) / (U)2);
  }
  __syncthreads();
}
template <class T> __device__ void cta_set_identity(int n, T* A, T diag) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t k = threadIdx.x; k < nn; k += NTHREADS) A[k] = ((k % n) == (k / n)) ? diag : (T)0;
  __syncthreads();
}

// ---------------------------------------------------------------- GEMM
// C = alpha * op(A) * op(B) + beta * C for n x n matrices.  ta/tb: 0 = as
// stored, 1 = transposed.  loA/loB: the stored operand is lower triangular
// (its upper triangle is zero), which restricts the k range.  C must not
// alias A or B.  Each thread owns R x R output micro-tiles.
template <class T, int R>
__device__ void cta_gemm_r(int n, int ta, int tb, int loA, int loB, T alpha, const T* __restrict__ A,
                           const T* __restrict__ B, T beta, T* __restrict__ C, int loC = 0) {
  const int nb = (n + R - 1) / R;
  const int tiles = nb * nb;
  for (int t = threadIdx.x; t < tiles; t += NTHREADS) {
    const int i0 = (t % nb) * R, j0 = (t / nb) * R;
    if (loC && j0 > i0 + R - 1) continue;  // only tiles touching the lower triangle
    int klo = 0, khi = n;  // k in [klo, khi)
    if (loA) {
      if (!ta) khi = min(khi, i0 + R);  // A(i,k) != 0 -> k <= i
      else klo = max(klo, i0);          // A(k,i) != 0 -> k >= i
    }
    if (loB) {
      if (!tb) klo = max(klo, j0);      // B(k,j) != 0 -> k >= j
      else khi = min(khi, j0 + R);      // B(j,k) != 0 -> k <= j
    }
    T acc[R][R];
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
      for (int c = 0; c < R; ++c) acc[r][c] = (T)0;
    for (int k = klo; k < khi; ++k) {
      T a[R], b[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int i = i0 + r;
        a[r] = (i < n) ? (ta ? A[k + (int64_t)i * n] : A[i + (int64_t)k * n]) : (T)0;
      }
#pragma unroll
      for (int c = 0; c < R; ++c) {
        const int j = j0 + c;
        b[c] = (j < n) ? (tb ? B[j + (int64_t)k * n] : B[k + (int64_t)j * n]) : (T)0;
      }
#pragma unroll
      for (int r = 0; r < R; ++r)
#pragma unroll
        for (int c = 0; c < R; ++c) acc[r][c] = fma(a[r], b[c], acc[r][c]);
    }
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
      for (int c = 0; c < R; ++c) {
        const int i = i0 + r, j = j0 + c;
        if (i < n && j < n) {
          const int64_t o = i + (int64_t)j * n;
          C[o] = (beta == (T)0) ? alpha * acc[r][c] : fma(alpha, acc[r][c], beta * C[o]);
        }
      }
  }
  __syncthreads();
}

template <class T>
__device__ __forceinline__ void cta_gemm_plain(int n, int ta, int tb, int loA, int loB, T alpha, const T* A,
                                               const T* B, T beta, T* C, int loC = 0) {
  if (n <= 24) cta_gemm_r<T, 2>(n, ta, tb, loA, loB, alpha, A, B, beta, C, loC);
  else cta_gemm_r<T, 4>(n, ta, tb, loA, loB, alpha, A, B, beta, C, loC);
}

// Shared-memory scratch handed to the routines that stage operands
// (nullptr / 0 bytes: operate in global memory).
struct Scratch {
  unsigned char* p;
  int64_t bytes;
};

// GEMM whose operands are first copied into shared memory when they fit
// (operands written earlier by this CTA would otherwise be re-read from L2).
// loC = 1: only the lower triangle of C is needed (a symmetric product);
// tiles strictly above the diagonal are skipped.
template <class T>
__device__ void cta_gemm(int n, int ta, int tb, int loA, int loB, T alpha, const T* A, const T* B, T beta, T* C,
                         Scratch sc, int loC = 0) {
  const int64_t nn = (int64_t)n * n;
  const int64_t need = (A == B ? 1 : 2) * nn * (int64_t)sizeof(T);
  if (sc.p != nullptr && need <= sc.bytes) {
    T* sA = (T*)sc.p;
    T* sB = (A == B) ? sA : sA + nn;
    for (int64_t k = threadIdx.x; k < nn; k += NTHREADS) {
      sA[k] = A[k];
      if (A != B) sB[k] = B[k];
    }
    __syncthreads();
    cta_gemm_plain<T>(n, ta, tb, loA, loB, alpha, sA, sB, beta, C, loC);
  } else {
    cta_gemm_plain<T>(n, ta, tb, loA, loB, alpha, A, B, beta, C, loC);
  }
}

// ---------------------------------------------------------------- Cholesky
// In-place lower Cholesky of the n x n matrix `a` (leading dimension lda);
// only the lower triangle is read.  Returns false (on every thread) if a
// pivot is not positive and finite, as LAPACK potrf (src/blocks.jl:94-100,
// src/schur_solvers.jl:15-19).  `flag` is a shared int.
template <class T>
__device__ bool cta_potrf(int n, T* a, int lda, int* flag) {
  if (threadIdx.x == 0) *flag = 0;
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    T* colk = a + (int64_t)k * lda;
    if (threadIdx.x == 0) {
      T d = colk[k];
      if (!(d > (T)0) || !Num<T>::finite(d)) *flag = 1;
      else colk[k] = Num<T>::sqrt_(d);
    }
    __syncthreads();
    if (*flag) return false;
    const T inv = (T)1 / colk[k];
    for (int i = k + 1 + threadIdx.x; i < n; i += NTHREADS) colk[i] *= inv;
    __syncthreads();
    const int m = n - k - 1;
    const int mm = m * m;
    for (int idx = threadIdx.x; idx < mm; idx += NTHREADS) {
      const int ii = idx % m, jj = idx / m;
      if (ii >= jj) {
        const int i = k + 1 + ii, j = k + 1 + jj;
        a[i + (int64_t)j * lda] = fma(-colk[i], colk[j], a[i + (int64_t)j * lda]);
      }
    }
    __syncthreads();
  }
  return true;
}

// Zero the strict upper triangle and flush the entries below
// eps^2 * max |L_ii| (src/blocks.jl:101-111).  Works on any leading dim.
template <class T>
__device__ void cta_flush_lower(int n, T* L, int lda, RedBuf* rb) {
  double dmax = 0.0;
  for (int i = threadIdx.x; i < n; i += NTHREADS) dmax = fmax(dmax, fabs((double)L[i + (int64_t)i * lda]));
  dmax = block_max(dmax, rb);
  const T tol = (T)((double)Num<T>::eps() * (double)Num<T>::eps() * dmax);
  const int64_t nn = (int64_t)n * n;
  for (int64_t k = threadIdx.x; k < nn; k += NTHREADS) {
    const int i = (int)(k % n), j = (int)(k / n);
    T* p = L + i + (int64_t)j * lda;
    if (i < j) *p = (T)0;
    else if (i > j && fabs(*p) < tol) *p = (T)0;
  }
  __syncthreads();
}

// Inverse of a lower-triangular L (ld = n) into Li (ld = n, lower, upper
// zeroed).  One thread per column; Li may live in shared memory.
template <class T>
__device__ void cta_trtri_lower(int n, const T* __restrict__ L, T* __restrict__ Li) {
  for (int j = threadIdx.x; j < n; j += NTHREADS) {
    T* x = Li + (int64_t)j * n;
    for (int i = 0; i < j; ++i) x[i] = (T)0;
    x[j] = (T)1 / L[j + (int64_t)j * n];
    for (int i = j + 1; i < n; ++i) {
      T s = (T)0;
      for (int k = j; k < i; ++k) s = fma(L[i + (int64_t)k * n], x[k], s);
      x[i] = -s / L[i + (int64_t)i * n];
    }
  }
  __syncthreads();
}

// Solve L L' x = b in place (L lower, ld = n), b of length n.
template <class T, class V>
__device__ void cta_potrs(int n, const T* __restrict__ L, V* x) {
  // forward: L u = b (column oriented)
  for (int k = 0; k < n; ++k) {
    if (threadIdx.x == 0) x[k] = x[k] / (V)L[k + (int64_t)k * n];
    __syncthreads();
    const V xk = x[k];
    for (int i = k + 1 + threadIdx.x; i < n; i += NTHREADS) x[i] -= (V)L[i + (int64_t)k * n] * xk;
    __syncthreads();
  }
  // backward: L' x = u (row of L' = column of L: dot products)
  for (int k = n - 1; k >= 0; --k) {
    // x[k] = (x[k] - sum_{i>k} L(i,k) x[i]) / L(k,k)
    V s = 0;
    for (int i = k + 1 + threadIdx.x; i < n; i += NTHREADS) s += (V)L[i + (int64_t)k * n] * x[i];
    s = warp_sum(s);
    __shared__ V part[NWARPS];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      V t = 0;
      for (int w = 0; w < NWARPS; ++w) t += part[w];
      x[k] = (x[k] - t) / (V)L[k + (int64_t)k * n];
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- Jacobi SVD
// One-sided (Hestenes) Jacobi on the columns of M (n x n, ld n): on return
// M V has mutually orthogonal columns and sigma[k] is the norm of column k.
// The eigenvalues of M'M are sigma^2 with eigenvectors V, which is what
// LowRankOpt.eigen! returns for the NT scaling (src/directions.jl:52-58).
// Every rotation is also applied to the columns of B (n x n): B = I gives
// V itself, B = Lx gives Lx V directly.  Parallel round-robin ordering; each
// column pair is handled by a group of G lanes (G = 8, 16 or 32 by n).
// Returns false if it did not converge in max_sweeps.
template <class T, int G>
__device__ bool cta_jacobi_svd_g(int n, T* M, T* B, T* sigma, int max_sweeps, int* counter, int* sweeps_out) {
  const int lane = threadIdx.x & 31;
  const int gl = lane & (G - 1);                      // lane within its group
  const int group = threadIdx.x / G;                  // global group index
  constexpr int NG = NTHREADS / G;
  const int N = (n % 2 == 0) ? n : n + 1;
  const T tol = (T)sqrt((double)n) * Num<T>::eps();
  bool converged = (n <= 1);
  int sweep = 0;
  for (; sweep < max_sweeps && !converged; ++sweep) {
    if (threadIdx.x == 0) *counter = 0;
    __syncthreads();
    int rotated = 0, big = 0;
    const T big_tol = Num<T>::sqrt_(tol);
    for (int r = 0; r < N - 1; ++r) {
      // every group runs the same number of pair slots so shuffles stay uniform
      const int slots = (N / 2 + NG - 1) / NG;
      for (int sidx = 0; sidx < slots; ++sidx) {
        const int k = group + sidx * NG;
        int p = -1, q = -1;
        if (k < N / 2) {
          if (k == 0) { p = N - 1; q = r; }
          else { p = (r + k) % (N - 1); q = (r - k + (N - 1)) % (N - 1); }
          if (p >= n || q >= n) { p = -1; q = -1; }
        }
        T app = 0, aqq = 0, apq = 0;
        if (p >= 0) {
          const T* mp = M + (int64_t)p * n;
          const T* mq = M + (int64_t)q * n;
          for (int i = gl; i < n; i += G) {
            const T a = mp[i], b = mq[i];
            app = fma(a, a, app); aqq = fma(b, b, aqq); apq = fma(a, b, apq);
          }
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) {
          app += __shfl_xor_sync(0xffffffffu, app, o);
          aqq += __shfl_xor_sync(0xffffffffu, aqq, o);
          apq += __shfl_xor_sync(0xffffffffu, apq, o);
        }
        const T scale_pq = Num<T>::sqrt_(app) * Num<T>::sqrt_(aqq);
        if (p >= 0 && fabs(apq) > tol * scale_pq) {
          if (fabs(apq) > big_tol * scale_pq) big = 1;
          // the angle only needs float accuracy (the next sweep removes what
          // is left); c and s are formed in T so the rotation is orthogonal
          // to T's rounding
          const float zf = (float)((aqq - app) / ((T)2 * apq));
          const float tf = (zf >= 0.0f ? 1.0f : -1.0f) / (fabsf(zf) + sqrtf(1.0f + zf * zf));
          const T t = (T)tf;
          const T c = Num<T>::rsqrt_((T)1 + t * t), sn = c * t;
          T* mp = M + (int64_t)p * n;
          T* mq = M + (int64_t)q * n;
          T* bp = B + (int64_t)p * n;
          T* bq = B + (int64_t)q * n;
          for (int i = gl; i < n; i += G) {
            const T a = mp[i], b = mq[i];
            mp[i] = c * a - sn * b;
            mq[i] = sn * a + c * b;
            const T u = bp[i], v = bq[i];
            bp[i] = c * u - sn * v;
            bq[i] = sn * u + c * v;
          }
          rotated = 1;
        }
      }
      __syncthreads();
    }
    rotated = __syncthreads_or(rotated);
    big = __syncthreads_or(big);
    // quadratic convergence: after a sweep whose rotations all had
    // |a_pq| <= sqrt(tol) sqrt(a_pp a_qq), the off-diagonals are O(tol)
    converged = !rotated || !big;
  }
  *sweeps_out = sweep;
  // column norms (uniform slot count so every lane reaches every shuffle)
  const int nslots = (n + NG - 1) / NG;
  for (int sidx = 0; sidx < nslots; ++sidx) {
    const int k = group + sidx * NG;
    T s = 0;
    if (k < n) {
      const T* mk = M + (int64_t)k * n;
      for (int i = gl; i < n; i += G) s = fma(mk[i], mk[i], s);
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (k < n && gl == 0) sigma[k] = Num<T>::sqrt_(s);
  }
  __syncthreads();
  return converged;
}

template <class T>
__device__ bool cta_jacobi_svd(int n, T* M, T* B, T* sigma, int max_sweeps, int* counter, int* sweeps_out) {
  if (n <= 16) return cta_jacobi_svd_g<T, 8>(n, M, B, sigma, max_sweeps, counter, sweeps_out);
  if (n <= 48) return cta_jacobi_svd_g<T, 16>(n, M, B, sigma, max_sweeps, counter, sweeps_out);
  return cta_jacobi_svd_g<T, 32>(n, M, B, sigma, max_sweeps, counter, sweeps_out);
}

// ---------------------------------------------------------------- tridiagonal
// Number of eigenvalues of the symmetric tridiagonal (a[0..k), b[1..k))
// smaller than x (Sturm count).
template <class T>
__device__ __forceinline__ int sturm_count(int k, const T* a, const T* b, T x, T pivmin) {
  int cnt = 0;
  T d = a[0] - x;
  if (fabs(d) < pivmin) d = -pivmin;
  if (d < 0) ++cnt;
  for (int i = 1; i < k; ++i) {
    d = (a[i] - x) - b[i] * b[i] / d;
    if (fabs(d) < pivmin) d = -pivmin;
    if (d < 0) ++cnt;
  }
  return cnt;
}

// Smallest eigenvalue of the tridiagonal (a, b) by warp-parallel multisection.
// Called by one full warp; every lane returns the result.
template <class T>
__device__ T warp_tridiag_eigmin_t(int k, const T* a, const T* b);

template <class T>
__device__ __forceinline__ T warp_tridiag_eigmin(int k, const T* a, const T* b) {
  return warp_tridiag_eigmin_t<T>(k, a, b);
}

// float64: bracket the eigenvalue with float Sturm counts (cheap divisions),
// then a few float64 multisection rounds inside the bracket.
template <>
__device__ __forceinline__ double warp_tridiag_eigmin<double>(int k, const double* a, const double* b) {
  const int lane = threadIdx.x & 31;
  double scale = 0;
  for (int i = 0; i < k; ++i) scale = fmax(scale, fabs(a[i]) + (i > 0 ? fabs(b[i]) : 0.0) + (i + 1 < k ? fabs(b[i + 1]) : 0.0));
  if (!(scale > 0.0) || !isfinite(scale)) return warp_tridiag_eigmin_t<double>(k, a, b);
  // float multisection on the scaled tridiagonal (entries in [-1, 1])
  const float inv = (float)(1.0 / scale);
  float lo = -1.0f, hi = 1.0f;
  const float pivf = 1e-30f;
  for (int it = 0; it < 5; ++it) {
    const float x = lo + (hi - lo) * (float)(lane + 1) / 33.0f;
    int c = 0;
    float d = (float)a[0] * inv - x;
    if (fabsf(d) < pivf) d = -pivf;
    c += d < 0.0f;
    for (int i = 1; i < k; ++i) {
      const float bi = (float)b[i] * inv;
      d = ((float)a[i] * inv - x) - bi * bi / d;
      if (fabsf(d) < pivf) d = -pivf;
      c += d < 0.0f;
    }
    const unsigned ball = __ballot_sync(0xffffffffu, c >= 1);
    if (ball == 0) { lo = lo + (hi - lo) * 32.0f / 33.0f; continue; }
    const int first = __ffs(ball) - 1;
    const float nhi = lo + (hi - lo) * (float)(first + 1) / 33.0f;
    const float nlo = first == 0 ? lo : lo + (hi - lo) * (float)first / 33.0f;
    lo = nlo; hi = nhi;
  }
  // widen by the float rounding of the scaled problem and polish in float64
  const double w = 4e-6 * fmax(1.0, fabs((double)lo) + fabs((double)hi));
  double dlo = ((double)lo - w) * scale, dhi = ((double)hi + w) * scale;
  const double pivmin = 4.93e-32 * fmax(scale, 1e-30);
  // confirm the bracket (fall back to the full search if rounding moved it)
  const int cl = sturm_count<double>(k, a, b, dlo, pivmin);
  const int ch = sturm_count<double>(k, a, b, dhi, pivmin);
  if (cl != 0 || ch < 1) return warp_tridiag_eigmin_t<double>(k, a, b);
  for (int it = 0; it < 16; ++it) {
    if (dhi - dlo <= 2.0 * 2.220446049250313e-16 * fmax(fabs(dlo), fabs(dhi)) + pivmin) break;
    const double x = dlo + (dhi - dlo) * (double)(lane + 1) / 33.0;
    const int c = sturm_count<double>(k, a, b, x, pivmin);
    const unsigned ball = __ballot_sync(0xffffffffu, c >= 1);
    if (ball == 0) { dlo = dlo + (dhi - dlo) * 32.0 / 33.0; continue; }
    const int first = __ffs(ball) - 1;
    const double nhi = dlo + (dhi - dlo) * (double)(first + 1) / 33.0;
    const double nlo = first == 0 ? dlo : dlo + (dhi - dlo) * (double)first / 33.0;
    dlo = nlo; dhi = nhi;
  }
  return (dlo + dhi) / 2;
}

template <class T>
__device__ T warp_tridiag_eigmin_t(int k, const T* a, const T* b) {
  const int lane = threadIdx.x & 31;
  T lo = 0, hi = 0, scale = 0;
  // Gershgorin interval
  for (int i = 0; i < k; ++i) {
    const T r = (i > 0 ? fabs(b[i]) : (T)0) + (i + 1 < k ? fabs(b[i + 1]) : (T)0);
    const T l = a[i] - r, h = a[i] + r;
    if (i == 0 || l < lo) lo = l;
    if (i == 0 || h > hi) hi = h;
    scale = fmax(scale, fmax(fabs(l), fabs(h)));
  }
  const T pivmin = (T)(Num<T>::eps() * Num<T>::eps()) * fmax(scale, (T)1e-30);
  for (int it = 0; it < 64; ++it) {
    if (hi - lo <= (T)2 * Num<T>::eps() * fmax(fabs(lo), fabs(hi)) + pivmin) break;
    const T x = lo + (hi - lo) * (T)(lane + 1) / (T)33;
    const int c = sturm_count(k, a, b, x, pivmin);
    const unsigned ball = __ballot_sync(0xffffffffu, c >= 1);
    if (ball == 0) { lo = lo + (hi - lo) * (T)32 / (T)33; continue; }
    const int first = __ffs(ball) - 1;  // smallest lane with count >= 1
    const T nhi = lo + (hi - lo) * (T)(first + 1) / (T)33;
    const T nlo = first == 0 ? lo : lo + (hi - lo) * (T)first / (T)33;
    lo = nlo; hi = nhi;
  }
  return (lo + hi) / (T)2;
}

// The j-th smallest eigenvalue (0-based) of the tridiagonal by bisection,
// computed by one thread.
template <class T>
__device__ T thread_tridiag_eig(int k, const T* a, const T* b, int j) {
  T lo = 0, hi = 0, scale = 0;
  for (int i = 0; i < k; ++i) {
    const T r = (i > 0 ? fabs(b[i]) : (T)0) + (i + 1 < k ? fabs(b[i + 1]) : (T)0);
    const T l = a[i] - r, h = a[i] + r;
    if (i == 0 || l < lo) lo = l;
    if (i == 0 || h > hi) hi = h;
    scale = fmax(scale, fmax(fabs(l), fabs(h)));
  }
  const T pivmin = (T)(Num<T>::eps() * Num<T>::eps()) * fmax(scale, (T)1e-30);
  for (int it = 0; it < 200; ++it) {
    if (hi - lo <= (T)2 * Num<T>::eps() * fmax(fabs(lo), fabs(hi)) + pivmin) break;
    const T x = (lo + hi) / (T)2;
    if (sturm_count(k, a, b, x, pivmin) >= j + 1) hi = x;
    else lo = x;
  }
  return (lo + hi) / (T)2;
}

// ---------------------------------------------------------------- warp routines
// Smallest eigenvalue of the symmetric Z (n x n) by Lanczos with full
// reorthogonalization, run by ONE warp (the role of
// LowRankOpt.lanczos_eigmin!, src/step.jl:151-183).  Q (n x n) holds the
// basis; a, bb, coef are vectors of length n+1, w of length n.  Stops when
// the smallest Ritz value is stable to 64 eps or the Krylov space is
// exhausted (k = n or b_k ~ 0).
template <class T>
__device__ T warp_lanczos_eigmin(int n, const T* Z, T* Qs, int kq, T* Qg, T* a, T* bb, T* w, T* coef, int* steps) {
  const int lane = threadIdx.x & 31;
  // column l of the basis: shared memory for l < kq, global memory after
  auto Qc = [&](int l) -> T* { return l < kq ? Qs + (int64_t)l * n : Qg + (int64_t)l * n; };
  T* Q = Qc(0);
  T nrm2 = 0;
  for (int i = lane; i < n; i += 32) {
    uint32_t h = (uint32_t)(i + 1) * 2654435761u;
    h ^= h >> 15; h *= 2246822519u; h ^= h >> 13;
    const T v = (T)((double)(h & 0xffffff) / 16777216.0 - 0.5) + (T)0.01;
    Q[i] = v;
    nrm2 = fma(v, v, nrm2);
  }
  nrm2 = warp_sum(nrm2);
  {
    const T inv = (T)1 / Num<T>::sqrt_(nrm2);
    for (int i = lane; i < n; i += 32) Q[i] *= inv;
  }
  __syncwarp();
  T theta = 0, theta_prev = (T)INFINITY, znorm = 0;
  int k = 0;
  for (int j = 0; j < n; ++j) {
    const T* qj = Qc(j);
    // w = Z q_j (Z symmetric; lanes read consecutive rows of each column)
    T wl[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) wl[t] = 0;
    for (int r = 0; r < n; ++r) {
      const T qr = qj[r];
      const T* zr = Z + (int64_t)r * n;
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const int i = lane + 32 * t;
        if (i < n) wl[t] = fma(zr[i], qr, wl[t]);
      }
    }
    T aj = 0;
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const int i = lane + 32 * t;
      if (i < n) aj = fma(qj[i], wl[t], aj);
    }
    aj = warp_sum(aj);
    const T bj = j > 0 ? bb[j] : (T)0;
    const T* qp = j > 0 ? Qc(j - 1) : qj;
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const int i = lane + 32 * t;
      if (i < n) {
        T v = wl[t] - aj * qj[i];
        if (j > 0) v -= bj * qp[i];
        wl[t] = v;
        w[i] = v;
      }
    }
    if (lane == 0) a[j] = aj;
    __syncwarp();
    // full reorthogonalization, twice: coef_l = Q_l . w (one lane per l)
    for (int pass = 0; pass < 2; ++pass) {
      for (int l = lane; l <= j; l += 32) {
        const T* ql = Qc(l);
        T s = 0;
        for (int i = 0; i < n; ++i) s = fma(ql[i], w[i], s);
        coef[l] = s;
      }
      __syncwarp();
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const int i = lane + 32 * t;
        if (i < n) {
          T v = wl[t];
          for (int l = 0; l <= j; ++l) v = fma(-coef[l], Qc(l)[i], v);
          wl[t] = v;
        }
      }
      __syncwarp();
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const int i = lane + 32 * t;
        if (i < n) w[i] = wl[t];
      }
      __syncwarp();
    }
    T bn = 0;
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const int i = lane + 32 * t;
      if (i < n) bn = fma(wl[t], wl[t], bn);
    }
    bn = Num<T>::sqrt_(warp_sum(bn));
    k = j + 1;
    znorm = fmax(znorm, fabs(aj) + bn + fabs(bj));
    if (lane == 0) bb[j + 1] = bn;
    __syncwarp();
    const bool exhausted = (k == n) || !(bn > Num<T>::eps() * znorm * (T)4);
    if (exhausted || (k >= 4 && (k % 4) == 0)) {
      theta = warp_tridiag_eigmin<T>(k, a, bb);
      const T tolr = Num<T>::eps() * (T)64 * fmax((T)1, fabs(theta));
      if (exhausted || fabs(theta - theta_prev) <= tolr) break;
      theta_prev = theta;
    }
    T* qn = Qc(j + 1);
    const T inv = (T)1 / bn;
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const int i = lane + 32 * t;
      if (i < n) qn[i] = wl[t] * inv;
    }
    __syncwarp();
  }
  *steps = k;
  return theta;
}

// Solve L L' x = b in place (L lower, ld m) by ONE warp; x (and L, when
// the caller staged it) in shared memory.
template <class T, class V>
__device__ void warp_potrs(int m, const T* __restrict__ L, V* x, V* rdiag) {
  const int lane = threadIdx.x & 31;
  // reciprocal diagonal once (lanes in parallel) instead of a division per row
  for (int k = lane; k < m; k += 32) rdiag[k] = (V)1 / (V)L[k + (int64_t)k * m];
  __syncwarp();
  for (int k = 0; k < m; ++k) {
    const V xk = x[k] * rdiag[k];
    __syncwarp();
    if (lane == 0) x[k] = xk;
    const T* lk = L + (int64_t)k * m;
    for (int i = k + 1 + lane; i < m; i += 32) x[i] -= (V)lk[i] * xk;
    __syncwarp();
  }
  for (int k = m - 1; k >= 0; --k) {
    const T* lk = L + (int64_t)k * m;
    V s = 0;
    for (int i = k + 1 + lane; i < m; i += 32) s += (V)lk[i] * x[i];
    s = warp_sum(s);
    if (lane == 0) x[k] = (x[k] - s) * rdiag[k];
    __syncwarp();
  }
}

// Full Lanczos tridiagonalization of the symmetric Z (n x n) by ONE warp:
// n steps with full reorthogonalization; when the Krylov space closes early
// (b ~ 0) it restarts from a new vector orthogonal to the basis (b = 0 in
// T), so T (a[0..n), bb[1..n)) has exactly the eigenvalues of Z.
template <class T>
__device__ void warp_lanczos_full(int n, const T* Z, T* Q, T* a, T* bb, T* w, T* coef) {
  const int lane = threadIdx.x & 31;
  auto start_vector = [&](int j, uint32_t seed) {
    T* q = Q + (int64_t)j * n;
    for (int i = lane; i < n; i += 32) {
      uint32_t h = (uint32_t)(i + 1) * 2654435761u + seed * 40503u;
      h ^= h >> 15; h *= 2246822519u; h ^= h >> 13;
      q[i] = (T)((double)(h & 0xffffff) / 16777216.0 - 0.5) + (T)0.01;
    }
    __syncwarp();
    // orthogonalize twice against the previous columns, then normalize
    for (int pass = 0; pass < 2; ++pass) {
      for (int l = lane; l < j; l += 32) {
        const T* ql = Q + (int64_t)l * n;
        T s = 0;
        for (int i = 0; i < n; ++i) s = fma(ql[i], q[i], s);
        coef[l] = s;
      }
      __syncwarp();
      for (int i = lane; i < n; i += 32) {
        T v = q[i];
        for (int l = 0; l < j; ++l) v = fma(-coef[l], Q[i + (int64_t)l * n], v);
        q[i] = v;
      }
      __syncwarp();
    }
    T nrm = 0;
    for (int i = lane; i < n; i += 32) nrm = fma(q[i], q[i], nrm);
    nrm = Num<T>::sqrt_(warp_sum(nrm));
    const T inv = nrm > (T)0 ? (T)1 / nrm : (T)0;
    for (int i = lane; i < n; i += 32) q[i] *= inv;
    __syncwarp();
  };
  start_vector(0, 1u);
  T znorm = 0;
  for (int j = 0; j < n; ++j) {
    const T* qj = Q + (int64_t)j * n;
    for (int i = lane; i < n; i += 32) {
      T s = 0;
      for (int r = 0; r < n; ++r) s = fma(Z[i + (int64_t)r * n], qj[r], s);
      w[i] = s;
    }
    __syncwarp();
    T aj = 0;
    for (int i = lane; i < n; i += 32) aj = fma(qj[i], w[i], aj);
    aj = warp_sum(aj);
    const T bj = j > 0 ? bb[j] : (T)0;
    const T* qp = j > 0 ? Q + (int64_t)(j - 1) * n : qj;
    for (int i = lane; i < n; i += 32) {
      T v = w[i] - aj * qj[i];
      if (j > 0) v -= bj * qp[i];
      w[i] = v;
    }
    if (lane == 0) a[j] = aj;
    __syncwarp();
    for (int pass = 0; pass < 2; ++pass) {
      for (int l = lane; l <= j; l += 32) {
        const T* ql = Q + (int64_t)l * n;
        T s = 0;
        for (int i = 0; i < n; ++i) s = fma(ql[i], w[i], s);
        coef[l] = s;
      }
      __syncwarp();
      for (int i = lane; i < n; i += 32) {
        T v = w[i];
        for (int l = 0; l <= j; ++l) v = fma(-coef[l], Q[i + (int64_t)l * n], v);
        w[i] = v;
      }
      __syncwarp();
    }
    if (j + 1 == n) break;
    T bn = 0;
    for (int i = lane; i < n; i += 32) bn = fma(w[i], w[i], bn);
    bn = Num<T>::sqrt_(warp_sum(bn));
    znorm = fmax(znorm, fabs(aj) + bn + fabs(bj));
    T* qn = Q + (int64_t)(j + 1) * n;
    if (bn > Num<T>::eps() * fmax(znorm, (T)1e-300) * (T)4) {
      const T inv = (T)1 / bn;
      for (int i = lane; i < n; i += 32) qn[i] = w[i] * inv;
      if (lane == 0) bb[j + 1] = bn;
      __syncwarp();
    } else {
      if (lane == 0) bb[j + 1] = (T)0;
      __syncwarp();
      start_vector(j + 1, (uint32_t)(j + 2));
    }
  }
}

// ---------------------------------------------------------------- Bunch-Kaufman
// Symmetric indefinite factorization A = P L D L' P' with 1x1 and 2x2
// pivots (Bunch-Kaufman partial pivoting, the LAPACK sytf2 "lower"
// algorithm), in place on the lower triangle of the m x m matrix `a`
// (leading dimension lda).  piv[k] = kp for a 1x1 pivot (rows k and kp
// swapped); piv[k] = piv[k+1] = -(kp + 1) for a 2x2 pivot whose second row
// was swapped with kp.  Returns false when a pivot column is exactly zero
// (singular).  `work` holds 2m scratch values.
template <class T>
__device__ bool cta_sytrf_lower(int m, T* a, int lda, double* piv, T* work, RedBuf* rb, int* flag) {
  const T alpha = (T)((1.0 + sqrt(17.0)) / 8.0);
  auto A = [&](int i, int j) -> T& { return a[i + (int64_t)j * lda]; };
  int k = 0;
  while (k < m) {
    // colmax and its row (smallest index on ties)
    double cm = -1.0;
    int ci = m;
    for (int i = k + 1 + threadIdx.x; i < m; i += NTHREADS) {
      const double v = fabs((double)A(i, k));
      if (v > cm) { cm = v; ci = i; }
    }
    // block argmax: encode (value, -index) through two reductions
    const double colmax_all = block_max(cm, rb);
    int cand = (cm == colmax_all && cm >= 0.0) ? ci : m;
    // smallest index attaining the max
    if (threadIdx.x == 0) *flag = m;
    __syncthreads();
    if (cand < m) atomicMin(flag, cand);
    __syncthreads();
    const int imax = *flag;
    __syncthreads();
    const double colmax = (k + 1 < m) ? fmax(colmax_all, 0.0) : 0.0;
    const double absakk = fabs((double)A(k, k));
    if (!(fmax(absakk, colmax) > 0.0)) return false;  // zero column (or NaN): singular
    int kp = k, kstep = 1;
    if (!(absakk >= (double)alpha * colmax)) {
      // rowmax: largest off-diagonal magnitude in row/column imax of the trailing matrix
      double rm = 0.0;
      for (int j = k + threadIdx.x; j < m; j += NTHREADS) {
        if (j == imax) continue;
        const double v = j < imax ? fabs((double)A(imax, j)) : fabs((double)A(j, imax));
        rm = fmax(rm, v);
      }
      const double rowmax = block_max(rm, rb);
      if (absakk >= (double)alpha * colmax * (colmax / rowmax)) kp = k;
      else if (fabs((double)A(imax, imax)) >= (double)alpha * rowmax) kp = imax;
      else { kp = imax; kstep = 2; }
    }
    const int kk = k + kstep - 1;
    if (kp != kk) {
      // symmetric interchange of rows/columns kk and kp in the trailing matrix
      for (int i = kp + 1 + threadIdx.x; i < m; i += NTHREADS) {
        const T t = A(i, kk); A(i, kk) = A(i, kp); A(i, kp) = t;
      }
      for (int j = kk + 1 + threadIdx.x; j < kp; j += NTHREADS) {
        const T t = A(j, kk); A(j, kk) = A(kp, j); A(kp, j) = t;
      }
      if (threadIdx.x == 0) {
        const T t = A(kk, kk); A(kk, kk) = A(kp, kp); A(kp, kp) = t;
        if (kstep == 2) { const T u = A(k + 1, k); A(k + 1, k) = A(kp, k); A(kp, k) = u; }
      }
      __syncthreads();
    }
    if (kstep == 1) {
      const T r1 = (T)1 / A(k, k);
      const int r = m - k - 1;
      const int rr = r * r;
      for (int idx = threadIdx.x; idx < rr; idx += NTHREADS) {
        const int ii = idx % r, jj = idx / r;
        if (ii >= jj) {
          const int i = k + 1 + ii, j = k + 1 + jj;
          A(i, j) -= r1 * A(i, k) * A(j, k);
        }
      }
      __syncthreads();
      for (int i = k + 1 + threadIdx.x; i < m; i += NTHREADS) A(i, k) *= r1;
      if (threadIdx.x == 0) piv[k] = (double)kp;
      __syncthreads();
    } else {
      if (k + 2 < m) {
        T d21 = A(k + 1, k);
        const T d11 = A(k + 1, k + 1) / d21, d22 = A(k, k) / d21;
        const T t = (T)1 / (d11 * d22 - (T)1);
        d21 = t / d21;
        T* wk = work;
        T* wk1 = work + m;
        for (int j = k + 2 + threadIdx.x; j < m; j += NTHREADS) {
          wk[j] = d21 * (d11 * A(j, k) - A(j, k + 1));
          wk1[j] = d21 * (d22 * A(j, k + 1) - A(j, k));
        }
        __syncthreads();
        const int r = m - k - 2;
        const int rr = r * r;
        for (int idx = threadIdx.x; idx < rr; idx += NTHREADS) {
          const int ii = idx % r, jj = idx / r;
          if (ii >= jj) {
            const int i = k + 2 + ii, j = k + 2 + jj;
            A(i, j) -= A(i, k) * wk[j] + A(i, k + 1) * wk1[j];
          }
        }
        __syncthreads();
        for (int j = k + 2 + threadIdx.x; j < m; j += NTHREADS) { A(j, k) = wk[j]; A(j, k + 1) = wk1[j]; }
      }
      if (threadIdx.x == 0) { piv[k] = (double)(-(kp + 1)); piv[k + 1] = (double)(-(kp + 1)); }
      __syncthreads();
    }
    k += kstep;
  }
  return true;
}

// Solve with the factorization of cta_sytrf_lower (the LAPACK sytrs
// "lower" algorithm), one warp, x in place.
template <class T, class V>
__device__ void warp_sytrs_lower(int m, const T* a, int lda, const double* piv, V* x) {
  const int lane = threadIdx.x & 31;
  auto A = [&](int i, int j) -> V { return (V)a[i + (int64_t)j * lda]; };
  int k = 0;
  while (k < m) {
    if (piv[k] >= 0.0) {
      const int kp = (int)piv[k];
      if (lane == 0 && kp != k) { const V t = x[k]; x[k] = x[kp]; x[kp] = t; }
      __syncwarp();
      const V xk = x[k];
      for (int i = k + 1 + lane; i < m; i += 32) x[i] -= A(i, k) * xk;
      __syncwarp();
      if (lane == 0) x[k] = xk / A(k, k);
      __syncwarp();
      k += 1;
    } else {
      const int kp = (int)(-piv[k]) - 1;
      if (lane == 0 && kp != k + 1) { const V t = x[k + 1]; x[k + 1] = x[kp]; x[kp] = t; }
      __syncwarp();
      const V xk = x[k], xk1 = x[k + 1];
      for (int i = k + 2 + lane; i < m; i += 32) x[i] -= A(i, k) * xk + A(i, k + 1) * xk1;
      __syncwarp();
      if (lane == 0) {
        const V akm1k = A(k + 1, k);
        const V akm1 = A(k, k) / akm1k, ak = A(k + 1, k + 1) / akm1k;
        const V denom = akm1 * ak - (V)1;
        const V bkm1 = xk / akm1k, bk = xk1 / akm1k;
        x[k] = (ak * bkm1 - bk) / denom;
        x[k + 1] = (akm1 * bk - bkm1) / denom;
      }
      __syncwarp();
      k += 2;
    }
  }
  k = m - 1;
  while (k >= 0) {
    if (piv[k] >= 0.0) {
      V s = 0;
      for (int i = k + 1 + lane; i < m; i += 32) s += A(i, k) * x[i];
      s = warp_sum(s);
      if (lane == 0) {
        x[k] -= s;
        const int kp = (int)piv[k];
        if (kp != k) { const V t = x[k]; x[k] = x[kp]; x[kp] = t; }
      }
      __syncwarp();
      k -= 1;
    } else {
      V s = 0, s1 = 0;
      for (int i = k + 1 + lane; i < m; i += 32) { s += A(i, k) * x[i]; s1 += A(i, k - 1) * x[i]; }
      s = warp_sum(s);
      s1 = warp_sum(s1);
      if (lane == 0) {
        x[k] -= s;
        x[k - 1] -= s1;
        const int kp = (int)(-piv[k]) - 1;
        if (kp != k) { const V t = x[k]; x[k] = x[kp]; x[kp] = t; }
      }
      __syncwarp();
      k -= 2;
    }
  }
}
