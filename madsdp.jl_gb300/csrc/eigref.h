// Refinement of an approximate symmetric eigendecomposition to FP64
// accuracy (the elementwise and cluster parts; the products are the
// caller's FP64 tensor-core products).
//
// One step, after Ogita and Aishima, "Iterative refinement for symmetric
// eigenvalue decomposition", Japan J. Indust. Appl. Math. 35 (2018): for
// an approximate eigenvector basis V of the symmetric N, with
// S = V'NV and R = V'V (so R~ = I - R),
//   lam_i = S_ii / R_ii,
//   e_ii  = R~_ii / 2,
//   e_ij  = (S_ij + lam_j R~_ij) / (lam_j - lam_i)      (i != j),
// and V (I + E) is the next basis: first order in the error of V, so the
// error is squared by each step.  A pair whose e_ij would exceed `tau`
// (eigenvalues too close for the first-order formula) is "coupled"; the
// coupled pairs define clusters, index ranges [a, a+k) covering every
// coupled pair; a pair whose residual S_ij + lam_j R~_ij is already at
// rounding level of max |lam| is never coupled (e_ij = R~_ij / 2, as for
// exactly repeated eigenvalues).  Inside a cluster E is the first-order orthonormalization
// O = I + R~_cc/2 alone, and the cluster's columns of I + E are then
// multiplied by the rotation Q that diagonalizes O S_cc O (cyclic Jacobi
// in one thread block, FP64), so the first-order terms between the cluster
// and the other vectors turn with it.  A cluster above kMaxCluster sets
// *flag (the caller then uses a dense eigensolver).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace eigref {

constexpr int kMaxCluster = 64;

// ints of the step's index workspace for order n
inline int64_t ibuf_ints(int n) { return 3 * (int64_t)n + 8; }

cudaError_t to_float(int64_t count, const double* src, float* dst, cudaStream_t st);
cudaError_t to_double(int64_t count, const float* src, double* dst, cudaStream_t st);
// A_ii += f * (*t) for the n x n column-major A; v_i += f * (*t)
// (shifting by the mean eigenvalue trace/n, a device scalar: the FP32
// eigensolver's absolute accuracy then scales with the spread of the
// spectrum rather than its magnitude, and the eigenvectors are the same)
cudaError_t shift_diag(int n, double* A, const double* t, double f, cudaStream_t st);
cudaError_t shift_vec(int n, double* v, const double* t, double f, cudaStream_t st);

// S (n x n, column-major, lower triangle read), R = V'V (lower triangle
// read).  Writes lam (n), E1 = I + E (n x n, full), uses ibuf, and sets
// the residual measures of the basis V (bits of non-negative doubles, which
// order like the values): res[0] = max_{i != j} |S_ij + lam_j R~_ij|,
// res[1] = max |R~_ij|, res[2] = max |lam_i|; *flag = 1 if a cluster is
// larger than kMaxCluster or a value is not finite.  V is accurate when
// max(res[0] / res[2], res[1]) is at rounding level.
cudaError_t step(int n, const double* S, const double* R, double tau, double* lam, double* E1, int* ibuf,
                 unsigned long long* res, int* flag, cudaStream_t st, int64_t* launches);

}  // namespace eigref
