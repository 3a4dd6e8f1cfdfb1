// Blocked right-looking Cholesky factorization (lower) of large dense
// symmetric matrices: the Schur complement matrix of the whole-GPU solver
// (DenseCholesky's factorize!, src/schur_solvers.jl:15-19) and its n x n
// block factorizations (src/blocks.jl:94-113, src/directions.jl:46).
//
// One launch per 32-wide block column: every thread block factors the
// 32 x 32 diagonal block in shared memory (redundantly, so no block waits on
// another), then solves its rows of the panel below against it
// (L21 = A21 L11^-T) and writes them back together with their bf16 slices;
// a second launch applies the trailing update A22 -= L21 L21' on the tensor
// cores (tcgemm.h, lower triangle only).  kFp64: FP64 diagonal blocks and
// FP64-accurate updates; kMixed: FP32 diagonal blocks and split-precision
// updates (an FP32-class factor for iterative refinement).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "tcgemm.h"

namespace chol {

struct Work {
  tcg::Sliced panel;     // slices of the panel below the diagonal block (K = 32)
  void* mem = nullptr;
  double* diag = nullptr;  // factored diagonal blocks (NB x NB per block column)
  double* dinv = nullptr;  // their inverses (the triangular solves)
  int64_t nmax = 0;
  int* err = nullptr;    // tensor-core error flag (device)
};

int64_t work_bytes(int64_t nmax);
// Bind to device memory of work_bytes(nmax) bytes.
cudaError_t init(Work* w, void* mem, int64_t nmax, int* err, cudaStream_t st);
// Lower Cholesky factor of A (n x n, leading dimension lda) in place; the
// strict upper triangle is not touched.  *info (device) becomes k + 1 for the
// first pivot k that is not positive and finite, else 0 (LAPACK potrf).
cudaError_t potrf(Work& w, int n, double* A, int64_t lda, int* info, tcg::Mode mode, cudaStream_t st,
                  int64_t* launches);
// x <- (L L')^-1 x with the factor of the last potrf of this workspace (the
// inverses of its diagonal blocks are kept); nothing is done when *info != 0.
cudaError_t solve(const Work& w, int n, const double* L, int64_t ld, double* x, const int* info, cudaStream_t st,
                  int64_t* launches);

}  // namespace chol
