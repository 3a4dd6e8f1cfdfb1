// Split-precision products on the 5th-generation tensor cores (tcgen05).
//
// C = alpha * op(A) op(B) + beta * C for float64 A, B, C, computed from
// bf16 slices of the operands (the Ozaki splitting):
//   - every row r of an operand gets a power-of-two exponent e_r with
//     max_k |x_rk| < 2^e_r; x_rk 2^-e_r in (-1, 1) is cut by rounding into
//     slices q_t 2^-(8t+7), t = 0..ns-1, with integers |q_t| <= 128, so each
//     slice is exact in bf16;
//   - the slice products q_t q_u (t + u <= ns - 1) are summed on the tensor
//     cores (kind::f16, bf16 inputs, FP32 accumulation in tensor memory);
//   - products of the same order t + u = s are accumulated together, and an
//     order's partial sum over a chunk of K is an integer below 2^24, so it
//     is exact in FP32 whatever rounding the tensor core's accumulator
//     applies (on GB300 it truncates: a sum that is not exact drifts by up
//     to one unit in the last place per MMA); each chunk's order sums are
//     converted to a 64-bit fixed-point integer, so chunks add exactly
//     (integer atomics for split K) and the result does not depend on the
//     order of the chunks;
//   - the highest orders share one inexact FP32 accumulator whose magnitude
//     is small enough that its truncation stays below the target accuracy.
//
// Two accuracies:
//   kMixed  3 slices, 6 products; order 0 exact per chunk of 1024, orders
//           1-2 in one accumulator: about FP32 accuracy (the split-precision
//           Schur assembly of the mixed whole-GPU path); 128 x 128 tiles;
//   kFp64   7 slices, 28 products; orders 0, 1, 2 and 3 exact per chunk of
//           256, orders 4-6 in one accumulator: relative error about 5e-15
//           of |A||B| (the FP64 path's products); 128 x 64 tiles, so the
//           five accumulators fit the 512 columns of tensor memory.
//
// Operands reach shared memory by TMA (cp.async.bulk.tensor, 64-byte
// swizzle, one 128 x 32 bf16 box per slice and stage), the MMA is issued by
// one thread, accumulators live in tensor memory and the epilogue reads them
// with tcgen05.ld.  Every wait is bounded; a wait that runs out sets the
// caller's error flag and the kernel returns after freeing its tensor
// memory.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace tcg {

enum Mode { kMixed = 0, kFp64 = 1 };
int slices_of(Mode m);

// Element (R, k) of a K-major operand: R = j * nr + i (j = batch, i < nr),
// x = p[j*bs + i*rs + k*ks].  With kmap (symmetric-vector form of n x n
// blocks), k -> (a, b) with a >= b and x = p[j*bs + a*rs + b*ks] * (a == b ? 1 : sqrt 2).
struct Source {
  const double* p = nullptr;
  int64_t rows = 0, K = 0;
  int64_t nr = 1;
  int64_t bs = 0, rs = 0, ks = 0;
  const int2* kmap = nullptr;
};

// bf16 slices [ns][Rpad][Kpad] and the row exponents [Rpad].
struct Sliced {
  __nv_bfloat16* s = nullptr;
  int32_t* ex = nullptr;
  int64_t rows = 0, Rpad = 0, K = 0, Kpad = 0;
  int ns = 0;
  CUtensorMap map;    // boxes of 128 rows (A operand, 128-column B tiles)
  CUtensorMap map64;  // boxes of 64 rows (64-column B tiles)
};

int64_t sliced_bytes(int64_t rows, int64_t K, int ns);
// Bind to device memory of sliced_bytes() bytes and encode the tensor maps.
// `zero` clears the memory first; the slicer itself writes every padded
// entry, so a rebinding to a new shape before slicing needs no clearing.
cudaError_t sliced_init(Sliced* s, void* mem, int64_t rows, int64_t K, int ns, cudaStream_t st, bool zero = true);
// Slice an operand (two launches).
cudaError_t slice(const Source& src, Sliced* dst, cudaStream_t st);

struct Out {
  double* C = nullptr;
  int64_t ldc = 0;
  double alpha = 1.0, beta = 0.0;  // beta 0 or 1 with one K chunk and alpha = +-2^p: written in the epilogue
  bool lower = false;           // only entries with row >= col (tiles below the diagonal)
  long long* fix = nullptr;     // M x N int64 workspace (split K or general alpha/beta)
  int64_t ldfix = 0;
  int* err = nullptr;           // device flag: nonzero when a bounded wait ran out
};
int64_t fix_bytes(int64_t M, int64_t N);
// True when this product needs the fixed-point workspace.
bool needs_fix(const Sliced& A, const Sliced& B, Mode mode, const Out& o);
// C = alpha * A B^T (+ beta C): A and B are K-major slices (rows of A = rows
// of C, rows of B = columns of C).  `launches` counts the kernels issued.
cudaError_t gemm(const Sliced& A, const Sliced& B, Mode mode, const Out& o, cudaStream_t st, int64_t* launches);

// ---- device helpers shared by kernels that write slices themselves
constexpr int kZeroExp = -1100;  // row exponent of an all-zero row

// exponent field of a double
__device__ __forceinline__ int exp_field(double x) { return (int)((__double_as_longlong(x) >> 52) & 0x7FF); }
// row exponent e with max |x| < 2^e from the largest exponent field
__device__ __forceinline__ int row_exp(int max_field) { return max_field == 0 ? kZeroExp : max_field - 1022; }

// x 2^(62 - e) as an integer (|x| < 2^e); zero and subnormal inputs give 0.
__device__ __forceinline__ long long to_fixed(double x, int e) {
  const long long b = __double_as_longlong(x);
  const int exf = (int)((b >> 52) & 0x7FF);
  if (exf == 0) return 0;
  const long long mant = (b & 0xFFFFFFFFFFFFFll) | (1ll << 52);
  const int sh = exf - 1075 + 62 - e;
  long long v = 0;
  if (sh >= 0) v = mant << min(sh, 9);
  else if (sh > -63) v = mant >> (-sh);
  return b < 0 ? -v : v;
}

// Cut x (row exponent e) into NS slices q_t 2^-8t (bf16) and store them
// at out[t * slice_stride].
template <int NS>
__device__ __forceinline__ void write_slices(double x, int e, __nv_bfloat16* out, int64_t slice_stride) {
  long long r = to_fixed(x, e);
#pragma unroll
  for (int t = 0; t < NS; ++t) {
    const int sft = 55 - 8 * t;
    const long long q = (r + (1ll << (sft - 1))) >> sft;
    r -= q * (1ll << sft);
    out[t * slice_stride] = __float2bfloat16_rn((float)q * __int_as_float((127 - 8 * t) << 23));
  }
}

}  // namespace tcg
