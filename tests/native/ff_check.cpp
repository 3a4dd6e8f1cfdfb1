// CPU test harness of the float-float arithmetic (csrc/ff.cuh): element-wise
// operations, the error-free transformations, a dot product and a
// Cholesky factorization carried out in float-float.
#include <cstdint>

#include "../../madsdp.jl_gb300/csrc/ff.cuh"

extern "C" {

// 1 where hi + lo equals the exact sum (op 0) or product (op 1) of the
// FP32 inputs (both exact in float64 for these operations)
void ff_eft_check(int op, int64_t n, const float* a, const float* b, int32_t* ok) {
  for (int64_t i = 0; i < n; ++i) {
    const ff r = op == 0 ? ff_two_sum(a[i], b[i]) : ff_two_prod(a[i], b[i]);
    const double exact = op == 0 ? (double)a[i] + (double)b[i] : (double)a[i] * (double)b[i];
    ok[i] = ((double)r.hi + (double)r.lo) == exact;
  }
}

// op: 0 add, 1 sub, 2 mul, 3 div, 4 sqrt(a), 5 fma (a * b + a); inputs are
// rounded to float-float first (ain / bin return those values)
void ff_elementwise(int op, int64_t n, const double* a, const double* b, double* ain, double* bin, double* out) {
  for (int64_t i = 0; i < n; ++i) {
    const ff x = ff_from_double(a[i]), y = ff_from_double(b[i]);
    ain[i] = ff_to_double(x);
    bin[i] = ff_to_double(y);
    ff r{};
    switch (op) {
      case 0: r = ff_add(x, y); break;
      case 1: r = ff_sub(x, y); break;
      case 2: r = ff_mul(x, y); break;
      case 3: r = ff_div(x, y); break;
      case 4: r = ff_sqrt(x); break;
      default: r = ff_fma(x, y, x); break;
    }
    out[i] = ff_to_double(r);
  }
}

double ff_dot(int64_t n, const double* x, const double* y) {
  ff s = ff_from(0.0f);
  for (int64_t i = 0; i < n; ++i) s = ff_fma(ff_from_double(x[i]), ff_from_double(y[i]), s);
  return ff_to_double(s);
}

// Lower Cholesky factor of the column-major n x n A in float-float
// (left-looking); returns 0 at a non-positive pivot.
int ff_cholesky(int n, const double* A, double* L) {
  ff* l = new ff[(size_t)n * n];
  int ok = 1;
  for (int j = 0; j < n && ok; ++j) {
    ff d = ff_from_double(A[(size_t)j + (size_t)j * n]);
    for (int p = 0; p < j; ++p) d = ff_sub(d, ff_mul(l[j + (size_t)p * n], l[j + (size_t)p * n]));
    if (!(d.hi > 0.0f)) {
      ok = 0;
      break;
    }
    const ff djj = ff_sqrt(d);
    l[j + (size_t)j * n] = djj;
    for (int i = j + 1; i < n; ++i) {
      ff s = ff_from_double(A[(size_t)i + (size_t)j * n]);
      for (int p = 0; p < j; ++p) s = ff_sub(s, ff_mul(l[i + (size_t)p * n], l[j + (size_t)p * n]));
      l[i + (size_t)j * n] = ff_div(s, djj);
    }
  }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) L[(size_t)i + (size_t)j * n] = i >= j && ok ? ff_to_double(l[i + (size_t)j * n]) : 0.0;
  delete[] l;
  return ok;
}

}  // extern "C"

extern "C" {

// the operators on pairs (a_i, b_i): out[6 i + k] for k = + - * / sqrt(|a|) fabs(a);
// cmp[4 i + k] for k = < > <= ==
void ff_operators(int64_t n, const double* a, const double* b, double* out, int32_t* cmp) {
  for (int64_t i = 0; i < n; ++i) {
    const ff x = ff_from_double(a[i]), y = ff_from_double(b[i]);
    out[6 * i + 0] = ff_to_double(x + y);
    out[6 * i + 1] = ff_to_double(x - y);
    out[6 * i + 2] = ff_to_double(x * y);
    out[6 * i + 3] = ff_to_double(x / y);
    out[6 * i + 4] = ff_to_double(sqrt(fabs(x)));
    out[6 * i + 5] = ff_to_double(fabs(x));
    ff z = x;
    z += y;
    z -= y;  // x + y - y, to check the compound forms run the same code
    (void)z;
    cmp[4 * i + 0] = x < y;
    cmp[4 * i + 1] = x > y;
    cmp[4 * i + 2] = x <= y;
    cmp[4 * i + 3] = x == y;
  }
}

}  // extern "C"

extern "C" {

// conversions: ff(double), ff(int), (ff)0 and fma(a, b, c) against the named functions
int ff_constructors(int64_t n, const double* a, const double* b, const double* c) {
  for (int64_t i = 0; i < n; ++i) {
    const ff x(a[i]), y(b[i]), z(c[i]);
    const ff f = ff_from_double(a[i]);
    if (x.hi != f.hi || x.lo != f.lo) return 1;
    const ff r = fma(x, y, z), q = ff_fma(x, y, z);
    if (r.hi != q.hi || r.lo != q.lo) return 2;
  }
  const ff zero = (ff)0, one = (ff)1, big(123456789);
  if (zero.hi != 0.0f || zero.lo != 0.0f || one.hi != 1.0f || one.lo != 0.0f) return 3;
  if (ff_to_double(big) != 123456789.0) return 4;  // 27 bits: exact in float-float
  ff v{};
  if (v.hi != 0.0f || v.lo != 0.0f) return 5;  // value-initialized
  return 0;
}

}  // extern "C"

extern "C" {
// double -> float-float -> double through the constructor and ff_from_double
void ff_roundtrip(int64_t n, const double* in, double* out_ctor, double* out_from) {
  for (int64_t i = 0; i < n; ++i) {
    out_ctor[i] = ff_to_double(ff(in[i]));
    out_from[i] = ff_to_double(ff_from_double(in[i]));
  }
}
}  // extern "C"
