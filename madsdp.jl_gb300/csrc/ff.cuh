// Float-float arithmetic: a value is the unevaluated sum hi + lo of two
// FP32 numbers with |lo| <= ulp(hi)/2, about 48 significant bits.
//
// GB300 runs FP32 fused multiply-adds at 128 per clock per SM and FP64 at
// 2, so float-float operations (7 to 20 FP32 instructions each) carry about
// 3.7x the float64 throughput at a precision (~2^-44 relative per
// operation) enough for the positive-definiteness checks and defect
// refinement of the interior-point iteration.
//
// The building blocks are the error-free transformations: Knuth's two-sum
// (s + e = a + b exactly) and the FMA two-product (p + e = a * b exactly),
// combined as in the double-double arithmetic of Dekker (1971) and of
// Hida, Li and Bailey's QD library.  Division and square root take one
// FP32 quotient or root and correct it with one float-float residual.  The
// only library operations used are IEEE FP32 +, -, *, /, sqrt and fma, so
// host and device give identical results (device code is compiled without
// fast-math; the FMAs are written out).
//
// Checked on the CPU by tests/test_ff.py (through tests/native/ff_check.cpp).
#pragma once
#include <cmath>

#ifdef __CUDACC__
#define FF_HD __host__ __device__ __forceinline__
#else
#define FF_HD inline
#endif

struct ff {
  float hi, lo;
  ff() = default;
  FF_HD constexpr ff(float h, float l) : hi(h), lo(l) {}
  // from a number: rounded to the nearest float-float (for double, hi is
  // the nearest float and lo the nearest float to the remainder)
  // the nearest float, and the nearest float to the remainder; beyond the
  // float range hi is infinite and lo is 0, so the value converts back to
  // the same infinity
  FF_HD explicit ff(double v) : hi((float)v), lo(hi - hi == 0.0f ? (float)(v - (double)hi) : 0.0f) {}
  FF_HD explicit ff(float v) : hi(v), lo(0.0f) {}
  FF_HD explicit ff(int v) : ff((double)v) {}
};

FF_HD float ff_fmaf(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}

// s + e = a + b exactly (Knuth)
FF_HD ff ff_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}

// s + e = a + b exactly, for |a| >= |b| or a = 0 (Dekker)
FF_HD ff ff_quick_two_sum(float a, float b) {
  const float s = a + b;
  return {s, b - (s - a)};
}

// p + e = a * b exactly (barring underflow)
FF_HD ff ff_two_prod(float a, float b) {
  const float p = a * b;
  return {p, ff_fmaf(a, b, -p)};
}

FF_HD ff ff_from(float a) { return {a, 0.0f}; }
FF_HD ff ff_neg(ff a) { return {-a.hi, -a.lo}; }

// a + b, relative error about 2^-44 (two two-sums, then renormalization)
FF_HD ff ff_add(ff a, ff b) {
  ff s = ff_two_sum(a.hi, b.hi);
  const ff t = ff_two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = ff_quick_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return ff_quick_two_sum(s.hi, s.lo);
}

FF_HD ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

// a * b
FF_HD ff ff_mul(ff a, ff b) {
  ff p = ff_two_prod(a.hi, b.hi);
  p.lo = ff_fmaf(a.hi, b.lo, ff_fmaf(a.lo, b.hi, p.lo));
  return ff_quick_two_sum(p.hi, p.lo);
}

// a * b for an FP32 b
FF_HD ff ff_mul_f(ff a, float b) {
  ff p = ff_two_prod(a.hi, b);
  p.lo = ff_fmaf(a.lo, b, p.lo);
  return ff_quick_two_sum(p.hi, p.lo);
}

// c + a * b
FF_HD ff ff_fma(ff a, ff b, ff c) { return ff_add(ff_mul(a, b), c); }

// a / b: FP32 quotient q1, residual r = a - q1 b in float-float, second
// quotient q2 = r / b; the result is q1 + q2 renormalized
FF_HD ff ff_div(ff a, ff b) {
  const float q1 = a.hi / b.hi;
  const ff r = ff_sub(a, ff_mul_f(b, q1));
  const float q2 = r.hi / b.hi;
  return ff_quick_two_sum(q1, q2);
}

// sqrt(a) for a >= 0: FP32 root x, one Newton correction computed from the
// float-float residual a - x^2
FF_HD ff ff_sqrt(ff a) {
  if (!(a.hi > 0.0f)) return {a.hi == 0.0f ? 0.0f : std::sqrt(a.hi), 0.0f};
  const float x = std::sqrt(a.hi);
  const ff r = ff_sub(a, ff_two_prod(x, x));
  return ff_quick_two_sum(x, r.hi / (2.0f * x));
}

// double <-> float-float (host-side conversions and tests)
FF_HD ff ff_from_double(double v) {
  const float hi = (float)v;
  return {hi, hi - hi == 0.0f ? (float)(v - (double)hi) : 0.0f};
}
FF_HD double ff_to_double(ff a) { return (double)a.hi + (double)a.lo; }

// Operators, so that the templated CTA routines (products, Cholesky) can be
// instantiated with T = ff.  Comparisons order by hi, then lo (exact for
// normalized values).
FF_HD ff operator+(ff a, ff b) { return ff_add(a, b); }
FF_HD ff operator-(ff a, ff b) { return ff_sub(a, b); }
FF_HD ff operator-(ff a) { return ff_neg(a); }
FF_HD ff operator*(ff a, ff b) { return ff_mul(a, b); }
FF_HD ff operator/(ff a, ff b) { return ff_div(a, b); }
FF_HD ff& operator+=(ff& a, ff b) { return a = ff_add(a, b); }
FF_HD ff& operator-=(ff& a, ff b) { return a = ff_sub(a, b); }
FF_HD ff& operator*=(ff& a, ff b) { return a = ff_mul(a, b); }
FF_HD bool operator<(ff a, ff b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
FF_HD bool operator>(ff a, ff b) { return b < a; }
FF_HD bool operator<=(ff a, ff b) { return !(b < a); }
FF_HD bool operator>=(ff a, ff b) { return !(a < b); }
FF_HD bool operator==(ff a, ff b) { return a.hi == b.hi && a.lo == b.lo; }
FF_HD bool operator!=(ff a, ff b) { return !(a == b); }
FF_HD ff sqrt(ff a) { return ff_sqrt(a); }
FF_HD ff fma(ff a, ff b, ff c) { return ff_fma(a, b, c); }  // a * b + c
FF_HD ff fabs(ff a) { return a.hi < 0.0f || (a.hi == 0.0f && a.lo < 0.0f) ? ff_neg(a) : a; }
