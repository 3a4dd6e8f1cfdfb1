// Host helpers of the Lanczos iteration for lambda_min (the whole-GPU
// solver's step lengths): the smallest eigenvalue of the symmetric
// tridiagonal T_k (diagonal a, off-diagonal b) by Sturm-count bisection,
// and the last component of its unit eigenvector by inverse iteration,
// which gives the Ritz residual |beta_k s_k| of the stopping rule.
// Host code only; checked on the CPU by tests/test_tridiag.py.
#pragma once
#include <algorithm>
#include <cmath>
#include <vector>

// number of eigenvalues of the tridiagonal (a, b) below x (Sturm count)
inline int sturm_count(const std::vector<double>& a, const std::vector<double>& b, int k, double x) {
  int c = 0;
  double d = 1.0;
  for (int i = 0; i < k; ++i) {
    d = a[i] - x - (i ? b[i - 1] * b[i - 1] / d : 0.0);
    if (d == 0.0) d = -1e-300;
    if (d < 0.0) ++c;
  }
  return c;
}

inline double tridiag_min(const std::vector<double>& a, const std::vector<double>& b, int k, double* norm) {
  double lo = INFINITY, hi = -INFINITY;
  for (int i = 0; i < k; ++i) {
    const double r = (i > 0 ? std::fabs(b[i - 1]) : 0.0) + (i < k - 1 ? std::fabs(b[i]) : 0.0);
    lo = std::min(lo, a[i] - r);
    hi = std::max(hi, a[i] + r);
  }
  *norm = std::max(std::fabs(lo), std::fabs(hi));
  for (int it = 0; it < 200; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    if (sturm_count(a, b, k, mid) >= 1) hi = mid; else lo = mid;
  }
  return 0.5 * (lo + hi);
}

// |last component| of the unit eigenvector of the tridiagonal for theta
// (two steps of inverse iteration with a tridiagonal LU)
inline double tridiag_last_component(const std::vector<double>& a, const std::vector<double>& b, int k, double theta,
                              double norm) {
  const double shift = theta - 1e-14 * std::max(norm, 1e-300);
  std::vector<double> y(k, 1.0), c(k), d(k);
  for (int rep = 0; rep < 2; ++rep) {
    // Thomas algorithm on (T - shift I) y_new = y
    double piv = a[0] - shift;
    if (piv == 0.0) piv = 1e-300;
    c[0] = k > 1 ? b[0] / piv : 0.0;
    d[0] = y[0] / piv;
    for (int i = 1; i < k; ++i) {
      piv = a[i] - shift - b[i - 1] * c[i - 1];
      if (piv == 0.0) piv = 1e-300;
      c[i] = i < k - 1 ? b[i] / piv : 0.0;
      d[i] = (y[i] - b[i - 1] * d[i - 1]) / piv;
    }
    y[k - 1] = d[k - 1];
    for (int i = k - 2; i >= 0; --i) y[i] = d[i] - c[i] * y[i + 1];
    double nrm = 0.0;
    for (int i = 0; i < k; ++i) nrm += y[i] * y[i];
    nrm = std::sqrt(nrm);
    if (!(nrm > 0.0) || !std::isfinite(nrm)) return 1.0;
    for (int i = 0; i < k; ++i) y[i] /= nrm;
  }
  return std::fabs(y[k - 1]);
}
