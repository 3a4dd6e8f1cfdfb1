// CPU restatement (C++) of MadSDP's PrimalDual interior-point method (NT or
// HKM direction, EigenStep or CholeskyBacktrack, Mehrotra or AdaptiveMu
// centering) with DenseCholesky and the ScaledIdentity start, for timing the
// CPU baseline without interpreter overhead and for checking GPU results at
// sizes the NumPy restatement is slow on.
//
// TEST INFRASTRUCTURE ONLY, like oracle/madsdp_oracle.py, whose algorithm it
// follows step by step (that module cites the reference file:line of each
// step: src/solver.jl, src/primal_dual.jl, src/directions.jl, src/step.jl,
// src/blocks.jl, src/schur_solvers.jl).  Only tests/ and the CPU legs of
// bench.py load it; the product path never does.  It is checked against the
// NumPy restatement in tests/test_oracle_cpp.py.
//
// Dense linear algebra is written here (no LAPACK): Cholesky with the flush
// of src/blocks.jl:101-111, triangular solves and inverse, and a symmetric
// eigensolver by Householder tridiagonalization followed by the implicit
// symmetric QL iteration with Wilkinson shifts (the textbook method behind
// LAPACK's steqr; written from the mathematics).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <thread>
#include <vector>

#include "../include/madsdp_gpu.h"

namespace {

constexpr double kEps = 2.220446049250313e-16;
using Vec = std::vector<double>;

// ------------------------------------------------------------ dense helpers
// n x n column-major: A(i, j) = A[i + j n]
struct Mat {
  int n = 0;
  Vec a;
  Mat() = default;
  explicit Mat(int n_) : n(n_), a((size_t)n_ * n_, 0.0) {}
  double& operator()(int i, int j) { return a[(size_t)i + (size_t)j * n]; }
  double operator()(int i, int j) const { return a[(size_t)i + (size_t)j * n]; }
};

// C = op(A) op(B)
void gemm(const Mat& A, bool ta, const Mat& B, bool tb, Mat& C) {
  const int n = A.n;
  C = Mat(n);
  for (int j = 0; j < n; ++j)
    for (int k = 0; k < n; ++k) {
      const double bkj = tb ? B(j, k) : B(k, j);
      if (bkj == 0.0) continue;
      double* cj = &C.a[(size_t)j * n];
      if (!ta) {
        const double* ak = &A.a[(size_t)k * n];
        for (int i = 0; i < n; ++i) cj[i] += ak[i] * bkj;
      } else {
        for (int i = 0; i < n; ++i) cj[i] += A(k, i) * bkj;
      }
    }
}

// A = (A + A') / 2 (src/blocks.jl:77-84)
void sym(Mat& A) {
  for (int j = 0; j < A.n; ++j)
    for (int i = j + 1; i < A.n; ++i) {
      const double v = (A(i, j) + A(j, i)) / 2;
      A(i, j) = v;
      A(j, i) = v;
    }
}

double dot(const Mat& A, const Mat& B) {
  double s = 0.0;
  for (size_t k = 0; k < A.a.size(); ++k) s += A.a[k] * B.a[k];
  return s;
}

double maxabs(const Vec& v) {
  double m = 0.0;
  for (double x : v) m = std::max(m, std::fabs(x));
  return m;
}

// In-place lower Cholesky of the lower triangle; false if a pivot is not
// positive and finite (LAPACK potrf semantics).
bool potrf(Mat& A) {
  const int n = A.n;
  for (int k = 0; k < n; ++k) {
    double d = A(k, k);
    for (int p = 0; p < k; ++p) d -= A(k, p) * A(k, p);
    if (!(d > 0.0) || !std::isfinite(d)) return false;
    d = std::sqrt(d);
    A(k, k) = d;
    for (int i = k + 1; i < n; ++i) {
      double s = A(i, k);
      for (int p = 0; p < k; ++p) s -= A(i, p) * A(k, p);
      A(i, k) = s / d;
    }
  }
  for (int j = 1; j < n; ++j)
    for (int i = 0; i < j; ++i) A(i, j) = 0.0;
  return true;
}

// Lower Cholesky factor of sym(M) with the flush of entries below
// eps^2 max|L_ii| (src/blocks.jl:94-113).
bool chol_factor(const Mat& M, Mat& L) {
  L = M;
  sym(L);
  for (double v : L.a)
    if (!std::isfinite(v)) return false;
  if (!potrf(L)) return false;
  double dmax = 0.0;
  for (int i = 0; i < L.n; ++i) dmax = std::max(dmax, std::fabs(L(i, i)));
  const double tol = kEps * kEps * dmax;
  for (double& v : L.a)
    if (std::fabs(v) < tol) v = 0.0;
  return true;
}

// X = L^-1 B (left) for lower triangular L
void trsm_left_lower(const Mat& L, Mat& B) {
  const int n = L.n;
  for (int j = 0; j < n; ++j) {
    double* bj = &B.a[(size_t)j * n];
    for (int i = 0; i < n; ++i) {
      double s = bj[i];
      for (int p = 0; p < i; ++p) s -= L(i, p) * bj[p];
      bj[i] = s / L(i, i);
    }
  }
}

// X = B L^-1 (right) for lower triangular L: X L = B
void trsm_right_lower(const Mat& L, Mat& B) {
  const int n = L.n;
  for (int j = n - 1; j >= 0; --j) {
    double* bj = &B.a[(size_t)j * n];
    for (int p = j + 1; p < n; ++p) {
      const double l = L(p, j);
      if (l == 0.0) continue;
      const double* bp = &B.a[(size_t)p * n];
      for (int i = 0; i < n; ++i) bj[i] -= bp[i] * l;
    }
    const double inv = 1.0 / L(j, j);
    for (int i = 0; i < n; ++i) bj[i] *= inv;
  }
}

// S^-1 = L^-T L^-1 from the Cholesky factor (potri)
void inverse_from_chol(const Mat& L, Mat& Si) {
  const int n = L.n;
  Mat Li(n);
  for (int i = 0; i < n; ++i) Li(i, i) = 1.0;
  trsm_left_lower(L, Li);  // Li = L^-1
  gemm(Li, true, Li, false, Si);
  sym(Si);
}

// ------------------------------------------------------------ eigensolver
// Householder reduction of the symmetric A to tridiagonal T = Q' A Q:
// diagonal d, subdiagonal e (e[i] couples i and i+1), Q accumulated when
// requested.
void tridiagonalize(Mat A, Vec& d, Vec& e, Mat* Q) {
  const int n = A.n;
  d.assign(n, 0.0);
  e.assign(n, 0.0);
  if (Q) {
    *Q = Mat(n);
    for (int i = 0; i < n; ++i) (*Q)(i, i) = 1.0;
  }
  Vec v(n, 0.0), p(n, 0.0), w(n, 0.0);
  for (int k = 0; k + 2 < n; ++k) {
    double nrm = 0.0;
    for (int i = k + 1; i < n; ++i) nrm += A(i, k) * A(i, k);
    nrm = std::sqrt(nrm);
    if (nrm == 0.0) {
      e[k] = 0.0;
      continue;
    }
    const double alpha = A(k + 1, k) > 0.0 ? -nrm : nrm;  // reflect x onto alpha e1
    for (int i = 0; i < n; ++i) v[i] = i > k ? A(i, k) : 0.0;
    v[k + 1] -= alpha;
    double vtv = 0.0;
    for (int i = k + 1; i < n; ++i) vtv += v[i] * v[i];
    if (vtv == 0.0) {
      e[k] = A(k + 1, k);
      continue;
    }
    const double beta = 2.0 / vtv;
    // p = beta A22 v, q = p - (beta/2)(p'v) v, A22 -= v q' + q v'
    double pv = 0.0;
    for (int i = k + 1; i < n; ++i) {
      double s = 0.0;
      for (int j = k + 1; j < n; ++j) s += A(i, j) * v[j];
      p[i] = beta * s;
      pv += p[i] * v[i];
    }
    const double K = 0.5 * beta * pv;
    for (int i = k + 1; i < n; ++i) p[i] -= K * v[i];
    for (int j = k + 1; j < n; ++j)
      for (int i = k + 1; i < n; ++i) A(i, j) -= v[i] * p[j] + p[i] * v[j];
    e[k] = alpha;
    if (Q) {
      Mat& q = *Q;
      for (int r = 0; r < n; ++r) {
        double s = 0.0;
        for (int j = k + 1; j < n; ++j) s += q(r, j) * v[j];
        w[r] = beta * s;
      }
      for (int j = k + 1; j < n; ++j)
        for (int r = 0; r < n; ++r) q(r, j) -= w[r] * v[j];
    }
  }
  for (int i = 0; i < n; ++i) d[i] = A(i, i);
  if (n >= 2) e[n - 2] = A(n - 1, n - 2);
  e[n - 1] = 0.0;
}

// Eigenvalues (ascending) of the symmetric tridiagonal (d, e) by the
// implicit QL iteration with Wilkinson shifts; the plane rotations are
// applied to the columns of Z when given.  False if an eigenvalue did not
// converge in 64 iterations.
bool tridiag_ql(Vec& d, Vec& e, Mat* Z) {
  const int n = (int)d.size();
  for (int l = 0; l < n; ++l) {
    for (int it = 0;; ++it) {
      int m = l;
      for (; m + 1 < n; ++m)
        if (std::fabs(e[m]) <= kEps * (std::fabs(d[m]) + std::fabs(d[m + 1]))) break;
      if (m == l) break;
      if (it >= 64) return false;
      double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
      double r = std::hypot(g, 1.0);
      g = d[m] - d[l] + e[l] / (g + (g >= 0.0 ? r : -r));
      double s = 1.0, c = 1.0, p = 0.0;
      bool split = false;
      for (int i = m - 1; i >= l; --i) {
        const double f = s * e[i], b = c * e[i];
        r = std::hypot(f, g);
        e[i + 1] = r;
        if (r == 0.0) {  // the rotation underflowed: deflate and restart
          d[i + 1] -= p;
          e[m] = 0.0;
          split = true;
          break;
        }
        s = f / r;
        c = g / r;
        g = d[i + 1] - p;
        r = (d[i] - g) * s + 2.0 * c * b;
        p = s * r;
        d[i + 1] = g + p;
        g = c * r - b;
        if (Z) {
          Mat& z = *Z;
          for (int k = 0; k < z.n; ++k) {
            const double t = z(k, i + 1);
            z(k, i + 1) = s * z(k, i) + c * t;
            z(k, i) = c * z(k, i) - s * t;
          }
        }
      }
      if (split) continue;
      d[l] -= p;
      e[l] = g;
      e[m] = 0.0;
    }
  }
  // ascending order (selection sort keeps the vectors with their values)
  for (int i = 0; i < n; ++i) {
    int k = i;
    for (int j = i + 1; j < n; ++j)
      if (d[j] < d[k]) k = j;
    if (k != i) {
      std::swap(d[i], d[k]);
      if (Z)
        for (int r = 0; r < Z->n; ++r) std::swap((*Z)(r, i), (*Z)(r, k));
    }
  }
  return true;
}

// eigh: A = V diag(w) V', w ascending (V when requested)
bool symeig(const Mat& A, Vec& w, Mat* V) {
  Vec e;
  tridiagonalize(A, w, e, V);
  return tridiag_ql(w, e, V);
}

// ------------------------------------------------------------ the solver
struct Block {
  int n = 0;
  Mat C;
  std::vector<int32_t> row, col;  // entries sorted by constraint
  Vec val;
  std::vector<int64_t> cptr;      // m + 1
  std::vector<int32_t> con;       // constraint of each sorted entry
  double cnorm = 0.0;
  bool rdnz = true;
  Mat X, S, Rd, Ls, Si, Lx, W, G, Gi, dX, dS, corr, ERd;
  Vec D;
};

struct Solver {
  int m = 0, ns = 0;
  std::vector<Block> B;
  Vec b, dlin, Clin;  // Clin m x ns column-major
  double bn = 0.0, dn = 0.0, cmax = 0.0;
  Vec y, dy, Rp, x, z, dx, dz, Rdlin, zinv, corrlin;
  Mat Lh;  // Cholesky factor of the Schur matrix
  double mu = 0.0, sigma = 0.0, alpha = 0.0, beta = 0.0;
  double pobj = 0.0, dobj = 0.0, inf_pr = 0.0, inf_du = 0.0, gap = 0.0;
  int iter = 0, status = MSDP_INITIAL;
  msdp_options opt{};
  msdp_components comp{};
  bool nt = true;  // NT or HKM

  int nu() const {
    int v = ns;
    for (const auto& blk : B) v += blk.n;
    return v;
  }

  // out += A_i(X)
  void jprod(const Block& k, const Mat& X, Vec& out) const {
    for (int j = 0; j < m; ++j) {
      double s = 0.0;
      for (int64_t q = k.cptr[j]; q < k.cptr[j + 1]; ++q) s += k.val[q] * X(k.row[q], k.col[q]);
      out[j] += s;
    }
  }
  // M = A_i*(v)
  void jtprod(const Block& k, const Vec& v, Mat& M) const {
    M = Mat(k.n);
    for (size_t q = 0; q < k.val.size(); ++q) M(k.row[q], k.col[q]) += k.val[q] * v[k.con[q]];
  }
  // out = base + sgn C_lin' v  (ns)
  void clin_t(const Vec& v, Vec& out) const {
    out.assign(ns, 0.0);
    for (int s = 0; s < ns; ++s) {
      double t = 0.0;
      for (int j = 0; j < m; ++j) t += Clin[(size_t)j + (size_t)s * m] * v[j];
      out[s] = t;
    }
  }
  // out += C_lin v  (m)
  void clin_add(const Vec& v, Vec& out) const {
    for (int s = 0; s < ns; ++s)
      for (int j = 0; j < m; ++j) out[j] += Clin[(size_t)j + (size_t)s * m] * v[s];
  }

  double total_complementarity() const {
    double s = 0.0;
    for (const auto& k : B) s += dot(k.X, k.S);
    for (int i = 0; i < ns; ++i) s += x[i] * z[i];
    return s;
  }

  // src/step.jl:12-47
  void update_residuals() {
    Vec acc(m, 0.0);
    for (const auto& k : B) jprod(k, k.X, acc);
    clin_add(x, acc);
    Rp.assign(m, 0.0);
    for (int j = 0; j < m; ++j) Rp[j] = b[j] - acc[j];
    for (auto& k : B) {
      Mat aty;
      jtprod(k, y, aty);
      k.Rd = Mat(k.n);
      double r = 0.0;
      for (size_t q = 0; q < k.Rd.a.size(); ++q) {
        k.Rd.a[q] = k.C.a[q] - k.S.a[q] - aty.a[q];
        r = std::max(r, std::fabs(k.Rd.a[q]));
      }
      k.rdnz = r > 100.0 * kEps * std::max(1.0, k.cnorm);
    }
    if (ns) {
      Vec cty;
      clin_t(y, cty);
      Rdlin.assign(ns, 0.0);
      for (int s = 0; s < ns; ++s) Rdlin[s] = dlin[s] - z[s] - cty[s];
    }
  }

  // src/primal_dual.jl:123-134, src/solver.jl:318-347
  void update_termination() {
    double p = 0.0;
    for (const auto& k : B) p += dot(k.C, k.X);
    for (int s = 0; s < ns; ++s) p += dlin[s] * x[s];
    double d = 0.0;
    for (int j = 0; j < m; ++j) d += b[j] * y[j];
    pobj = p;
    dobj = d;
    inf_pr = (m ? maxabs(Rp) : 0.0) / std::max(1.0, bn);
    double rd = 0.0, cn = cmax;
    for (const auto& k : B) rd = std::max(rd, maxabs(k.Rd.a));
    if (ns) {
      rd = std::max(rd, maxabs(Rdlin));
      cn = std::max(cn, dn);
    }
    inf_du = rd / std::max(1.0, cn);
    gap = std::fabs(p - d) / std::max(1.0, std::fabs(p) + std::fabs(d));
    if (std::max(std::max(inf_pr, inf_du), gap) <= opt.tol) status = MSDP_SOLVE_SUCCEEDED;
    else if (iter >= opt.max_iter) status = MSDP_MAXIMUM_ITERATIONS_EXCEEDED;
    if (status == MSDP_REGULAR && mu < opt.mu_min) status = MSDP_SEARCH_DIRECTION_BECOMES_TOO_SMALL;
  }

  // S^-1 (src/primal_dual.jl:29-37), the NT scaling (src/directions.jl:45-75)
  // and the Cholesky factor of X that EigenStep uses
  bool prepare() {
    for (auto& k : B) {
      if (!chol_factor(k.S, k.Ls)) return false;
      inverse_from_chol(k.Ls, k.Si);
      if (!nt) {
        if (comp.step == MSDP_EIGEN_STEP && !chol_factor(k.X, k.Lx)) return false;
        continue;
      }
      if (!chol_factor(k.X, k.Lx)) return false;
      Mat M, N, V;
      gemm(k.Ls, true, k.Lx, false, M);
      gemm(M, true, M, false, N);
      sym(N);
      Vec lam;
      if (!symeig(N, lam, &V)) return false;
      for (double l : lam)
        if (!(l > 0.0)) return false;
      const int n = k.n;
      k.D.assign(n, 0.0);
      Vec sc(n);
      for (int i = 0; i < n; ++i) {
        k.D[i] = std::sqrt(lam[i]);
        sc[i] = std::sqrt(k.D[i]);
      }
      gemm(k.Lx, false, V, false, k.G);  // G = Lx V / sc
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) k.G(i, j) /= sc[j];
      k.Gi = Mat(n);  // Gi = diag(sc) V' Lx^-1
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) k.Gi(i, j) = V(j, i) * sc[i];
      trsm_right_lower(k.Lx, k.Gi);
      gemm(k.G, false, k.G, true, k.W);
      sym(k.W);
    }
    zinv.assign(ns, 0.0);
    for (int s = 0; s < ns; ++s) zinv[s] = 1.0 / z[s];
    return true;
  }

  // H_jk = sum_i <A_ij, W_i A_ik W_i> + C_lin diag(x/z) C_lin' (lower),
  // then the regularization retry loop (src/solver.jl:299-314)
  // H_jk = <A_j, L A_k R>: (L, R) = (W, W) for NT, (S^-1, X) for HKM
  // (src/directions.jl:212,247); both symmetric.
  const Mat& scale_L(const Block& k) const { return nt ? k.W : k.Si; }
  const Mat& scale_R(const Block& k) const { return nt ? k.W : k.X; }

  // Per constraint k: T = L A_k R (A_k R by rows, then one product), and
  // H_jk = A_j(T) for j >= k; cost m (2 n^3 + nnz) + n nnz.
  void schur_by_columns(const Block& k, Mat& H0) const {
    const int n = k.n;
    const Mat& L = scale_L(k);
    const Mat& R = scale_R(k);
    Mat AR(n), T;
    for (int c = 0; c < m; ++c) {
      if (k.cptr[c] == k.cptr[c + 1]) continue;
      std::fill(AR.a.begin(), AR.a.end(), 0.0);
      for (int64_t f = k.cptr[c]; f < k.cptr[c + 1]; ++f) {  // row r_f of A_k R += v_f R(c_f, :)
        const int r = k.row[f], cf = k.col[f];
        const double v = k.val[f];
        for (int q = 0; q < n; ++q) AR(r, q) += v * R(cf, q);
      }
      gemm(L, false, AR, false, T);
      for (int j = c; j < m; ++j) {
        double s = 0.0;
        for (int64_t e = k.cptr[j]; e < k.cptr[j + 1]; ++e) s += k.val[e] * T(k.row[e], k.col[e]);
        H0(j, c) += s;
      }
    }
  }

  bool factorize_schur() {
    Mat H0(m);
    for (const auto& k : B) {
      // the cheaper of the two summation orders of the same sum
      const double nnz = (double)k.val.size();
      if (nnz * nnz > 2.0 * (double)m * (2.0 * k.n * (double)k.n * k.n + nnz)) {
        schur_by_columns(k, H0);
        continue;
      }
      for (int j = 0; j < m; ++j)
        for (int c = 0; c <= j; ++c) {
          double s = 0.0;
          for (int64_t e = k.cptr[j]; e < k.cptr[j + 1]; ++e) {
            const int re = k.row[e], ce = k.col[e];
            double t = 0.0;
            // L(r_e, r_f) R(c_f, c_e), L symmetric: both read down a column
            const double* wr = &scale_L(k).a[(size_t)re * k.n];
            const double* wc = &scale_R(k).a[(size_t)ce * k.n];
            for (int64_t f = k.cptr[c]; f < k.cptr[c + 1]; ++f) t += k.val[f] * wr[k.row[f]] * wc[k.col[f]];
            s += k.val[e] * t;
          }
          H0(j, c) += s;
        }
    }
    for (int s = 0; s < ns; ++s) {
      const double w = x[s] * zinv[s];
      for (int j = 0; j < m; ++j)
        for (int c = 0; c <= j; ++c) H0(j, c) += Clin[(size_t)j + (size_t)s * m] * w * Clin[(size_t)c + (size_t)s * m];
    }
    double reg = opt.regularize_schur;
    for (int t = 0; t < opt.max_schur_reg; ++t) {
      Lh = H0;
      if (reg > 0.0)
        for (int j = 0; j < m; ++j) Lh(j, j) += reg;
      if (potrf(Lh)) return true;
      reg = reg == 0.0 ? 1e-12 : 10.0 * reg;
    }
    return false;
  }

  void schur_solve(Vec& v) const {
    for (int i = 0; i < m; ++i) {
      double s = v[i];
      for (int p = 0; p < i; ++p) s -= Lh(i, p) * v[p];
      v[i] = s / Lh(i, i);
    }
    for (int i = m - 1; i >= 0; --i) {
      double s = v[i];
      for (int p = i + 1; p < m; ++p) s -= Lh(p, i) * v[p];
      v[i] = s / Lh(i, i);
    }
  }

  // E(M): NT sym(W M W), HKM sym(X M S^-1) (src/directions.jl:80-84,116-120)
  void apply_E(const Block& k, const Mat& M, Mat& out) const {
    Mat t;
    gemm(nt ? k.W : k.X, false, M, false, t);
    gemm(t, false, nt ? k.W : k.Si, false, out);
    sym(out);
  }

  // rhs, Schur solve and directions (src/step.jl:63-124)
  void solve_directions(double mu_, bool corrected) {
    Vec h = Rp;
    for (auto& k : B) {
      if (!corrected && k.rdnz) apply_E(k, k.Rd, k.ERd);
      Mat buf(k.n);
      for (size_t q = 0; q < buf.a.size(); ++q) {
        double v = k.X.a[q] - mu_ * k.Si.a[q];
        if (k.rdnz) v += k.ERd.a[q];
        if (corrected) v -= k.corr.a[q];
        buf.a[q] = v;
      }
      jprod(k, buf, h);
    }
    if (ns) {
      Vec v(ns);
      for (int s = 0; s < ns; ++s) {
        double t = x[s] - mu_ * zinv[s] + x[s] * zinv[s] * Rdlin[s];
        if (corrected) t -= corrlin[s];
        v[s] = t;
      }
      clin_add(v, h);
    }
    schur_solve(h);
    dy = h;
    for (auto& k : B) {
      Mat atdy, e1;
      jtprod(k, dy, atdy);
      k.dS = Mat(k.n);
      for (size_t q = 0; q < atdy.a.size(); ++q) k.dS.a[q] = k.Rd.a[q] - atdy.a[q];
      sym(k.dS);
      apply_E(k, atdy, e1);
      k.dX = Mat(k.n);
      for (size_t q = 0; q < e1.a.size(); ++q) {
        double v = mu_ * k.Si.a[q] - k.X.a[q] + e1.a[q];
        if (k.rdnz) v -= k.ERd.a[q];
        if (corrected) v += k.corr.a[q];
        k.dX.a[q] = v;
      }
      sym(k.dX);
    }
    if (ns) {
      Vec ctdy;
      clin_t(dy, ctdy);
      dz.assign(ns, 0.0);
      dx.assign(ns, 0.0);
      for (int s = 0; s < ns; ++s) {
        dz[s] = Rdlin[s] - ctdy[s];
        double v = mu_ * zinv[s] - x[s] - x[s] * zinv[s] * dz[s];
        if (corrected) v += corrlin[s];
        dx[s] = v;
      }
    }
  }

  // Mehrotra second-order term (src/step.jl:128-136): NT
  // src/directions.jl:90-100, HKM sym(-(dX dS) S^-1) (:123-127)
  void correction() {
    for (auto& k : B) {
      const int n = k.n;
      if (!nt) {
        Mat t;
        gemm(k.dX, false, k.dS, false, t);
        gemm(t, false, k.Si, false, k.corr);
        for (double& v : k.corr.a) v = -v;
        sym(k.corr);
        continue;
      }
      Mat t1, t2, Mm;
      gemm(k.Gi, false, k.dX, false, t1);
      gemm(t1, false, k.dS, false, t2);
      gemm(t2, false, k.G, false, Mm);
      Mat rnt(n);
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) rnt(i, j) = -(Mm(i, j) + Mm(j, i)) / (k.D[i] + k.D[j]);
      gemm(k.G, false, rnt, false, t1);
      gemm(t1, false, k.G, true, k.corr);
      sym(k.corr);
    }
    corrlin.assign(ns, 0.0);
    for (int s = 0; s < ns; ++s) corrlin[s] = -dx[s] * dz[s] * zinv[s];
  }

  // smallest eigenvalue of L^-1 D L^-T (src/step.jl:150-163, 178-183)
  double eigen_step(const Mat& L, const Mat& Dm) const {
    Mat Z = Dm;
    trsm_left_lower(L, Z);  // L^-1 D
    Mat Zt(Z.n);
    for (int j = 0; j < Z.n; ++j)
      for (int i = 0; i < Z.n; ++i) Zt(i, j) = Z(j, i);
    trsm_left_lower(L, Zt);  // L^-1 (L^-1 D)'
    sym(Zt);
    Vec w;
    if (!symeig(Zt, w, nullptr)) return 0.0;
    const double lam = w.empty() ? INFINITY : w[0];
    return lam > -std::sqrt(kEps) ? 1.0 : std::min(1.0, -comp.tau / lam);
  }

  static double max_scalar_step(const Vec& v, const Vec& dv) {
    double a = INFINITY;
    for (size_t i = 0; i < v.size(); ++i)
      if (dv[i] < 0.0) a = std::min(a, -v[i] / dv[i]);
    return a;
  }

  // LAPACK potrf on the lower triangle of M + a D succeeds (src/blocks.jl:133-137)
  static bool is_posdef(const Mat& M, double a, const Mat& D) {
    Mat T(M.n);
    for (size_t q = 0; q < T.a.size(); ++q) {
      T.a[q] = M.a[q] + a * D.a[q];
      if (!std::isfinite(T.a[q])) return false;
    }
    return potrf(T);
  }

  // CholeskyBacktrack (src/step.jl:202-221)
  double backtrack(bool primal) const {
    double a = 1.0;
    for (const auto& k : B) {
      const Mat& M = primal ? k.X : k.S;
      const Mat& D = primal ? k.dX : k.dS;
      while (!is_posdef(M, a, D)) {
        a *= comp.shrink;
        if (a < kEps) return 0.0;
      }
    }
    if (a != 1.0) a *= comp.boundary;
    if (ns) a = std::min(a, comp.boundary * max_scalar_step(primal ? x : z, primal ? dx : dz));
    return a;
  }

  // src/step.jl:148-228
  void step_lengths(double& a, double& bt) const {
    if (comp.step == MSDP_CHOLESKY_BACKTRACK) {
      a = backtrack(true);
      bt = backtrack(false);
      return;
    }
    a = 1.0;
    bt = 1.0;
    for (const auto& k : B) {
      a = std::min(a, eigen_step(k.Lx, k.dX));
      bt = std::min(bt, eigen_step(k.Ls, k.dS));
    }
    if (ns) {
      a = std::min(a, comp.tau * max_scalar_step(x, dx));
      bt = std::min(bt, comp.tau * max_scalar_step(z, dz));
    }
  }

  // src/step.jl:231-243
  double affine_complementarity(double a, double bt) const {
    double s = 0.0;
    for (const auto& k : B) {
      s += dot(k.X, k.S);
      s += bt * dot(k.X, k.dS);
      s += a * dot(k.dX, k.S);
      s += a * bt * dot(k.dX, k.dS);
    }
    for (int i = 0; i < ns; ++i) s += (x[i] + a * dx[i]) * (z[i] + bt * dz[i]);
    return s / std::max(nu(), 1);
  }

  // src/primal_dual.jl:56-72
  void take_step(double a, double bt) {
    alpha = a;
    beta = bt;
    for (auto& k : B) {
      for (size_t q = 0; q < k.X.a.size(); ++q) {
        k.X.a[q] += a * k.dX.a[q];
        k.S.a[q] += bt * k.dS.a[q];
      }
      sym(k.X);
      sym(k.S);
    }
    for (int j = 0; j < m; ++j) y[j] += bt * dy[j];
    for (int s = 0; s < ns; ++s) {
      x[s] += a * dx[s];
      z[s] += bt * dz[s];
    }
    iter += 1;
    update_residuals();
  }

  // src/primal_dual.jl:85-101
  void iterate_mehrotra() {
    if (!prepare() || !factorize_schur()) {
      status = MSDP_ERROR_IN_STEP_COMPUTATION;
      return;
    }
    const double mu0 = total_complementarity() / std::max(nu(), 1);
    mu = mu0;
    solve_directions(0.0, false);
    double aa = 0.0, ba = 0.0;
    step_lengths(aa, ba);
    const double mua = affine_complementarity(aa, ba);
    sigma = std::min(std::max(std::pow(mua / std::max(mu0, kEps), comp.sigma_exponent), 1e-8), 1.0);
    correction();
    solve_directions(sigma * mu0, true);
    double a = 0.0, bt = 0.0;
    step_lengths(a, bt);
    take_step(a, bt);
  }

  // src/primal_dual.jl:104-121
  void iterate_adaptive() {
    if (!prepare() || !factorize_schur()) {
      status = MSDP_ERROR_IN_STEP_COMPUTATION;
      return;
    }
    solve_directions(mu, false);
    double a = 0.0, bt = 0.0;
    step_lengths(a, bt);
    take_step(a, bt);
    double m1 = comp.ratio * total_complementarity() / std::max(nu(), 1);
    if (std::min(a, bt) < 0.5) m1 *= 1.5;
    if (a + bt > 1.6) m1 *= 0.75;
    if (a + bt > 1.9) m1 /= 1 + 0.1 * iter;
    mu = m1;
  }

  // ScaledIdentity start (src/solver.jl:214-233) and solve! (:385-396)
  void solve() {
    double cs = cmax;
    if (ns) cs = std::max(cs, dn);
    const double beta0 = comp.scale > 0.0
                             ? comp.scale
                             : std::max(10.0, std::sqrt(std::max(bn, 1.0) * std::max(cs, 1.0)) * std::sqrt((double)nu()));
    for (auto& k : B) {
      k.X = Mat(k.n);
      k.S = Mat(k.n);
      for (int i = 0; i < k.n; ++i) k.X(i, i) = k.S(i, i) = beta0;
    }
    y.assign(m, 0.0);
    x.assign(ns, beta0);
    z.assign(ns, beta0);
    iter = 0;
    status = MSDP_REGULAR;
    update_residuals();
    mu = total_complementarity() / std::max(nu(), 1);  // src/primal_dual.jl:10-19
    if (comp.centering == MSDP_ADAPTIVE_MU) mu *= comp.initial_ratio;
    update_termination();
    while (status == MSDP_REGULAR) {
      if (comp.centering == MSDP_ADAPTIVE_MU) iterate_adaptive();
      else iterate_mehrotra();
      if (status != MSDP_REGULAR) break;
      update_termination();
    }
  }
};

bool load(const msdp_problem_desc& d, Solver& s) {
  if (d.nblocks < 0 || d.m < 0 || d.ns < 0) return false;
  s.m = d.m;
  s.ns = d.ns;
  s.b.assign(d.b, d.b + d.m);
  s.dlin.assign(d.d_lin, d.d_lin + d.ns);
  s.Clin.assign(d.C_lin, d.C_lin + (size_t)d.m * d.ns);
  s.bn = maxabs(s.b);
  s.dn = maxabs(s.dlin);
  s.B.resize(d.nblocks);
  for (int i = 0; i < d.nblocks; ++i) {
    Block& k = s.B[i];
    k.n = d.sides[i];
    if (k.n <= 0) return false;
    k.C = Mat(k.n);
    std::copy(d.C[i], d.C[i] + (size_t)k.n * k.n, k.C.a.begin());
    k.cnorm = maxabs(k.C.a);
    s.cmax = std::max(s.cmax, k.cnorm);
    const int64_t nnz = d.A_nnz[i];
    std::vector<int64_t> idx(nnz);
    std::iota(idx.begin(), idx.end(), 0);
    const int32_t* con = d.A_con[i];
    std::stable_sort(idx.begin(), idx.end(), [&](int64_t a, int64_t b) { return con[a] < con[b]; });
    k.cptr.assign(s.m + 1, 0);
    for (int64_t q = 0; q < nnz; ++q) {
      const int64_t e = idx[q];
      if (con[e] < 0 || con[e] >= s.m || d.A_row[i][e] < 0 || d.A_row[i][e] >= k.n || d.A_col[i][e] < 0 ||
          d.A_col[i][e] >= k.n)
        return false;
      k.con.push_back(con[e]);
      k.row.push_back(d.A_row[i][e]);
      k.col.push_back(d.A_col[i][e]);
      k.val.push_back(d.A_val[i][e]);
      k.cptr[con[e] + 1] += 1;
    }
    for (int j = 0; j < s.m; ++j) k.cptr[j + 1] += k.cptr[j];
  }
  return true;
}

}  // namespace

extern "C" {

// The defaults of src/options.jl:3-15 (the same values msdp_default_options
// gives; this library does not link the CUDA one).
void msdp_cpu_default_options(msdp_options* o) {
  std::memset(o, 0, sizeof(*o));
  o->tol = 1e-7;
  o->max_iter = 100;
  o->max_schur_reg = 8;
  o->max_wall_time = 3600.0;
  o->mu_min = 1e-14;
  o->regularize_schur = 1e-12;
  o->datasparsity = 8;
  o->mixed_refine = 2;
}

// The defaults of src/components.jl (PrimalDual, NT, EigenStep(0.95),
// Mehrotra(3), ScaledIdentity(), DenseCholesky; CholeskyBacktrack(0.8,
// 0.95), AdaptiveMu(1/4, 1/2), DualShift(1, 1e10), DualCentering(0.2, 1, 2)).
void msdp_cpu_default_components(msdp_components* c) {
  std::memset(c, 0, sizeof(*c));
  c->algorithm = MSDP_PRIMAL_DUAL;
  c->direction = MSDP_NT;
  c->step = MSDP_EIGEN_STEP;
  c->centering = MSDP_MEHROTRA;
  c->initial_point = MSDP_SCALED_IDENTITY;
  c->schur = MSDP_DENSE_CHOLESKY;
  c->precision = MSDP_FP64;
  c->centering_max_iter = 50;
  c->tau = 0.95;
  c->shrink = 0.8;
  c->boundary = 0.95;
  c->sigma_exponent = 3.0;
  c->initial_ratio = 0.25;
  c->ratio = 0.5;
  c->scale = 0.0;
  c->initial_shift = 1.0;  // DualShift and DualCentering: not run here, kept equal to the library's
  c->max_shift = 1e10;
  c->dc_beta = 0.2;
  c->dc_delta = 1.0;
  c->dc_A = 2.0;
}

// One solve with `comp` and `opt` (the defaults when null); writes status,
// iter, the objectives, the three termination measures, mu, sigma, alpha,
// beta and the wall time of the solve in solve_ns.  Components other than
// PrimalDual with DenseCholesky from ScaledIdentity: MSDP_ERR_UNSUPPORTED.
int msdp_cpu_solve(const msdp_problem_desc* d, const msdp_components* comp, const msdp_options* opt,
                   msdp_stats* out) {
  if (!d || !out) return MSDP_ERR_INVALID_ARGUMENT;
  Solver s;
  if (opt) s.opt = *opt; else msdp_cpu_default_options(&s.opt);
  if (comp) s.comp = *comp; else msdp_cpu_default_components(&s.comp);
  const msdp_components& c = s.comp;
  if (c.algorithm != MSDP_PRIMAL_DUAL || c.schur != MSDP_DENSE_CHOLESKY || c.initial_point != MSDP_SCALED_IDENTITY ||
      (c.direction != MSDP_NT && c.direction != MSDP_HKM) ||
      (c.step != MSDP_EIGEN_STEP && c.step != MSDP_CHOLESKY_BACKTRACK) ||
      (c.centering != MSDP_MEHROTRA && c.centering != MSDP_ADAPTIVE_MU))
    return MSDP_ERR_UNSUPPORTED;
  s.nt = c.direction == MSDP_NT;
  if (!load(*d, s)) return MSDP_ERR_INVALID_ARGUMENT;
  const auto t0 = std::chrono::steady_clock::now();
  s.solve();
  const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::memset(out, 0, sizeof(*out));
  out->status = s.status; out->iter = s.iter; out->iter_fp64 = s.iter;
  out->pobj = s.pobj; out->dobj = s.dobj; out->inf_pr = s.inf_pr; out->inf_du = s.inf_du; out->gap = s.gap;
  out->mu = s.mu; out->sigma = s.sigma; out->alpha = s.alpha; out->beta = s.beta; out->solve_ns = sec * 1e9;
  return MSDP_OK;
}

// Solves problems[0..count) on `threads` host threads (one problem per
// thread at a time, in order of an atomic counter) until all are done or
// `seconds` (> 0) have passed; returns how many were solved.
int msdp_cpu_solve_many(const msdp_problem_desc* problems, int32_t count, int32_t threads, double seconds,
                        const msdp_components* comp, const msdp_options* opt, msdp_stats* out) {
  if (!problems || !out || count < 0 || threads <= 0) return MSDP_ERR_INVALID_ARGUMENT;
  std::atomic<int> next{0}, done{0};
  const auto t0 = std::chrono::steady_clock::now();
  auto work = [&]() {
    for (;;) {
      if (seconds > 0.0 &&
          std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() >= seconds)
        return;
      const int i = next.fetch_add(1);
      if (i >= count) return;
      if (msdp_cpu_solve(problems + i, comp, opt, out + i) == MSDP_OK) done.fetch_add(1);
      else out[i].status = -1;
    }
  };
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t) pool.emplace_back(work);
  for (auto& th : pool) th.join();
  return done.load();
}

// Test hook: eigenvalues (ascending) and optionally eigenvectors of the
// symmetric n x n column-major A.
int msdp_cpu_symeig(int32_t n, const double* A, double* w, double* V) {
  if (n <= 0 || !A || !w) return MSDP_ERR_INVALID_ARGUMENT;
  Mat M(n);
  std::copy(A, A + (size_t)n * n, M.a.begin());
  Vec ev;
  Mat Q;
  if (!symeig(M, ev, V ? &Q : nullptr)) return MSDP_ERR_CUDA;
  std::copy(ev.begin(), ev.end(), w);
  if (V) std::copy(Q.a.begin(), Q.a.end(), V);
  return MSDP_OK;
}

}  // extern "C"
