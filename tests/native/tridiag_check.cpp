// CPU test harness of the tridiagonal helpers of the Lanczos iteration
// (csrc/tridiag.h).
#include <vector>

#include "../../madsdp.jl_gb300/csrc/tridiag.h"

extern "C" {

// smallest eigenvalue of the k x k tridiagonal (a, b); norm bound in *norm
double check_tridiag_min(int k, const double* a, const double* b, double* norm) {
  std::vector<double> av(a, a + k), bv(b, b + (k > 1 ? k - 1 : 0));
  return tridiag_min(av, bv, k, norm);
}

double check_last_component(int k, const double* a, const double* b, double theta, double norm) {
  std::vector<double> av(a, a + k), bv(b, b + (k > 1 ? k - 1 : 0));
  return tridiag_last_component(av, bv, k, theta, norm);
}

int check_sturm_count(int k, const double* a, const double* b, double x) {
  std::vector<double> av(a, a + k), bv(b, b + (k > 1 ? k - 1 : 0));
  return sturm_count(av, bv, k, x);
}

}  // extern "C"
