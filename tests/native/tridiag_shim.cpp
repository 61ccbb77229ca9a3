// Test-only C shim over the header-only tridiagonal routines used by the device Lanczos, so
// that the CPU tests can check them against LAPACK (numpy.linalg.eigh).
#include "../../imps_cpp_tools_gb300/csrc/imps_tridiag.h"

extern "C" {
double shim_tri_eigval(int k, const double* a, const double* b, int i) {
  return imps::tri_eigval(k, a, b, i);
}
// the nlow lowest eigenpairs, vectors column-major k x nlow
void shim_tri_lowest(int k, const double* a, const double* b, int nlow, double* w, double* Z) {
  imps::tri_lowest_pairs(k, a, b, nlow, w, Z);
}
void shim_arrow_tridiag(int kk, const double* th, const double* s, double* Q, double* qa, double* qb) {
  imps::arrow_tridiag(kk, th, s, Q, qa, qb);
}
}
