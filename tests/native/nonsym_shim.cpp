// Test-only C shim over the header-only nonsymmetric routines used by the device Arnoldi
// solver, so that the CPU tests can check them against LAPACK (numpy.linalg.eig).
#include "../../imps_cpp_tools_gb300/csrc/imps_nonsym.h"

extern "C" {
// eigenvalues of a general k x k column-major matrix; returns 0 on success
int shim_dense_eigvals(int k, const double* G, double* wr, double* wi) {
  return imps::dense_eigvals(k, G, wr, wi) ? 0 : 1;
}
// eigenvector for lam = (lr, li): y interleaved (re, im), k complex entries
void shim_dense_eigvec(int k, const double* G, double gnorm, double lr, double li, double* y) {
  imps::dense_eigvec(k, G, gnorm, imps::cplx(lr, li), reinterpret_cast<imps::cplx*>(y));
}
// order of k eigenvalues for which = 0 (LM), 1 (LR), 2 (SR)
void shim_order_ritz(int k, const double* wr, const double* wi, int which, int* idx) {
  auto o = imps::order_ritz(k, wr, wi, which);
  for (int i = 0; i < k; ++i) idx[i] = o[i];
}
}
