// Krylov kernels (kernels_krylov.cu) used by the device Lanczos and GMRES drivers.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "imps_internal.h"

namespace imps {

constexpr int kMaxCols = 128;  // max Krylov basis size handled by one projection kernel
constexpr int kGmresKrylov = 80;  // default restart length of the device GMRES

struct KrylovWs {
  double* partials = nullptr;     // kr_partials_elems() doubles
  unsigned int* counter = nullptr;
  unsigned int* sync = nullptr;   // 2 zeroed counters of the cooperative CGS2 step (grid barrier)
  int* err = nullptr;             // set when a grid-barrier wait times out
};

size_t kr_partials_elems();
int kr_multidot(const KrylovWs& ws, const double* V, int64_t ldv, int ncols, const double* w,
                int64_t n, double* h, int mode, double* out_sqrt, cudaStream_t st);
int kr_gemv_sub(const double* V, int64_t ldv, int ncols, const double* h, double* w, int64_t n,
                cudaStream_t st);
int kr_gemv(const double* V, int64_t ldv, int ncols, const double* h, double* y, int64_t n,
            cudaStream_t st);
// One CGS2 Lanczos/Arnoldi step on w = A v_{nc-1} against V[:, 0..nc-1]: h[0..nc-1] = total
// projection coefficients, h[nc] = |w| after projection, vnext = w / h[nc] (flag set when
// |w| underflows); h2 (nc doubles) is scratch.  One cooperative launch when n <= 152 * 2048
// (else, or when the cooperative launch is refused, four launches).  nloc > 0 (Lanczos, whose
// projected matrix is tridiagonal): the first pass projects out only the last nloc columns,
// the second pass all of them — half the FP64 work of two full passes, the same orthogonality
// (the first pass removes the large components, the second the rounding-level ones).  The
// four-launch path always runs two full passes.
int kr_cgs2_step(const KrylovWs& ws, const double* V, int64_t ldv, int nc, double* w, int64_t n,
                 double* h, double* h2, double* vnext, int* flag, cudaStream_t st, int nloc = 0);
// One CGS2 step (two full passes) of P systems in four launches (blockIdx.y = system): system q
// has its basis at V + q sV (columns ldv apart), w at w + q sw, its coefficient column at
// h + q sh (h[nc] = |w| after projection), its new basis vector at vnext + q sV and its breakdown
// flag at flags[q] (flags may be NULL).  h2: P x kMaxCols scratch; partials: P x CGRID x
// kMaxCols doubles; counters: P zeroed counters (each reset by its last block).
int kr_cgs2_step_batch(double* partials, unsigned int* counters, int P, const double* V, int64_t sV, int64_t ldv,
                       int nc, double* w, int64_t sw, int64_t n, double* h, int64_t sh, double* h2, double* vnext,
                       int* flags, cudaStream_t st);
int kr_basis_rotate(const double* V, int64_t ldv, int m, const double* W, int kk, double* out,
                    int64_t ldo, int64_t n, cudaStream_t st);
int kr_scale_inv(const double* x, const double* nrm, double* y, int64_t n, int* flag, cudaStream_t st);
int kr_axpby(double a, const double* x, double b, double* y, int64_t n, cudaStream_t st);
int kr_fill_random(double* x, int64_t n, uint64_t seed, cudaStream_t st);
int kr_proj_epilogue(const double* x, const double* t, const double* s, const double* rho, double* y,
                     int64_t n, cudaStream_t st);
int kr_trace_prod(const KrylovWs& ws, const double* X, const double* R, const int64_t* boff,
                  const int32_t* bdim, int nb, double* out, cudaStream_t st, const int32_t* bcols = nullptr);
int kr_fac_epilogue(const double* ure, const double* uim, const double* tre, const double* tim, double c,
                    double s, const double* tau, const double* rho, double* ore, double* oim, int64_t n,
                    cudaStream_t st);
int kr_fac_epilogue_batch(const double* u, const double* t, const double* fre, const double* fim, double* out,
                          int64_t n, int P, cudaStream_t st);
int kr_segsq(const KrylovWs& ws, const double* X, const int64_t* soff, const int64_t* slen, int ns,
             double* out, cudaStream_t st);
int kr_absmax(const KrylovWs& ws, const double* x, int64_t n, double* out, cudaStream_t st);
int kr_sign_of_first(const double* x, double* s, cudaStream_t st);
}  // namespace imps
