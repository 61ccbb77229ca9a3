// Per-sector dense decompositions of block-sparse MPS tensors on the device (FP64 always).
//
// The reference stacks, per charge sector, the blocks of A_s into one dense matrix
// (MPSBlockMat::GetDenseMat, MPSBlockMat.hpp:468-526 with GetSingleSecData :636-719) and
// runs LAPACK on it: qr_econ + sign fix (qr_pos, helpers.hpp:181-195) or svd_econ
// (MPSBlockUtilities.hpp:78-244, BlockObj.hpp:2422-2541).  Here every sector is one CTA:
//  * gather: blocks -> packed column-major dense matrices (transposed for dir = r, so that
//    every matrix is handled as "tall": M = stacked dimension, N = sector dimension);
//  * Householder QR with explicit Q and diag(R) >= 0;
//  * one-sided (Hestenes) Jacobi SVD, singular values sorted descending;
//  * scatter back to the block layout.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "imps_decomp.h"
#include "imps_status.h"

namespace {

constexpr int DT = 256;  // threads per CTA (8 warps)

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block-wide sum, result broadcast to all threads
__device__ double bsum(double v, double* sh) {
  v = wsum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += sh[i];
  return t;
}

__global__ void gather_kernel(const imps::GatherEntry* __restrict__ ent, int nent,
                              const double* __restrict__ src, double* __restrict__ dst) {
  const imps::GatherEntry e = ent[blockIdx.x];
  const int64_t n = (int64_t)e.rows * e.cols;
  for (int64_t t = threadIdx.x; t < n; t += blockDim.x) {
    const int i = (int)(t % e.rows), j = (int)(t / e.rows);  // element (i,j) of the block
    const double v = src[e.src_off + t];
    int64_t di, dj;
    if (e.transpose) { di = e.c0 + j; dj = e.r0 + i; } else { di = e.r0 + i; dj = e.c0 + j; }
    dst[e.dst_off + di + dj * e.dst_ld] = v;
  }
}

__global__ void scatter_kernel(const imps::GatherEntry* __restrict__ ent, int nent,
                               const double* __restrict__ dense, double* __restrict__ dst) {
  const imps::GatherEntry e = ent[blockIdx.x];
  const int64_t n = (int64_t)e.rows * e.cols;
  for (int64_t t = threadIdx.x; t < n; t += blockDim.x) {
    const int i = (int)(t % e.rows), j = (int)(t / e.rows);
    int64_t di, dj;
    if (e.transpose) { di = e.c0 + j; dj = e.r0 + i; } else { di = e.r0 + i; dj = e.c0 + j; }
    dst[e.src_off + t] = dense[e.dst_off + di + dj * e.dst_ld];
  }
}

// Step k of the Householder QR of the M x N matrix a (column-major, ld = M): the reflector
// of column k below the diagonal (v[k] = 1 implicit), tau_s[k] its scalar, R's row k on and
// right of the diagonal.
__device__ void householder_step(double* a, int M, int N, int k, double* tau_s, double* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double p = 0.0;
  for (int i = k + threadIdx.x; i < M; i += blockDim.x) p += a[i + (int64_t)k * M] * a[i + (int64_t)k * M];
  const double nrm2 = bsum(p, sh);
  const double x0 = a[k + (int64_t)k * M];
  const double normx = sqrt(nrm2);
  double tau = 0.0, beta = x0, scal = 0.0;
  const double tail2 = nrm2 - x0 * x0;
  if (normx > 0.0 && tail2 > 0.0) {
    beta = -copysign(normx, x0);
    tau = (beta - x0) / beta;
    scal = 1.0 / (x0 - beta);
  }
  __syncthreads();
  if (tau != 0.0)
    for (int i = k + 1 + threadIdx.x; i < M; i += blockDim.x) a[i + (int64_t)k * M] *= scal;
  if (threadIdx.x == 0) { a[k + (int64_t)k * M] = beta; tau_s[k] = tau; }
  __syncthreads();
  if (tau != 0.0) {
    for (int j = k + 1 + warp; j < N; j += nw) {
      double* cj = a + (int64_t)j * M;
      const double* v = a + (int64_t)k * M;
      double w = 0.0;
      for (int i = k + 1 + lane; i < M; i += 32) w += v[i] * cj[i];
      w = wsum(w) + cj[k];
      const double tw = tau * w;
      if (lane == 0) cj[k] -= tw;
      for (int i = k + 1 + lane; i < M; i += 32) cj[i] -= tw * v[i];
    }
  }
  __syncthreads();
}

// Householder QR of the M x N matrix a (in place, column-major, ld = M), K = min(M, N):
// reflectors below the diagonal, R on and above it, tau_s[k] their scalars.
__device__ void householder(double* a, int M, int N, double* tau_s, double* sh) {
  const int K = min(M, N);
  for (int k = 0; k < K; ++k) householder_step(a, M, N, k, tau_s, sh);
}

// Householder QR with column pivoting (A P = Q R, M >= N): before step k the column of largest
// remaining norm (rows k..M-1; the first on ties) is swapped into place; piv[k] = the original
// index of column k.  cn: N doubles of scratch; sel: one shared int.
__device__ void householder_pivoted(double* a, int M, int N, double* tau_s, int* piv, double* cn, double* sh,
                                    int* sel) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int j = threadIdx.x; j < N; j += blockDim.x) piv[j] = j;
  __syncthreads();
  for (int k = 0; k < N; ++k) {
    for (int j = k + warp; j < N; j += nw) {
      const double* cj = a + (int64_t)j * M;
      double t = 0.0;
      for (int i = k + lane; i < M; i += 32) t = fma(cj[i], cj[i], t);
      t = wsum(t);
      if (lane == 0) cn[j] = t;
    }
    __syncthreads();
    if (warp == 0) {
      double best = -1.0;
      int bi = k;
      for (int j = k + lane; j < N; j += 32)
        if (cn[j] > best) { best = cn[j]; bi = j; }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (lane == 0) *sel = bi;
    }
    __syncthreads();
    const int jm = *sel;
    if (jm != k) {
      double* ck = a + (int64_t)k * M;
      double* cm = a + (int64_t)jm * M;
      for (int i = threadIdx.x; i < M; i += blockDim.x) {
        const double t = ck[i];
        ck[i] = cm[i];
        cm[i] = t;
      }
      if (threadIdx.x == 0) {
        const int t = piv[k];
        piv[k] = piv[jm];
        piv[jm] = t;
      }
    }
    __syncthreads();
    householder_step(a, M, N, k, tau_s, sh);
  }
}

// Apply H_0 ... H_{K-1} (reflectors of `a`) to the M x P matrix c (ld M), backwards.
__device__ void apply_reflectors(const double* a, int M, int K, const double* tau_s, double* c, int P) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int k = K - 1; k >= 0; --k) {
    const double tau = tau_s[k];
    if (tau != 0.0) {
      const double* v = a + (int64_t)k * M;
      for (int j = warp; j < P; j += nw) {
        double* cj = c + (int64_t)j * M;
        double w = 0.0;
        for (int i = k + 1 + lane; i < M; i += 32) w += v[i] * cj[i];
        w = wsum(w) + cj[k];
        const double tw = tau * w;
        if (lane == 0) cj[k] -= tw;
        for (int i = k + 1 + lane; i < M; i += 32) cj[i] -= tw * v[i];
      }
    }
    __syncthreads();
  }
}

// Householder QR of the M x N matrix A (in place, column-major, ld = M), K = min(M,N).
// Outputs Q (M x K, ld M) and R (K x N, ld K) with diag(R) >= 0.
__global__ void __launch_bounds__(DT) qr_kernel(const imps::DenseMat* __restrict__ mats,
                                                double* __restrict__ A, double* __restrict__ Q,
                                                double* __restrict__ R, int transpose_out) {
  __shared__ double sh[32];
  __shared__ double tau_s[512];
  const imps::DenseMat mt = mats[blockIdx.x];
  const int M = mt.M, N = mt.N, K = min(M, N);
  double* a = A + mt.a_off;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  householder(a, M, N, tau_s, sh);
  // R (K x N) and the sign of its diagonal
  double* q = Q + mt.q_off;
  double* r = R + mt.r_off;
  __shared__ double sgn[512];
  for (int i = threadIdx.x; i < K; i += blockDim.x) sgn[i] = a[i + (int64_t)i * M] < 0.0 ? -1.0 : 1.0;
  __syncthreads();
  for (int64_t t = threadIdx.x; t < (int64_t)K * N; t += blockDim.x) {
    const int i = (int)(t % K), j = (int)(t / K);
    const double v = (j >= i) ? a[i + (int64_t)j * M] * sgn[i] : 0.0;
    if (transpose_out) r[j + (int64_t)i * N] = v;  // R^T (N x K)
    else r[i + (int64_t)j * K] = v;
  }
  // Q = H_0 ... H_{K-1} [I; 0]   (backward accumulation)
  for (int64_t t = threadIdx.x; t < (int64_t)M * K; t += blockDim.x) {
    const int i = (int)(t % M), j = (int)(t / M);
    q[t] = (i == j) ? 1.0 : 0.0;
  }
  __syncthreads();
  for (int k = K - 1; k >= 0; --k) {
    const double tau = tau_s[k];
    if (tau != 0.0) {
      const double* v = a + (int64_t)k * M;
      for (int j = k + warp; j < K; j += nw) {
        double* cj = q + (int64_t)j * M;
        double w = 0.0;
        for (int i = k + 1 + lane; i < M; i += 32) w += v[i] * cj[i];
        w = wsum(w) + cj[k];
        const double tw = tau * w;
        if (lane == 0) cj[k] -= tw;
        for (int i = k + 1 + lane; i < M; i += 32) cj[i] -= tw * v[i];
      }
    }
    __syncthreads();
  }
  for (int64_t t = threadIdx.x; t < (int64_t)M * K; t += blockDim.x) {
    const int j = (int)(t / M);
    q[t] *= sgn[j];
  }
}

// Left null space of the M x N matrix A (M > N, full column rank; dir l of Nullspace,
// MPSBlockUtilities.hpp:247-300): the last M - N columns of the full Householder Q,
// NS = H_0 ... H_{N-1} [0; I_{M-N}] (M x (M - N), orthonormal, orthogonal to A's columns).
__global__ void __launch_bounds__(DT) nullspace_kernel(const imps::DenseMat* __restrict__ mats,
                                                       double* __restrict__ A, double* __restrict__ NS) {
  __shared__ double sh[32];
  __shared__ double tau_s[512];
  const imps::DenseMat mt = mats[blockIdx.x];
  const int M = mt.M, N = mt.N, P = M - N;
  if (P <= 0) return;
  double* a = A + mt.a_off;
  double* ns = NS + mt.ns_off;
  householder(a, M, N, tau_s, sh);
  for (int64_t t = threadIdx.x; t < (int64_t)M * P; t += blockDim.x) {
    const int i = (int)(t % M), j = (int)(t / M);
    ns[t] = (i == N + j) ? 1.0 : 0.0;
  }
  __syncthreads();
  apply_reflectors(a, M, min(M, N), tau_s, ns, P);
}

// One-sided Jacobi SVD of the M x N matrix held in U (in place, M >= N), in global memory (the
// fallback for N > kJacobiMaxN): on exit U holds the left singular vectors (M x N), S the
// singular values (descending), V the right singular vectors (N x N).  Round-robin pair
// ordering; every warp rotates disjoint column pairs.
__global__ void __launch_bounds__(DT) svd_kernel(const imps::DenseMat* __restrict__ mats,
                                                 double* __restrict__ U, double* __restrict__ S,
                                                 double* __restrict__ V, double* __restrict__ Wk,
                                                 int max_sweeps, int* __restrict__ status) {
  __shared__ int rotated;
  __shared__ int perm[512];
  const imps::DenseMat mt = mats[blockIdx.x];
  const int M = mt.M, N = mt.N;
  double* u = U + mt.q_off;
  double* v = V + mt.r_off;
  double* s = S + mt.s_off;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int64_t t = threadIdx.x; t < (int64_t)N * N; t += blockDim.x)
    v[t] = ((t % N) == (t / N)) ? 1.0 : 0.0;
  const int P = N + (N & 1);  // players (padded to even)
  for (int i = threadIdx.x; i < P; i += blockDim.x) perm[i] = i;
  __syncthreads();
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    if (threadIdx.x == 0) rotated = 0;
    __syncthreads();
    for (int round = 0; round < P - 1; ++round) {
      for (int pr = warp; pr < P / 2; pr += nw) {
        int p = perm[pr], q = perm[P - 1 - pr];
        if (p >= N || q >= N) continue;
        if (p > q) { const int t = p; p = q; q = t; }
        double* cp = u + (int64_t)p * M;
        double* cq = u + (int64_t)q * M;
        double al = 0.0, be = 0.0, ga = 0.0;
        for (int i = lane; i < M; i += 32) {
          const double x = cp[i], y = cq[i];
          al += x * x; be += y * y; ga += x * y;
        }
        al = wsum(al); be = wsum(be); ga = wsum(ga);
        if (fabs(ga) > (double)M * 2.220446049250313e-16 * sqrt(al * be) && ga != 0.0) {
          const double zeta = (be - al) / (2.0 * ga);
          const double t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
          const double c = 1.0 / sqrt(1.0 + t * t), sn = c * t;
          for (int i = lane; i < M; i += 32) {
            const double x = cp[i], y = cq[i];
            cp[i] = c * x - sn * y;
            cq[i] = sn * x + c * y;
          }
          double* vp = v + (int64_t)p * N;
          double* vq = v + (int64_t)q * N;
          for (int i = lane; i < N; i += 32) {
            const double x = vp[i], y = vq[i];
            vp[i] = c * x - sn * y;
            vq[i] = sn * x + c * y;
          }
          if (lane == 0) rotated = 1;
        }
      }
      __syncthreads();
      // rotate players 1..P-1 (player 0 fixed)
      if (threadIdx.x == 0) {
        const int last = perm[P - 1];
        for (int i = P - 1; i > 1; --i) perm[i] = perm[i - 1];
        perm[1] = last;
      }
      __syncthreads();
    }
    const int any = rotated;
    __syncthreads();  // every thread has read the flag before thread 0 resets it
    if (!any) break;
  }
  if (threadIdx.x == 0 && sweep >= max_sweeps && status) atomicExch(status, 1);
  // singular values and normalisation
  double* sv = Wk + mt.w_off;  // N scratch values
  for (int j = warp; j < N; j += nw) {
    const double* c = u + (int64_t)j * M;
    double a2 = 0.0;
    for (int i = lane; i < M; i += 32) a2 += c[i] * c[i];
    a2 = wsum(a2);
    if (lane == 0) sv[j] = sqrt(a2);
  }
  __syncthreads();
  for (int j = warp; j < N; j += nw) {
    double* c = u + (int64_t)j * M;
    const double inv = sv[j] > 0.0 ? 1.0 / sv[j] : 0.0;
    for (int i = lane; i < M; i += 32) c[i] *= inv;
  }
  __syncthreads();
  // order descending (stable selection of ranks), applied by permuting into S and via the
  // rank table; U and V columns are permuted through the scratch area
  if (threadIdx.x == 0) {
    for (int j = 0; j < N; ++j) perm[j] = j;
    for (int a = 1; a < N; ++a) {  // insertion sort on indices by sv descending
      const int key = perm[a];
      int b = a - 1;
      while (b >= 0 && sv[perm[b]] < sv[key]) { perm[b + 1] = perm[b]; --b; }
      perm[b + 1] = key;
    }
  }
  __syncthreads();
  for (int j = threadIdx.x; j < N; j += blockDim.x) s[j] = sv[perm[j]];
  // permute columns of U (M x N) and V (N x N) using Wk as a staging copy
  double* stage = Wk + mt.w_off + N;
  for (int64_t t = threadIdx.x; t < (int64_t)M * N; t += blockDim.x) stage[t] = u[t];
  __syncthreads();
  for (int64_t t = threadIdx.x; t < (int64_t)M * N; t += blockDim.x) {
    const int i = (int)(t % M), j = (int)(t / M);
    u[t] = stage[i + (int64_t)perm[j] * M];
  }
  __syncthreads();
  for (int64_t t = threadIdx.x; t < (int64_t)N * N; t += blockDim.x) stage[t] = v[t];
  __syncthreads();
  for (int64_t t = threadIdx.x; t < (int64_t)N * N; t += blockDim.x) {
    const int i = (int)(t % N), j = (int)(t / N);
    v[t] = stage[i + (int64_t)perm[j] * N];
  }
}

constexpr int JT = 1024;  // threads of the shared-memory SVD kernels
// every column pair of a round has its own lane group (no loop over pairs in jacobi_sweeps)
static_assert((imps::kJacobiMaxN + 1) / 2 <= JT / 2, "FP64 sweeps: one 2-lane group per pair");
static_assert((imps::kMixedMaxN + 1) / 2 <= JT / 16, "FP32 sweeps: one 16-lane group per pair");

// One-sided (Hestenes) Jacobi sweeps on the N columns of B (column-major, ld, shared memory),
// the rotations accumulated into V.  G lanes per column pair split the rows (G = 1: a lane
// owns a pair, so the rotation parameters are computed once per pair, which matters on a GPU
// whose FP64 rate is a few operations per clock per SM); pairs follow the circle round-robin
// schedule in closed form; a pair is rotated while |<b_p, b_q>| > tol |b_p| |b_q|.  Returns the
// number of sweeps run (the last one without rotations), or max_sweeps + 1 if still rotating.
template <typename T, int G>
__device__ int jacobi_sweeps(T* B, T* V, int N, int ld, double tol, int max_sweeps, int* flag) {
  const int P = N + (N & 1);  // players, padded to even; player P-1 stays fixed
  const int k = threadIdx.x / G, gl = threadIdx.x % G;
  const T tl = (T)tol;
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    if (threadIdx.x == 0) *flag = 0;
    __syncthreads();
    for (int r = 0; r < P - 1; ++r) {
      int p = 0, q = N;
      if (k < P / 2) {
        p = k == 0 ? r : (r + k) % (P - 1);
        q = k == 0 ? P - 1 : (r - k + (P - 1)) % (P - 1);
        if (p > q) { const int t = p; p = q; q = t; }
      }
      const bool valid = k < P / 2 && q < N;  // p < q, so q < N implies p < N
      T al = 0, be = 0, ga = 0;
      if (valid) {
        const T* bp = B + (int64_t)p * ld;
        const T* bq = B + (int64_t)q * ld;
        for (int i = gl; i < N; i += G) {
          const T x = bp[i], y = bq[i];
          al = fma(x, x, al);
          be = fma(y, y, be);
          ga = fma(x, y, ga);
        }
      }
#pragma unroll
      for (int o = G / 2; o > 0; o >>= 1) {  // every lane of the warp takes part
        al += __shfl_xor_sync(0xffffffffu, al, o);
        be += __shfl_xor_sync(0xffffffffu, be, o);
        ga += __shfl_xor_sync(0xffffffffu, ga, o);
      }
      if (valid && ga != (T)0 && fabs(ga) > tl * sqrt(al * be)) {
        const T zeta = (be - al) / ((T)2 * ga);
        const T t = copysign((T)1, zeta) / (fabs(zeta) + sqrt((T)1 + zeta * zeta));
        const T c = (T)1 / sqrt((T)1 + t * t), sn = c * t;
        T* bp = B + (int64_t)p * ld;
        T* bq = B + (int64_t)q * ld;
        T* vp = V + (int64_t)p * ld;
        T* vq = V + (int64_t)q * ld;
        for (int i = gl; i < N; i += G) {
          const T x = bp[i], y = bq[i];
          bp[i] = c * x - sn * y;
          bq[i] = sn * x + c * y;
          const T xv = vp[i], yv = vq[i];
          vp[i] = c * xv - sn * yv;
          vq[i] = sn * xv + c * yv;
        }
        if (gl == 0) *flag = 1;
      }
      __syncthreads();
    }
    const int any = *flag;
    __syncthreads();  // every thread has read the flag before thread 0 resets it
    if (!any) return sweep + 1;
  }
  return max_sweeps + 1;
}

// SVD of the M x N sector matrix held in U (M >= N, N <= kJacobiMaxN), with the
// preconditioning of Drmac and Veselic (SIAM J. Matrix Anal. Appl. 29 (2008) 1322): Householder
// QR with column pivoting A P = Q R, then one-sided Jacobi on the columns of X = R^T, which is
// strongly graded and converges in a few sweeps (the unpivoted form needs 15-30 sweeps on
// sectors whose singular values span many decades).  X Vx = Ux S gives R = Vx S Ux^T, so
// U = Q [Vx; 0] and V = P Ux.  MIXED: the first sweeps run in FP32 (many times the FP64 rate
// on this GPU) on a copy of X; their rotations V0 are made orthonormal in FP64 by one
// Cholesky-QR step (V0^T V0 = L L^T, V0 <- V0 L^-T), and FP64 sweeps on B = X V0, accumulating
// into V0, converge quadratically from there.  Either way the last sweep passes the FP64 test
// |<b_p, b_q>| <= N eps |b_p| |b_q| for all pairs.  Outputs as svd_kernel: U (M x N) left
// singular vectors, S descending, V (N x N) right singular vectors.
template <bool MIXED>
__global__ void __launch_bounds__(JT) svd_pjac_kernel(const imps::SvdSets sets, int a_smem, int max_sweeps,
                                                      int* __restrict__ status) {
  extern __shared__ double smem[];
  __shared__ double sh[32];
  __shared__ int flag, sel;
  int bi = blockIdx.x, ks = 0;
  while (ks + 1 < sets.nsets && bi >= sets.s[ks].n) {
    bi -= sets.s[ks].n;
    ++ks;
  }
  const imps::DenseMat mt = sets.s[ks].mats[bi];
  double* __restrict__ U = sets.s[ks].U;
  double* __restrict__ S = sets.s[ks].S;
  double* __restrict__ V = sets.s[ks].V;
  double* __restrict__ Wk = sets.s[ks].W;
  const int M = mt.M, N = mt.N;
  if (N <= 0 || M < N) return;
  const int ld = N | 1;  // odd: lanes owning different columns hit different banks
  const int64_t sq = (int64_t)ld * N;
  double* tau = Wk + mt.w_off;
  double* xs = smem;                       // X = R^T (FP64), rotated into B (FP64-only form)
  double* vs = xs + sq;                    // Vx
  double* tmp = MIXED ? vs + sq : nullptr; // FP32 X and V, then L, then B
  double* sig = (MIXED ? tmp : vs) + sq;
  double* cn = sig + N;
  int* perm = (int*)(cn + N);
  int* piv = perm + N;
  double* a = a_smem ? (double*)(piv + N) : Wk + mt.w_off + N;
  double* u = U + mt.q_off;
  for (int64_t t = threadIdx.x; t < (int64_t)M * N; t += blockDim.x) a[t] = u[t];
  __syncthreads();
  householder_pivoted(a, M, N, tau, piv, cn, sh, &sel);
  for (int t = threadIdx.x; t < N * N; t += blockDim.x) {
    const int i = t % N, j = t / N;
    xs[i + j * ld] = i >= j ? a[j + (int64_t)i * M] : 0.0;  // X = R^T, lower triangular
    vs[i + j * ld] = i == j ? 1.0 : 0.0;
  }
  __syncthreads();
  const double tol = (double)N * 2.220446049250313e-16;
  double* B = xs;
  if (MIXED) {
    float* xf = (float*)tmp;
    float* vf = xf + sq;
    for (int t = threadIdx.x; t < N * N; t += blockDim.x) {
      const int i = t % N, j = t / N;
      xf[i + j * ld] = (float)xs[i + j * ld];
      vf[i + j * ld] = i == j ? 1.0f : 0.0f;
    }
    __syncthreads();
    jacobi_sweeps<float, 16>(xf, vf, N, ld, 1e-5, 8, &flag);
    for (int t = threadIdx.x; t < N * N; t += blockDim.x) {
      const int i = t % N, j = t / N;
      vs[i + j * ld] = (double)vf[i + j * ld];
    }
    __syncthreads();
    // Cholesky-QR: lower triangle of G = V0^T V0 into tmp, G = L L^T in place, V0 <- V0 L^-T
    for (int t = threadIdx.x; t < N * N; t += blockDim.x) {
      const int i = t % N, j = t / N;
      if (i < j) continue;
      const double* ci = vs + (int64_t)i * ld;
      const double* cj = vs + (int64_t)j * ld;
      double g = 0.0;
      for (int r = 0; r < N; ++r) g = fma(ci[r], cj[r], g);
      tmp[i + j * ld] = g;
    }
    __syncthreads();
    for (int kk = 0; kk < N; ++kk) {
      if (threadIdx.x == 0) tmp[kk + kk * ld] = sqrt(fmax(tmp[kk + kk * ld], 1e-300));
      __syncthreads();
      const double dk = tmp[kk + kk * ld];
      for (int i = kk + 1 + threadIdx.x; i < N; i += blockDim.x) tmp[i + kk * ld] /= dk;
      __syncthreads();
      const int rem = N - kk - 1;
      for (int t = threadIdx.x; t < rem * rem; t += blockDim.x) {
        const int i = kk + 1 + t % rem, j = kk + 1 + t / rem;
        if (i >= j) tmp[i + j * ld] -= tmp[i + kk * ld] * tmp[j + kk * ld];
      }
      __syncthreads();
    }
    for (int r = threadIdx.x; r < N; r += blockDim.x) {  // row r of V0: x L^T = V0[r, :]
      for (int j = 0; j < N; ++j) {
        double x = vs[r + j * ld];
        for (int kk = 0; kk < j; ++kk) x = fma(-vs[r + kk * ld], tmp[j + kk * ld], x);
        vs[r + j * ld] = x / tmp[j + j * ld];
      }
    }
    __syncthreads();
    // B = X V0 (X lower triangular) into tmp
    for (int t = threadIdx.x; t < N * N; t += blockDim.x) {
      const int i = t % N, j = t / N;
      const double* vj = vs + (int64_t)j * ld;
      double b = 0.0;
      for (int kk = 0; kk <= i; ++kk) b = fma(xs[i + kk * ld], vj[kk], b);
      tmp[i + j * ld] = b;
    }
    __syncthreads();
    B = tmp;
  }
  const int sw = jacobi_sweeps<double, 2>(B, vs, N, ld, tol, max_sweeps, &flag);
  if (threadIdx.x == 0 && sw > max_sweeps && status) atomicExch(status, 1);
  // singular values, descending (ties by index)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int j = warp; j < N; j += nw) {
    const double* c = B + (int64_t)j * ld;
    double a2 = 0.0;
    for (int i = lane; i < N; i += 32) a2 = fma(c[i], c[i], a2);
    a2 = wsum(a2);
    if (lane == 0) sig[j] = sqrt(a2);
  }
  __syncthreads();
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    int rk = 0;
    for (int i = 0; i < N; ++i) rk += (sig[i] > sig[j] || (sig[i] == sig[j] && i < j)) ? 1 : 0;
    perm[rk] = j;
  }
  __syncthreads();
  double* s_out = S + mt.s_off;
  double* v_out = V + mt.r_off;
  for (int j = threadIdx.x; j < N; j += blockDim.x) s_out[j] = sig[perm[j]];
  for (int t = threadIdx.x; t < N * N; t += blockDim.x) {  // V = P Ux: row piv[i] of V = row i of Ux
    const int i = t % N, j = t / N;
    const int pj = perm[j];
    v_out[piv[i] + (int64_t)j * N] = sig[pj] > 0.0 ? B[i + (int64_t)pj * ld] / sig[pj] : 0.0;
  }
  for (int64_t t = threadIdx.x; t < (int64_t)M * N; t += blockDim.x) {  // U = Q [Vx; 0]
    const int i = (int)(t % M), j = (int)(t / M);
    u[t] = i < N ? vs[i + (int64_t)perm[j] * ld] : 0.0;
  }
  __syncthreads();
  apply_reflectors(a, M, N, tau, u, N);
}

// Y = X (M x N) transposed into (N x M), per matrix (used for V^T outputs)
__global__ void transpose_kernel(const imps::DenseMat* __restrict__ mats, const double* __restrict__ X,
                                 double* __restrict__ Y, int use_r) {
  const imps::DenseMat mt = mats[blockIdx.x];
  const int n = mt.N;
  const double* x = X + mt.r_off;
  double* y = Y + mt.r_off;
  for (int64_t t = threadIdx.x; t < (int64_t)n * n; t += blockDim.x) {
    const int i = (int)(t % n), j = (int)(t / n);
    y[j + (int64_t)i * n] = x[t];
  }
  (void)use_r;
}

// X_q[:, j] *= S_q[j]^power for square sector blocks (BlockDiagMat << BlockLam,
// BlockObj.hpp:2316 with lam = S^power)
__global__ void colscale_kernel(const imps::DenseMat* __restrict__ mats, double* __restrict__ X,
                                const double* __restrict__ S, double power) {
  const imps::DenseMat mt = mats[blockIdx.x];
  const int n = mt.N;
  double* x = X + mt.r_off;
  const double* s = S + mt.s_off;
  for (int64_t t = threadIdx.x; t < (int64_t)n * n; t += blockDim.x) {
    const int j = (int)(t / n);
    x[t] *= pow(s[j], power);
  }
}

}  // namespace

namespace imps {

int dc_colscale(const DenseMat* d_mats, int nmat, double* X, const double* S, double power, cudaStream_t st) {
  if (nmat > 0) imps::count_launch();
  if (nmat > 0) colscale_kernel<<<nmat, 256, 0, st>>>(d_mats, X, S, power);
  return cudaGetLastError() == cudaSuccess ? IMPS_OK : IMPS_ERR_CUDA;
}

int dc_gather(const GatherEntry* d_ent, int nent, const double* src, double* dense, cudaStream_t st) {
  if (nent > 0) imps::count_launch();
  if (nent > 0) gather_kernel<<<nent, 256, 0, st>>>(d_ent, nent, src, dense);
  return cudaGetLastError() == cudaSuccess ? IMPS_OK : IMPS_ERR_CUDA;
}

int dc_scatter(const GatherEntry* d_ent, int nent, const double* dense, double* dst, cudaStream_t st) {
  if (nent > 0) imps::count_launch();
  if (nent > 0) scatter_kernel<<<nent, 256, 0, st>>>(d_ent, nent, dense, dst);
  return cudaGetLastError() == cudaSuccess ? IMPS_OK : IMPS_ERR_CUDA;
}

int dc_qr(const DenseMat* d_mats, int nmat, double* A, double* Q, double* R, int transpose_r, cudaStream_t st) {
  if (nmat > 0) imps::count_launch();
  if (nmat > 0) qr_kernel<<<nmat, DT, 0, st>>>(d_mats, A, Q, R, transpose_r);
  return cudaGetLastError() == cudaSuccess ? IMPS_OK : IMPS_ERR_CUDA;
}

int dc_nullspace(const DenseMat* d_mats, int nmat, double* A, double* NS, cudaStream_t st) {
  if (nmat <= 0) return IMPS_OK;
  imps::count_launch();
  nullspace_kernel<<<nmat, DT, 0, st>>>(d_mats, A, NS);
  return cudaGetLastError() == cudaSuccess ? IMPS_OK : IMPS_ERR_CUDA;
}

int dc_svd(const DenseMat* d_mats, int nmat, int maxN, int64_t maxMN, double* U, double* S, double* V, double* W,
           int* status, cudaStream_t st) {
  SvdSets sets{};
  sets.nsets = 1;
  sets.s[0] = SvdSet{d_mats, U, S, V, W, nmat};
  return dc_svd_sets(sets, maxN, maxMN, status, st);
}

int dc_svd_sets(const SvdSets& sets, int maxN, int64_t maxMN, int* status, cudaStream_t st) {
  if (sets.nsets < 1 || sets.nsets > kSvdSets) return IMPS_ERR_BAD_ARG;
  int nmat = 0;
  for (int k = 0; k < sets.nsets; ++k) nmat += sets.s[k].n;
  if (nmat <= 0) return IMPS_OK;
  if (maxN > kJacobiMaxN) {  // global-memory fallback, one launch per set
    for (int k = 0; k < sets.nsets; ++k) {
      if (sets.s[k].n <= 0) continue;
      imps::count_launch();
      svd_kernel<<<sets.s[k].n, DT, 0, st>>>(sets.s[k].mats, sets.s[k].U, sets.s[k].S, sets.s[k].V, sets.s[k].W,
                                             40, status);
    }
    return cudaGetLastError() == cudaSuccess ? IMPS_OK : IMPS_ERR_CUDA;
  }
  imps::count_launch();
  constexpr size_t kSmemMax = 226 * 1024;  // dynamic part; the static flags and sums take < 1 KB
  const bool mixed = maxN <= kMixedMaxN;
  const int64_t ld = maxN | 1;
  const size_t base = ((size_t)(mixed ? 3 : 2) * ld * maxN + 2 * (size_t)maxN) * 8 + (size_t)2 * maxN * 4 + 16;
  const int a_smem = base + (size_t)maxMN * 8 <= kSmemMax ? 1 : 0;
  const size_t bytes = base + (a_smem ? (size_t)maxMN * 8 : 0);
  if (bytes > kSmemMax) return IMPS_ERR_TOO_LARGE;
  static bool attr_set = false;
  if (!attr_set) {
    if (cudaFuncSetAttribute(svd_pjac_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemMax) !=
            cudaSuccess ||
        cudaFuncSetAttribute(svd_pjac_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemMax) !=
            cudaSuccess)
      return IMPS_ERR_CUDA;
    attr_set = true;
  }
  if (mixed) svd_pjac_kernel<true><<<nmat, JT, bytes, st>>>(sets, a_smem, 20, status);
  else svd_pjac_kernel<false><<<nmat, JT, bytes, st>>>(sets, a_smem, 30, status);
  return cudaGetLastError() == cudaSuccess ? IMPS_OK : IMPS_ERR_CUDA;
}

int dc_transpose_sq(const DenseMat* d_mats, int nmat, const double* X, double* Y, cudaStream_t st) {
  if (nmat > 0) imps::count_launch();
  if (nmat > 0) transpose_kernel<<<nmat, 256, 0, st>>>(d_mats, X, Y, 1);
  return cudaGetLastError() == cudaSuccess ? IMPS_OK : IMPS_ERR_CUDA;
}

}  // namespace imps
