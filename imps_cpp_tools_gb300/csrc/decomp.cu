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

// Householder QR of the M x N matrix a (in place, column-major, ld = M), K = min(M, N):
// reflectors below the diagonal, R on and above it, tau_s[k] their scalars.
__device__ void householder(double* a, int M, int N, double* tau_s, double* sh) {
  const int K = min(M, N);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int k = 0; k < K; ++k) {
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

// One-sided Jacobi SVD of the M x N matrix held in U (in place, M >= N): on exit U holds the
// left singular vectors (M x N), S the singular values (descending), V the right singular
// vectors (N x N).  Round-robin pair ordering; every warp rotates disjoint column pairs.
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
        if (fabs(ga) > 1e-15 * sqrt(al * be) && ga != 0.0) {
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
    if (!rotated) break;
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

int dc_svd(const DenseMat* d_mats, int nmat, double* U, double* S, double* V, double* W, int* status,
           cudaStream_t st) {
  if (nmat > 0) imps::count_launch();
  if (nmat > 0) svd_kernel<<<nmat, DT, 0, st>>>(d_mats, U, S, V, W, 40, status);
  return cudaGetLastError() == cudaSuccess ? IMPS_OK : IMPS_ERR_CUDA;
}

int dc_transpose_sq(const DenseMat* d_mats, int nmat, const double* X, double* Y, cudaStream_t st) {
  if (nmat > 0) imps::count_launch();
  if (nmat > 0) transpose_kernel<<<nmat, 256, 0, st>>>(d_mats, X, Y, 1);
  return cudaGetLastError() == cudaSuccess ? IMPS_OK : IMPS_ERR_CUDA;
}

}  // namespace imps
