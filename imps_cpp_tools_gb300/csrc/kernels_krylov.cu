// Krylov-space kernels (FP64 always): dot products, CGS2 projections, norms, scaling and the
// small sequential steps of GMRES (Givens rotations) kept on the device so that an iteration
// needs no host round trip.  Reductions use a fixed grid and a last-block finisher, so every
// result is bitwise reproducible run to run (no floating-point atomics).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>

#include "imps_krylov.h"
#include "imps_status.h"

namespace {

constexpr int RB = 256;      // threads per reduction block
constexpr int RGRID = 128;   // fixed reduction grid of multidot (RGRID * kMaxCols partials)
constexpr int CGRID = 152;   // max grid of the fused CGS2 kernels (one block per SM)
constexpr int CSUB = 1024;   // rows of w staged in shared memory per CGS2 sub-chunk

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum; result valid in thread 0.
__device__ double block_sum(double v, double* sh) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
  if (w == 0) v = warp_sum(v);
  __syncthreads();
  return v;
}

// h[c] = scale_c * sum_r V[r + c*ldv] * w[r], c = 0..ncols-1 (ncols <= kMaxCols).
// mode 0: h = result; mode 1: h += result.  Also optional out_norm = sqrt(h[0]) when
// V == w and ncols == 1 (norm use).
__global__ void __launch_bounds__(RB) multidot_kernel(const double* __restrict__ V, int64_t ldv,
                                                      int ncols, const double* __restrict__ w,
                                                      int64_t n, double* __restrict__ partials,
                                                      unsigned int* __restrict__ counter,
                                                      double* __restrict__ h, int mode,
                                                      double* __restrict__ out_sqrt) {
  __shared__ double sh[32];
  __shared__ bool last;
  for (int c = 0; c < ncols; ++c) {
    const double* v = V + c * ldv;
    double acc = 0.0;
    for (int64_t r = (int64_t)blockIdx.x * RB + threadIdx.x; r < n; r += (int64_t)gridDim.x * RB)
      acc = fma(v[r], w[r], acc);
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) partials[c * RGRID + blockIdx.x] = acc;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned int prev = atomicAdd(counter, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  for (int c = 0; c < ncols; ++c) {
    double v = threadIdx.x < gridDim.x ? ((volatile double*)partials)[c * RGRID + threadIdx.x] : 0.0;
    v = block_sum(v, sh);
    if (threadIdx.x == 0) {
      h[c] = mode ? h[c] + v : v;
      if (out_sqrt && c == 0) *out_sqrt = sqrt(v);
    }
  }
  if (threadIdx.x == 0) *counter = 0u;
}

// One fused pass of classical Gram-Schmidt over the basis V[:, 0..nc-1] (nc <= kMaxCols):
//   MODE 0:  h = V^T w
//   MODE 1:  w -= V hin;  h = V^T w;  hacc += h      (second CGS pass)
//   MODE 2:  w -= V hin;  *hout = |w|
// At most one block per SM (CT threads); each walks sub-chunks of <= CSUB rows (grid-stride).
// The (updated) rows of w are staged in shared memory, then warps take groups of 4 columns and
// lanes stride the rows, so V is read coalesced and the chunk just read for the update is
// re-read from L2.  Per-block column sums go to partials[c * gridDim.x + block]; the last
// block to finish reduces them in a fixed order (bitwise reproducible), with L2 loads unrolled
// four deep so that the tail is one round of latency per column group, and resets the counter.
constexpr int CT = 512;
// Batched over systems (blockIdx.y = system): every pointer advances by its stride per system
// (sV for V, sw for w, s_in / s_out / s_acc for hin / hout / hacc, sp for partials, one counter
// each); the single-system launches pass zero strides and one grid row.
template <int MODE>
__global__ void __launch_bounds__(CT) cgs_pass_kernel(const double* __restrict__ V, int64_t ldv, int nc,
                                                     double* __restrict__ w, int64_t n, int sub,
                                                     const double* hin, double* hout, double* hacc,
                                                     double* __restrict__ partials,
                                                     unsigned int* __restrict__ counter, int64_t sV = 0,
                                                     int64_t sw = 0, int64_t s_in = 0, int64_t s_out = 0,
                                                     int64_t s_acc = 0, int64_t sp = 0) {
  {
    const int64_t sy = blockIdx.y;
    V += sy * sV;
    w += sy * sw;
    if (hin) hin += sy * s_in;
    hout += sy * s_out;
    if (hacc) hacc += sy * s_acc;
    partials += sy * sp;
    counter += sy;
  }
  __shared__ double wsm[CSUB];
  __shared__ double hs[imps::kMaxCols];
  __shared__ double sacc[imps::kMaxCols];
  __shared__ double sh[32];
  __shared__ bool last;
  constexpr int NW = CT / 32;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (MODE != 0)
    for (int c = threadIdx.x; c < nc; c += blockDim.x) hs[c] = hin[c];
  for (int c = threadIdx.x; c < imps::kMaxCols; c += blockDim.x) sacc[c] = 0.0;
  double nacc = 0.0;
  __syncthreads();
  for (int64_t base = (int64_t)blockIdx.x * sub; base < n; base += (int64_t)gridDim.x * sub) {
    const int len = (int)min((int64_t)sub, n - base);
    for (int t = threadIdx.x; t < len; t += blockDim.x) {
      const int64_t r = base + t;
      double x = w[r];
      if (MODE != 0) {
        const double* vr = V + r;
        double a[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        int c = 0;
        for (; c + 8 <= nc; c += 8) {
#pragma unroll
          for (int q = 0; q < 8; ++q) a[q] = fma(-vr[(int64_t)(c + q) * ldv], hs[c + q], a[q]);
        }
        for (; c < nc; ++c) a[0] = fma(-vr[(int64_t)c * ldv], hs[c], a[0]);
        x += ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
        w[r] = x;
      }
      if (MODE == 2) nacc = fma(x, x, nacc);
      else wsm[t] = x;
    }
    if (MODE == 2) continue;
    __syncthreads();
    for (int c0 = warp * 4; c0 < nc; c0 += 4 * NW) {
      // columns past nc read column nc-1 (valid memory) and are discarded
      const double* v0 = V + base + (int64_t)min(c0, nc - 1) * ldv;
      const double* v1 = V + base + (int64_t)min(c0 + 1, nc - 1) * ldv;
      const double* v2 = V + base + (int64_t)min(c0 + 2, nc - 1) * ldv;
      const double* v3 = V + base + (int64_t)min(c0 + 3, nc - 1) * ldv;
      double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
      for (int t = lane; t < len; t += 32) {
        const double x = wsm[t];
        a0 = fma(v0[t], x, a0);
        a1 = fma(v1[t], x, a1);
        a2 = fma(v2[t], x, a2);
        a3 = fma(v3[t], x, a3);
      }
      a0 = warp_sum(a0);
      a1 = warp_sum(a1);
      a2 = warp_sum(a2);
      a3 = warp_sum(a3);
      if (lane == 0) {
        sacc[c0] += a0;
        if (c0 + 1 < nc) sacc[c0 + 1] += a1;
        if (c0 + 2 < nc) sacc[c0 + 2] += a2;
        if (c0 + 3 < nc) sacc[c0 + 3] += a3;
      }
    }
    __syncthreads();
  }
  const int G = gridDim.x;
  if (MODE == 2) {
    nacc = block_sum(nacc, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = nacc;
  } else {
    __syncthreads();
    for (int c = threadIdx.x; c < nc; c += blockDim.x) partials[(int64_t)c * G + blockIdx.x] = sacc[c];
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(counter, 1u) == (unsigned)G - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  // partials written by other blocks: read through L2 (__ldcg), never a stale L1 line
  if (MODE == 2) {
    double v = 0.0;
    for (int b = threadIdx.x; b < G; b += blockDim.x) v += __ldcg(partials + b);
    v = block_sum(v, sh);
    if (threadIdx.x == 0) *hout = sqrt(v);
  } else {
    for (int c = warp; c < nc; c += NW) {
      const double* pc = partials + (int64_t)c * G;
      double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
      int b = lane;
      for (; b + 96 < G; b += 128) {
        s0 += __ldcg(pc + b);
        s1 += __ldcg(pc + b + 32);
        s2 += __ldcg(pc + b + 64);
        s3 += __ldcg(pc + b + 96);
      }
      for (; b < G; b += 32) s0 += __ldcg(pc + b);
      double v = warp_sum((s0 + s1) + (s2 + s3));
      if (lane == 0) {
        hout[c] = v;
        if (MODE == 1) hacc[c] += v;
      }
    }
  }
  if (threadIdx.x == 0) *counter = 0u;
}

// ---- single-launch CGS2 step (cooperative grid, all blocks co-resident) ----------------------
// Block b owns rows [b*sub, (b+1)*sub) of w (sub <= COOP_SUB), kept in shared memory through the
// three passes.  Each reduction is one grid barrier: every block writes its per-column partial
// sums, then every block sums all partials itself in the same fixed order (identical,
// reproducible results in every block).  Barrier waits are bounded: on timeout *err is set, the
// remaining work is skipped, and the exit protocol still resets the counters.
constexpr int COOP_SUB = 2048;

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned int* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// arrival counter sync[0] grows by gridDim.x per barrier; target = k * gridDim.x at barrier k
__device__ bool grid_barrier(unsigned int* sync, unsigned target, int* err, bool ok) {
  __shared__ int good;
  __syncthreads();
  if (threadIdx.x == 0) {
    int g = ok ? 1 : 0;
    __threadfence();
    atomicAdd(sync, 1u);
    if (g) {
      for (long long it = 0; ld_acquire_u32(sync) < target; ++it) {
        if (it > (1ll << 22) || *(volatile int*)err) {
          atomicExch(err, 1);
          g = 0;
          break;
        }
        __nanosleep(32);
      }
    }
    good = g;
  }
  __syncthreads();
  return good != 0;
}

// dst[c] = sum_b P[c*G + b] for c < nc (warps over columns, lanes over blocks, L2 loads)
__device__ void reduce_partials(const double* P, int G, int nc, double* dst) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int c = warp; c < nc; c += nw) {
    const double* pc = P + (int64_t)c * G;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int b = lane;
    for (; b + 96 < G; b += 128) {
      s0 += __ldcg(pc + b);
      s1 += __ldcg(pc + b + 32);
      s2 += __ldcg(pc + b + 64);
      s3 += __ldcg(pc + b + 96);
    }
    for (; b < G; b += 32) s0 += __ldcg(pc + b);
    const double v = warp_sum((s0 + s1) + (s2 + s3));
    if (lane == 0) dst[c] = v;
  }
}

// P[c*G + block] = sum_{t < len} Vb[t + c*ldv] * x[t]  (x in shared memory)
__device__ void block_dots(const double* __restrict__ Vb, int64_t ldv, int nc, const double* x, int len,
                           double* P, int G) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int c0 = warp * 4; c0 < nc; c0 += 4 * nw) {
    const double* v0 = Vb + (int64_t)min(c0, nc - 1) * ldv;
    const double* v1 = Vb + (int64_t)min(c0 + 1, nc - 1) * ldv;
    const double* v2 = Vb + (int64_t)min(c0 + 2, nc - 1) * ldv;
    const double* v3 = Vb + (int64_t)min(c0 + 3, nc - 1) * ldv;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
#pragma unroll 2
    for (int t = lane; t < len; t += 32) {
      const double xt = x[t];
      a0 = fma(v0[t], xt, a0);
      a1 = fma(v1[t], xt, a1);
      a2 = fma(v2[t], xt, a2);
      a3 = fma(v3[t], xt, a3);
    }
    a0 = warp_sum(a0);
    a1 = warp_sum(a1);
    a2 = warp_sum(a2);
    a3 = warp_sum(a3);
    if (lane == 0) {
      P[(int64_t)c0 * G + blockIdx.x] = a0;
      if (c0 + 1 < nc) P[(int64_t)(c0 + 1) * G + blockIdx.x] = a1;
      if (c0 + 2 < nc) P[(int64_t)(c0 + 2) * G + blockIdx.x] = a2;
      if (c0 + 3 < nc) P[(int64_t)(c0 + 3) * G + blockIdx.x] = a3;
    }
  }
}

// x[t] -= sum_c Vb[t + c*ldv] * hs[c]
__device__ void update_rows(const double* __restrict__ Vb, int64_t ldv, int nc, const double* hs, double* x,
                            int len) {
  for (int t = threadIdx.x; t < len; t += blockDim.x) {
    const double* vr = Vb + t;
    double a[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    int c = 0;
    for (; c + 8 <= nc; c += 8) {
#pragma unroll
      for (int q = 0; q < 8; ++q) a[q] = fma(-vr[(int64_t)(c + q) * ldv], hs[c + q], a[q]);
    }
    for (; c < nc; ++c) a[0] = fma(-vr[(int64_t)c * ldv], hs[c], a[0]);
    x[t] += ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
  }
}

// c_loc: the first pass projects out columns c_loc..nc-1 only (Lanczos: the two columns the
// three-term recurrence couples w to; 0 = all columns); the second pass is always full.
__global__ void __launch_bounds__(CT) cgs2_coop_kernel(const double* __restrict__ V, int64_t ldv, int nc,
                                                      double* __restrict__ w, int64_t n, int sub, double* h,
                                                      double* __restrict__ vnext, int* flag,
                                                      double* __restrict__ partials, unsigned int* sync,
                                                      int* err, int c_loc) {
  __shared__ double wsm[COOP_SUB];
  __shared__ double h1[imps::kMaxCols];
  __shared__ double h2[imps::kMaxCols + 1];
  __shared__ double sh[32];
  __shared__ double beta;
  const int G = gridDim.x;
  const int64_t base = (int64_t)blockIdx.x * sub;
  const int len = (int)max((int64_t)0, min((int64_t)sub, n - base));
  const double* Vb = V + base;
  double* P0 = partials;
  double* P1 = partials + (int64_t)G * imps::kMaxCols;
  double* P2 = P1 + (int64_t)G * imps::kMaxCols;
  bool ok = true;
  for (int t = threadIdx.x; t < len; t += blockDim.x) wsm[t] = w[base + t];
  for (int c = threadIdx.x; c < c_loc; c += blockDim.x) h1[c] = 0.0;
  __syncthreads();
  // pass 1: h1 = V^T w over columns c_loc..nc-1
  const int nloc = nc - c_loc;
  const double* Vloc = Vb + (int64_t)c_loc * ldv;
  block_dots(Vloc, ldv, nloc, wsm, len, P0, G);
  ok = grid_barrier(sync, (unsigned)G, err, ok);
  if (ok) reduce_partials(P0, G, nloc, h1 + c_loc);
  __syncthreads();
  // pass 2: w -= V h1; h2 = V^T w
  if (ok) {
    update_rows(Vloc, ldv, nloc, h1 + c_loc, wsm, len);
    __syncthreads();
    block_dots(Vb, ldv, nc, wsm, len, P1, G);
  }
  // |w|^2 before the second update rides along as column nc of the same partials
  {
    double n1 = 0.0;
    if (ok)
      for (int t = threadIdx.x; t < len; t += blockDim.x) n1 = fma(wsm[t], wsm[t], n1);
    n1 = block_sum(n1, sh);
    if (threadIdx.x == 0) P1[(int64_t)nc * G + blockIdx.x] = n1;
  }
  ok = grid_barrier(sync, 2u * G, err, ok);
  if (ok) reduce_partials(P1, G, nc + 1, h2);  // h2[nc] = |w1|^2
  __syncthreads();
  // pass 3: w -= V h2; beta = |w|.  V orthonormal: |w2|^2 = |w1|^2 - |h2|^2 exactly, and the
  // second-pass coefficients are tiny unless w1 nearly lies in span(V); then (identically in
  // every block, which all hold the same reduced values) the norm is reduced explicitly.
  __shared__ bool pyth;
  if (threadIdx.x == 0) {
    double s2 = 0.0;
    for (int c = 0; c < nc; ++c) s2 = fma(h2[c], h2[c], s2);
    pyth = s2 <= 0.1 * h2[nc];
    if (pyth) beta = sqrt(h2[nc] - s2);
  }
  __syncthreads();
  if (ok) update_rows(Vb, ldv, nc, h2, wsm, len);
  __syncthreads();
  if (!pyth) {
    double nacc = 0.0;
    if (ok)
      for (int t = threadIdx.x; t < len; t += blockDim.x) nacc = fma(wsm[t], wsm[t], nacc);
    nacc = block_sum(nacc, sh);
    if (threadIdx.x == 0) P2[blockIdx.x] = nacc;
    ok = grid_barrier(sync, 3u * G, err, ok);
    if (ok) reduce_partials(P2, G, 1, sh);  // warp 0 writes sh[0]
    __syncthreads();
    if (threadIdx.x == 0 && ok) beta = sqrt(sh[0]);
  }
  if (ok) {
    __syncthreads();
    const double bt = beta;
    const bool bad = !(fabs(bt) > 1e-300) || !isfinite(bt);
    const double inv = bad ? 0.0 : 1.0 / bt;
    for (int t = threadIdx.x; t < len; t += blockDim.x) {
      w[base + t] = wsm[t];
      vnext[base + t] = wsm[t] * inv;
    }
    if (blockIdx.x == 0) {
      for (int c = threadIdx.x; c < nc; c += blockDim.x) h[c] = h1[c] + h2[c];
      if (threadIdx.x == 0) {
        h[nc] = bt;
        if (bad && flag) *flag = 1;
      }
    }
  }
  // exit: the last block out resets both counters (every block has passed every barrier)
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(sync + 1, 1u) == (unsigned)G - 1) {
      sync[0] = 0u;
      sync[1] = 0u;
      __threadfence();
    }
  }
}

// w[r] -= sum_c V[r + c*ldv] * h[c]
__global__ void gemv_sub_kernel(const double* __restrict__ V, int64_t ldv, int ncols,
                                const double* __restrict__ h, double* __restrict__ w, int64_t n) {
  __shared__ double hs[imps::kMaxCols];
  for (int c = threadIdx.x; c < ncols; c += blockDim.x) hs[c] = h[c];
  __syncthreads();
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x) {
    double acc = w[r];
    for (int c = 0; c < ncols; ++c) acc = fma(-V[r + c * ldv], hs[c], acc);
    w[r] = acc;
  }
}

// y[r] = sum_c V[r + c*ldv] * h[c]
__global__ void gemv_kernel(const double* __restrict__ V, int64_t ldv, int ncols,
                            const double* __restrict__ h, double* __restrict__ y, int64_t n) {
  __shared__ double hs[imps::kMaxCols];
  for (int c = threadIdx.x; c < ncols; c += blockDim.x) hs[c] = h[c];
  __syncthreads();
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int c = 0; c < ncols; ++c) acc = fma(V[r + c * ldv], hs[c], acc);
    y[r] = acc;
  }
}

// y = x / *nrm  (guarded: a zero norm writes zeros and raises the breakdown flag)
// out[:, t] = sum_i V[:, i] * W[i + t*m] for t < kk (column-major W, m <= kMaxCols): the
// basis rotation of a thick restart, one pass over V per 16 output columns (V stays in L2).
__global__ void __launch_bounds__(256) basis_rotate_kernel(const double* __restrict__ V, int64_t ldv,
                                                           int m, const double* __restrict__ W, int kk,
                                                           double* __restrict__ out, int64_t ldo,
                                                           int64_t n) {
  constexpr int CT = 16;
  __shared__ double ws[imps::kMaxCols * CT];
  for (int t0 = 0; t0 < kk; t0 += CT) {
    const int nt = min(CT, kk - t0);
    __syncthreads();
    for (int e = threadIdx.x; e < m * CT; e += blockDim.x) {
      const int i = e / CT, t = e % CT;
      ws[e] = t < nt ? W[i + (int64_t)(t0 + t) * m] : 0.0;
    }
    __syncthreads();
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
         r += (int64_t)gridDim.x * blockDim.x) {
      double acc[CT];
#pragma unroll
      for (int t = 0; t < CT; ++t) acc[t] = 0.0;
      int i = 0;
      for (; i + 8 <= m; i += 8) {  // eight loads in flight per thread
        double v[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) v[q] = V[r + (int64_t)(i + q) * ldv];
#pragma unroll
        for (int q = 0; q < 8; ++q)
#pragma unroll
          for (int t = 0; t < CT; ++t) acc[t] = fma(v[q], ws[(i + q) * CT + t], acc[t]);
      }
      for (; i < m; ++i) {
        const double v = V[r + (int64_t)i * ldv];
#pragma unroll
        for (int t = 0; t < CT; ++t) acc[t] = fma(v, ws[i * CT + t], acc[t]);
      }
#pragma unroll
      for (int t = 0; t < CT; ++t)
        if (t < nt) out[r + (int64_t)(t0 + t) * ldo] = acc[t];
    }
  }
}

__global__ void scale_inv_kernel(const double* __restrict__ x, const double* __restrict__ nrm,
                                 double* __restrict__ y, int64_t n, int* __restrict__ flag, int64_t sx = 0,
                                 int64_t sn = 0, int64_t sy = 0) {
  {  // batched: blockIdx.y = system (x, nrm, y, flag advance by their strides)
    const int64_t q = blockIdx.y;
    x += q * sx;
    nrm += q * sn;
    y += q * sy;
    if (flag) flag += q;
  }
  const double s = *nrm;
  const bool bad = !(fabs(s) > 1e-300) || !isfinite(s);
  if (bad && flag && blockIdx.x == 0 && threadIdx.x == 0) *flag = 1;
  const double inv = bad ? 0.0 : 1.0 / s;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x)
    y[r] = x[r] * inv;
}

// y = a*x + b*y with host scalars
__global__ void axpby_kernel(double a, const double* __restrict__ x, double b, double* __restrict__ y,
                             int64_t n) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x)
    y[r] = a * x[r] + b * y[r];
}

// y = x - t + (*s) * rho   (InvEfun_proj epilogue, InvEBlockFunctions.hpp:40-44)
__global__ void proj_epilogue_kernel(const double* __restrict__ x, const double* __restrict__ t,
                                     const double* __restrict__ s, const double* __restrict__ rho,
                                     double* __restrict__ y, int64_t n) {
  const double sc = *s;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x)
    y[r] = x[r] + sc * rho[r] - t[r];
}

// sum over blocks q of trace(X_q * R_q) = sum_{i,j} X_q[i + j m] * R_q[j + i m]
// sum_b tr(X_b R_b): X_b is rows x cols at boff[b], R_b the cols x rows block at the same
// offset (blocks paired in order; bcols == nullptr: square blocks).  A flat grid-stride loop
// over all elements (about one per thread: the loads are independent, so the transposed R
// reads do not form a latency chain); each element finds its block by binary search over the
// block offsets, cached in shared memory.  Partial sums are combined in a fixed order by the
// last CTA to finish (gridDim.x <= RB).
constexpr int kTraceCache = 1024;
__global__ void __launch_bounds__(RB) trace_prod_kernel(const double* __restrict__ X,
                                                        const double* __restrict__ R,
                                                        const int64_t* __restrict__ boff,
                                                        const int32_t* __restrict__ bdim,
                                                        const int32_t* __restrict__ bcols, int nb,
                                                        double* __restrict__ partials,
                                                        unsigned int* __restrict__ counter,
                                                        double* __restrict__ out) {
  __shared__ int64_t so[kTraceCache];
  __shared__ int32_t sm[kTraceCache], sc[kTraceCache];
  __shared__ double sh[32];
  __shared__ bool last;
  const bool cached = nb <= kTraceCache;
  if (cached)
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
      so[b] = boff[b];
      sm[b] = bdim[b];
      sc[b] = bcols ? bcols[b] : bdim[b];
    }
  __syncthreads();
  auto off = [&](int b) -> int64_t { return cached ? so[b] : boff[b]; };
  auto rows = [&](int b) -> int { return cached ? sm[b] : bdim[b]; };
  auto cols = [&](int b) -> int { return cached ? sc[b] : (bcols ? bcols[b] : bdim[b]); };
  double acc = 0.0;
  if (nb > 0) {
    const int64_t ntot = off(nb - 1) + (int64_t)rows(nb - 1) * cols(nb - 1);
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ntot;
         e += (int64_t)gridDim.x * blockDim.x) {
      // the last block starting at or before e (a later block at the same offset is the one
      // that is not empty)
      int lo = 0, hi = nb - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (off(mid) <= e) lo = mid;
        else hi = mid - 1;
      }
      const int m = rows(lo), nc = cols(lo);
      const int64_t o = off(lo);
      const int t = (int)(e - o);
      const int i = t % m, j = t / m;
      acc = fma(X[e], R[o + j + (int64_t)i * nc], acc);
    }
  }
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = acc;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  double v = threadIdx.x < gridDim.x ? ((volatile double*)partials)[threadIdx.x] : 0.0;
  v = block_sum(v, sh);
  if (threadIdx.x == 0) { *out = v; *counter = 0u; }
}

// sum of squares over a list of segments (off, len) -> *out (plain sum, no sqrt)
__global__ void __launch_bounds__(RB) segsq_kernel(const double* __restrict__ X,
                                                   const int64_t* __restrict__ soff,
                                                   const int64_t* __restrict__ slen, int ns,
                                                   double* __restrict__ partials,
                                                   unsigned int* __restrict__ counter,
                                                   double* __restrict__ out) {
  __shared__ double sh[32];
  __shared__ bool last;
  double acc = 0.0;
  for (int s = 0; s < ns; ++s) {
    const double* x = X + soff[s];
    for (int64_t e = (int64_t)blockIdx.x * RB + threadIdx.x; e < slen[s]; e += (int64_t)gridDim.x * RB)
      acc = fma(x[e], x[e], acc);
  }
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = acc;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  double v = threadIdx.x < gridDim.x ? ((volatile double*)partials)[threadIdx.x] : 0.0;
  v = block_sum(v, sh);
  if (threadIdx.x == 0) { *out = v; *counter = 0u; }
}

// max |x| -> *out
__global__ void __launch_bounds__(RB) absmax_kernel(const double* __restrict__ x, int64_t n,
                                                    double* __restrict__ partials,
                                                    unsigned int* __restrict__ counter,
                                                    double* __restrict__ out) {
  __shared__ double sh[RB];
  __shared__ bool last;
  double m = 0.0;
  for (int64_t r = (int64_t)blockIdx.x * RB + threadIdx.x; r < n; r += (int64_t)gridDim.x * RB)
    m = fmax(m, fabs(x[r]));
  sh[threadIdx.x] = m;
  __syncthreads();
  for (int s = RB / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[blockIdx.x] = sh[0];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  sh[threadIdx.x] = threadIdx.x < gridDim.x ? ((volatile double*)partials)[threadIdx.x] : 0.0;
  __syncthreads();
  for (int s = RB / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) { *out = sh[0]; *counter = 0u; }
}

__global__ void sign_first_kernel(const double* __restrict__ x, double* __restrict__ s) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *s = x[0] < 0.0 ? -1.0 : 1.0;
}

// x[i] uniform in [-1, 1) from splitmix64(seed + i): a reproducible start vector
__global__ void fill_random_kernel(double* __restrict__ x, int64_t n, uint64_t seed) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(i + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    x[i] = (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
  }
}

int grid_for(int64_t n) {
  int64_t g = (n + 255) / 256;
  if (g > 152 * 8) g = 152 * 8;
  if (g < 1) g = 1;
  return (int)g;
}

}  // namespace

namespace imps {

int kr_multidot(const KrylovWs& ws, const double* V, int64_t ldv, int ncols, const double* w,
                int64_t n, double* h, int mode, double* out_sqrt, cudaStream_t st) {
  if (ncols > kMaxCols) return IMPS_ERR_BAD_ARG;
  int grid = (int)((n + RB - 1) / RB);
  if (grid > RGRID) grid = RGRID;
  if (grid < 1) grid = 1;
  imps::count_launch();
  multidot_kernel<<<grid, RB, 0, st>>>(V, ldv, ncols, w, n, ws.partials, ws.counter, h, mode, out_sqrt);
  return IMPS_OK;
}

int kr_gemv_sub(const double* V, int64_t ldv, int ncols, const double* h, double* w, int64_t n,
                cudaStream_t st) {
  imps::count_launch();
  gemv_sub_kernel<<<grid_for(n), 256, 0, st>>>(V, ldv, ncols, h, w, n);
  return IMPS_OK;
}

int kr_gemv(const double* V, int64_t ldv, int ncols, const double* h, double* y, int64_t n,
            cudaStream_t st) {
  imps::count_launch();
  gemv_kernel<<<grid_for(n), 256, 0, st>>>(V, ldv, ncols, h, y, n);
  return IMPS_OK;
}

int kr_basis_rotate(const double* V, int64_t ldv, int m, const double* W, int kk, double* out,
                    int64_t ldo, int64_t n, cudaStream_t st) {
  if (m < 1 || m > kMaxCols || kk < 1 || n < 1) return IMPS_ERR_BAD_ARG;
  imps::count_launch();
  basis_rotate_kernel<<<grid_for(n), 256, 0, st>>>(V, ldv, m, W, kk, out, ldo, n);
  return IMPS_OK;
}

int kr_cgs2_step(const KrylovWs& ws, const double* V, int64_t ldv, int nc, double* w, int64_t n,
                 double* h, double* h2, double* vnext, int* flag, cudaStream_t st, int nloc) {
  if (nc < 1 || nc > kMaxCols) return IMPS_ERR_BAD_ARG;
  int c_loc = (nloc > 0 && nloc < nc) ? nc - nloc : 0;
  // (column nc of the second partials region carries |w|^2, hence nc < kMaxCols)
  if (ws.sync && ws.err && n <= (int64_t)CGRID * COOP_SUB && nc < kMaxCols) {
    // one cooperative launch: w stays in shared memory, one grid barrier per reduction
    int64_t gc = (n + 255) / 256;
    if (gc > CGRID) gc = CGRID;
    int64_t subc = (n + gc - 1) / gc;
    subc = ((subc + 31) / 32) * 32;
    const int gridc = (int)((n + subc - 1) / subc);
    int subi = (int)subc;
    double* partials = ws.partials;
    unsigned int* sync = ws.sync;
    int* err = ws.err;
    void* args[] = {(void*)&V, (void*)&ldv, (void*)&nc, (void*)&w, (void*)&n, (void*)&subi, (void*)&h,
                    (void*)&vnext, (void*)&flag, (void*)&partials, (void*)&sync, (void*)&err, (void*)&c_loc};
    if (cudaLaunchCooperativeKernel((const void*)cgs2_coop_kernel, dim3(gridc), dim3(CT), args, 0, st) ==
        cudaSuccess) {
      imps::count_launch();
      return IMPS_OK;
    }
    (void)cudaGetLastError();  // not co-resident here: fall back to four launches
  }
  int64_t g = (n + 255) / 256;  // >= 256 rows per block, at most one block per SM
  if (g > CGRID) g = CGRID;
  if (g < 1) g = 1;
  const int grid = (int)g;
  int64_t sub = (n + grid - 1) / grid;
  sub = ((sub + 31) / 32) * 32;
  if (sub > CSUB) sub = CSUB;
  imps::count_launch(4);
  cgs_pass_kernel<0><<<grid, CT, 0, st>>>(V, ldv, nc, w, n, (int)sub, nullptr, h, nullptr, ws.partials,
                                          ws.counter);
  cgs_pass_kernel<1><<<grid, CT, 0, st>>>(V, ldv, nc, w, n, (int)sub, h, h2, h, ws.partials, ws.counter);
  cgs_pass_kernel<2><<<grid, CT, 0, st>>>(V, ldv, nc, w, n, (int)sub, h2, h + nc, nullptr, ws.partials,
                                          ws.counter);
  scale_inv_kernel<<<grid_for(n), 256, 0, st>>>(w, h + nc, vnext, n, flag);
  return IMPS_OK;
}

int kr_cgs2_step_batch(double* partials, unsigned int* counters, int P, const double* V, int64_t sV, int64_t ldv,
                       int nc, double* w, int64_t sw, int64_t n, double* h, int64_t sh, double* h2, double* vnext,
                       int* flags, cudaStream_t st) {
  if (nc < 1 || nc >= kMaxCols || P < 1) return IMPS_ERR_BAD_ARG;
  int64_t g = (n + 255) / 256;
  if (g > CGRID) g = CGRID;
  if (g < 1) g = 1;
  int64_t sub = (n + g - 1) / g;
  sub = ((sub + 31) / 32) * 32;
  if (sub > CSUB) sub = CSUB;
  const dim3 grid((unsigned)g, (unsigned)P);
  const int64_t sp = (int64_t)g * kMaxCols;  // partials per system (column c at c * g)
  const int64_t sh2 = kMaxCols;              // h2: one kMaxCols block per system
  imps::count_launch(4);
  // h = V^T w; then w -= V h, h2 = V^T w, h += h2; then w -= V h2, |w| -> h[nc]
  cgs_pass_kernel<0><<<grid, CT, 0, st>>>(V, ldv, nc, w, n, (int)sub, nullptr, h, nullptr, partials, counters, sV,
                                          sw, 0, sh, 0, sp);
  cgs_pass_kernel<1><<<grid, CT, 0, st>>>(V, ldv, nc, w, n, (int)sub, h, h2, h, partials, counters, sV, sw, sh, sh2,
                                          sh, sp);
  cgs_pass_kernel<2><<<grid, CT, 0, st>>>(V, ldv, nc, w, n, (int)sub, h2, h + nc, nullptr, partials, counters, sV,
                                          sw, sh2, sh, 0, sp);
  scale_inv_kernel<<<dim3((unsigned)grid_for(n), (unsigned)P), 256, 0, st>>>(w, h + nc, vnext, n, flags, sw, sh, sV);
  return cudaGetLastError() == cudaSuccess ? IMPS_OK : IMPS_ERR_CUDA;
}

int kr_scale_inv(const double* x, const double* nrm, double* y, int64_t n, int* flag, cudaStream_t st) {
  imps::count_launch();
  scale_inv_kernel<<<grid_for(n), 256, 0, st>>>(x, nrm, y, n, flag);
  return IMPS_OK;
}

int kr_fill_random(double* x, int64_t n, uint64_t seed, cudaStream_t st) {
  imps::count_launch();
  fill_random_kernel<<<grid_for(n), 256, 0, st>>>(x, n, seed);
  return IMPS_OK;
}

int kr_axpby(double a, const double* x, double b, double* y, int64_t n, cudaStream_t st) {
  imps::count_launch();
  axpby_kernel<<<grid_for(n), 256, 0, st>>>(a, x, b, y, n);
  return IMPS_OK;
}

int kr_proj_epilogue(const double* x, const double* t, const double* s, const double* rho, double* y,
                     int64_t n, cudaStream_t st) {
  imps::count_launch();
  proj_epilogue_kernel<<<grid_for(n), 256, 0, st>>>(x, t, s, rho, y, n);
  return IMPS_OK;
}

int kr_trace_prod(const KrylovWs& ws, const double* X, const double* R, const int64_t* boff,
                  const int32_t* bdim, int nb, double* out, cudaStream_t st, const int32_t* bcols) {
  imps::count_launch();
  constexpr int grid = 128;  // <= RB: the finishing CTA sums the partials of every CTA
  trace_prod_kernel<<<grid, RB, 0, st>>>(X, R, boff, bdim, bcols, nb, ws.partials, ws.counter, out);
  return IMPS_OK;
}

// out = u - fac * t + tau * rho on split complex planes (fac = c + i s; tau, rho optional):
//   out_re = u_re - (c t_re - s t_im) + tau_re rho,  out_im = u_im - (s t_re + c t_im) + tau_im rho
__global__ void fac_epilogue_kernel(const double* __restrict__ ure, const double* __restrict__ uim,
                                    const double* __restrict__ tre, const double* __restrict__ tim, double c,
                                    double sn, const double* __restrict__ tau, const double* __restrict__ rho,
                                    double* __restrict__ ore, double* __restrict__ oim, int64_t n) {
  const double tr = tau ? tau[0] : 0.0, ti = tau ? tau[1] : 0.0;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const double a = tre[r], b = tim[r];
    const double p = rho ? rho[r] : 0.0;
    ore[r] = ure[r] - (c * a - sn * b) + tr * p;
    oim[r] = uim[r] - (sn * a + c * b) + ti * p;
  }
}

int kr_fac_epilogue(const double* ure, const double* uim, const double* tre, const double* tim, double c,
                    double s, const double* tau, const double* rho, double* ore, double* oim, int64_t n,
                    cudaStream_t st) {
  imps::count_launch();
  fac_epilogue_kernel<<<grid_for(n), 256, 0, st>>>(ure, uim, tre, tim, c, s, tau, rho, ore, oim, n);
  return IMPS_OK;
}

// Batched form over P systems stacked as [re_0 | im_0 | re_1 | im_1 | ...] (planes of n):
// out_j = u_j - f_j T u_j with the complex factor f_j = fre[j] + i fim[j] (device arrays).
__global__ void fac_epilogue_batch_kernel(const double* __restrict__ u, const double* __restrict__ t,
                                          const double* __restrict__ fre, const double* __restrict__ fim,
                                          double* __restrict__ out, int64_t n, int P) {
  const int64_t total = (int64_t)P * n;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = i / n, r = i - j * n;
    const int64_t re = 2 * j * n + r, im = re + n;
    const double c = fre[j], sn = fim[j], a = t[re], b = t[im];
    out[re] = u[re] - (c * a - sn * b);
    out[im] = u[im] - (sn * a + c * b);
  }
}

int kr_fac_epilogue_batch(const double* u, const double* t, const double* fre, const double* fim, double* out,
                          int64_t n, int P, cudaStream_t st) {
  imps::count_launch();
  fac_epilogue_batch_kernel<<<grid_for((int64_t)P * n), 256, 0, st>>>(u, t, fre, fim, out, n, P);
  return IMPS_OK;
}

int kr_segsq(const KrylovWs& ws, const double* X, const int64_t* soff, const int64_t* slen, int ns,
             double* out, cudaStream_t st) {
  imps::count_launch();
  segsq_kernel<<<64, RB, 0, st>>>(X, soff, slen, ns, ws.partials, ws.counter, out);
  return IMPS_OK;
}

int kr_absmax(const KrylovWs& ws, const double* x, int64_t n, double* out, cudaStream_t st) {
  int grid = (int)((n + RB - 1) / RB);
  if (grid > RGRID) grid = RGRID;
  if (grid < 1) grid = 1;
  imps::count_launch();
  absmax_kernel<<<grid, RB, 0, st>>>(x, n, ws.partials, ws.counter, out);
  return IMPS_OK;
}

int kr_sign_of_first(const double* x, double* s, cudaStream_t st) {
  imps::count_launch();
  sign_first_kernel<<<1, 32, 0, st>>>(x, s);
  return IMPS_OK;
}

size_t kr_partials_elems() {
  return std::max((size_t)RGRID * kMaxCols, (size_t)3 * CGRID * kMaxCols);
}

}  // namespace imps
