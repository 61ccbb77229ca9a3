// FP64 kernels for the block-sparse hot path on sm_103a.
//
//  * grouped_gemm_f64: output-stationary grouped GEMM over the planner's tile/term tables, one
//    CTA per table entry: an output tile, or one of `nparts` shares of its K chunks (split-K,
//    over all of its terms in order; the share count is set per tile by the host); inside a CTA
//    the chunks are dealt to K groups whose partial tiles are summed in a fixed order.  With one
//    share the tile is written directly; otherwise every CTA stores its partial tile and the
//    last CTA of the tile to finish (an atomic ticket after a memory fence; nobody waits) sums
//    the partials in share order and writes the tile.  Deterministic for a given plan; no
//    separate zero-fill: the first write also performs the reference's memset of `out`,
//    VUMPS_helpers.hpp:69.
//  * Krylov BLAS-1 (reductions without atomics: fixed-grid partials + one finishing block).
#include <cuda_runtime.h>

#include <cstdint>

#include "imps_internal.h"
#include "imps_status.h"

using imps::Term;
using imps::Tile;

namespace {

constexpr int TK = 16;

// Named barrier over the NT threads of one K group (ids 1..KS; 0 is __syncthreads).
__device__ __forceinline__ void group_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// TMxTN tile computed by KS groups of (TM/RM)*(TN/RN) threads, each thread holding RM x RN
// accumulators.  The tile's K chunks (TK wide, over all of its terms in order) are dealt
// round-robin to the KS groups, so a tile with few rows still keeps KS times more warps busy;
// the groups' partial tiles are summed in a fixed order through shared memory (deterministic).
template <int TM, int TN, int RM, int RN, int KS>
__global__ void __launch_bounds__((TM / RM) * (TN / RN) * KS)
grouped_gemm_f64_kernel(const Tile* __restrict__ tiles, const Term* __restrict__ terms,
                        imps_dslots slots, double* __restrict__ ws, int* __restrict__ cnt) {
  constexpr int NT = (TM / RM) * (TN / RN);
  constexpr int TX = TN / RN;  // threads along n
  constexpr int AS = TK * (TM + 1), BS = TK * (TN + 1);
  constexpr int STAGE = KS * (AS + BS);
  constexpr int RED = (KS - 1) * NT * RM * RN;
  __shared__ double smem[STAGE > RED ? STAGE : RED];
  __shared__ int last;
  const Tile tl = tiles[blockIdx.x];
  const int splits = tl.nparts, part = tl.part;
  // this CTA's chunk range [c_lo, c_hi) of the tile's chunk sequence
  int c_lo = 0, c_hi = 1 << 30;
  if (splits > 1) {
    int nch = 0;
    for (int t = tl.t0; t < tl.t1; ++t) nch += (terms[t].k + TK - 1) / TK;
    c_lo = (int)((int64_t)nch * part / splits);
    c_hi = (int)((int64_t)nch * (part + 1) / splits);
  }
  const int g = threadIdx.x / NT;
  const int tid = threadIdx.x - g * NT;
  const int tx = tid % TX, ty = tid / TX;
  double* As = smem + g * (AS + BS);  // [TK][TM + 1]
  double* Bs = As + AS;               // [TK][TN + 1]
  double acc[RM][RN];
#pragma unroll
  for (int i = 0; i < RM; ++i)
#pragma unroll
    for (int j = 0; j < RN; ++j) acc[i][j] = 0.0;

  int chunk = 0;
  for (int t = tl.t0; t < tl.t1 && chunk < c_hi; ++t) {
    const Term tm = terms[t];
    const int nk = (tm.k + TK - 1) / TK;
    if (chunk + nk <= c_lo) {  // wholly before this split's range
      chunk += nk;
      continue;
    }
    const double* __restrict__ A = slots.p[tm.a_slot] + tm.a_off;
    const double* __restrict__ B = slots.p[tm.b_slot] + tm.b_off;
    const double alpha = tm.alpha;
    for (int k0 = 0; k0 < tm.k; k0 += TK, ++chunk) {
      if (chunk < c_lo || chunk >= c_hi || (chunk - c_lo) % KS != g) continue;
      // A tile: rows m0..m0+TM, cols k0..k0+TK of op(A)
      for (int e = tid; e < TM * TK; e += NT) {
        int m, k;
        if (tm.a_t) { k = e % TK; m = e / TK; } else { m = e % TM; k = e / TM; }
        const int gm = tl.m0 + m, gk = k0 + k;
        double v = 0.0;
        if (m < tl.mt && gk < tm.k)
          v = tm.a_t ? A[(int64_t)gm * tm.a_ld + gk] : A[gm + (int64_t)gk * tm.a_ld];
        As[k * (TM + 1) + m] = alpha * v;
      }
      for (int e = tid; e < TN * TK; e += NT) {
        int n, k;
        if (tm.b_t) { n = e % TN; k = e / TN; } else { k = e % TK; n = e / TK; }
        const int gn = tl.n0 + n, gk = k0 + k;
        double v = 0.0;
        if (n < tl.nt && gk < tm.k)
          v = tm.b_t ? B[gn + (int64_t)gk * tm.b_ld] : B[gk + (int64_t)gn * tm.b_ld];
        Bs[k * (TN + 1) + n] = v;
      }
      group_sync(g + 1, NT);
      const int kmax = min(TK, tm.k - k0);
      for (int k = 0; k < kmax; ++k) {
        double a[RM], b[RN];
#pragma unroll
        for (int i = 0; i < RM; ++i) a[i] = As[k * (TM + 1) + ty + i * (TM / RM)];
#pragma unroll
        for (int j = 0; j < RN; ++j) b[j] = Bs[k * (TN + 1) + tx + j * TX];
#pragma unroll
        for (int i = 0; i < RM; ++i)
#pragma unroll
          for (int j = 0; j < RN; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
      }
      group_sync(g + 1, NT);
    }
  }
  if (KS > 1) {
    __syncthreads();  // every group is done with its staging buffers: reuse them for the sums
    double* red = smem;
    if (g > 0) {
#pragma unroll
      for (int i = 0; i < RM; ++i)
#pragma unroll
        for (int j = 0; j < RN; ++j) red[(((g - 1) * NT + tid) * RM + i) * RN + j] = acc[i][j];
    }
    __syncthreads();
    if (g > 0) return;  // only group 0 (its own named barrier below) goes on
    for (int q = 1; q < KS; ++q)
#pragma unroll
      for (int i = 0; i < RM; ++i)
#pragma unroll
        for (int j = 0; j < RN; ++j) acc[i][j] += red[(((q - 1) * NT + tid) * RM + i) * RN + j];
  }
  if (splits > 1) {
    // partial tile -> workspace; the last CTA of the tile sums all partials in split order
    double* wp = ws + ((int64_t)tl.ws_unit + part) * (TM * TN);
#pragma unroll
    for (int i = 0; i < RM; ++i)
#pragma unroll
      for (int j = 0; j < RN; ++j) wp[(ty + i * (TM / RM)) * TN + tx + j * TX] = acc[i][j];
    __threadfence();
    group_sync(1, NT);
    if (tid == 0) last = atomicAdd(cnt + tl.cnt_idx, 1) == splits - 1;
    group_sync(1, NT);
    if (!last) return;
    __threadfence();
#pragma unroll
    for (int i = 0; i < RM; ++i)
#pragma unroll
      for (int j = 0; j < RN; ++j) {
        const int e = (ty + i * (TM / RM)) * TN + tx + j * TX;
        double sum = 0.0;
        for (int q = 0; q < splits; ++q) sum += __ldcg(ws + ((int64_t)tl.ws_unit + q) * (TM * TN) + e);
        acc[i][j] = sum;
      }
    if (tid == 0) cnt[tl.cnt_idx] = 0;  // re-armed for the next launch of this stage
  }
  double* __restrict__ C = slots.p[tl.c_slot] + tl.c_off;
#pragma unroll
  for (int i = 0; i < RM; ++i) {
    const int m = ty + i * (TM / RM);
    if (m >= tl.mt) continue;
#pragma unroll
    for (int j = 0; j < RN; ++j) {
      const int n = tx + j * TX;
      if (n >= tl.nt) continue;
      double* p = C + (tl.m0 + m) + (int64_t)(tl.n0 + n) * tl.c_ld;
      *p = tl.accumulate ? *p + acc[i][j] : acc[i][j];
    }
  }
}

}  // namespace

int imps_launch_grouped_f64(const void* d_tiles, int ntiles, const void* d_terms, imps_dslots slots,
                            int tile_m, int splits, double* ws, int* cnt, void* stream) {
  if (ntiles <= 0) return IMPS_OK;
  if (splits < 1 || (splits > 1 && (!ws || !cnt))) return IMPS_ERR_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  const int grid = ntiles;  // one CTA per table entry (a tile or one K share of it)
  imps::count_launch();
  if (tile_m == 16) {
    grouped_gemm_f64_kernel<16, 16, 2, 2, 4><<<grid, 256, 0, st>>>((const Tile*)d_tiles, (const Term*)d_terms,
                                                                  slots, ws, cnt);
  } else {
    grouped_gemm_f64_kernel<32, 32, 2, 4, 2><<<grid, 256, 0, st>>>((const Tile*)d_tiles, (const Term*)d_terms,
                                                                   slots, ws, cnt);
  }
  return cudaGetLastError() == cudaSuccess ? IMPS_OK : IMPS_ERR_CUDA;
}
