// Tensor-core (tcgen05, sm_103a) execution of planner stages in split-BF16 precision.
//
// Every FP64 operand x is split as x = hi + mid + lo with hi, mid, lo in BF16; a product is
// formed from the six terms hi*hi + hi*mid + mid*hi + hi*lo + mid*mid + lo*hi (the dropped
// terms are O(2^-24) relative), accumulated in FP32 in tensor memory, and written back to
// the FP64 output.  Operands are packed once into the canonical UMMA layout (K-major, no
// swizzle: 8 rows x 16 bytes core matrices; LBO = stride between the two 8-element K
// chunks, SBO = stride between 8-row groups = 128 B):
//     packed[kstep][split][chunk][row group][8 rows][8 bf16]
// so that the two K-steps of one pipeline stage are one contiguous bulk copy.
//
// Kernel roles (128 threads, one CTA per output tile of <= 128 x 128):
//   warp 0 lane 0 : producer, cp.async.bulk global -> shared, mbarrier complete_tx
//   warp 1 lane 0 : MMA issuer, tcgen05.mma.cta_group::1.kind::f16 into TMEM, tcgen05.commit
//   warps 0-3     : epilogue, tcgen05.ld 32x32b -> FP64 global
// Every mbarrier wait is bounded; on timeout the CTA records an error, drains what it
// issued (bounded), frees its TMEM and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <map>
#include <tuple>
#include <vector>

#include "imps_status.h"
#include "imps_tc.h"

namespace imps {

namespace {

constexpr int TC_M = 128;        // UMMA M (rows of every tile, zero padded)
constexpr int TC_NMAX = 128;     // max UMMA N per tile
constexpr int TC_KSTAGE = 2;     // K-steps (of 16) per pipeline stage
constexpr int TC_NSTAGE = 4;     // pipeline depth
constexpr int TC_THREADS = 128;
constexpr int A_STAGE_BYTES = TC_KSTAGE * 3 * TC_M * 32;     // 24 KB
constexpr int B_STAGE_BYTES = TC_KSTAGE * 3 * TC_NMAX * 32;  // 24 KB
constexpr int STAGE_BYTES = A_STAGE_BYTES + B_STAGE_BYTES;
// the whole opt-in shared memory of the SM: pipeline (4 x 48 KB) + alignment slack + headroom
// so that every descriptor-addressed access stays inside this CTA's allocation
constexpr int SMEM_BYTES = 230400;  // 225 KB (opt-in maximum 227 KB minus static shared memory)
static_assert(TC_NSTAGE * STAGE_BYTES + 1024 <= SMEM_BYTES, "tcgen05 pipeline does not fit");
constexpr uint32_t WAIT_LIMIT = 1u << 24;

struct TcTerm {
  int64_t a_off, b_off;  // bf16 element offsets into the packed buffer
  int32_t ksteps;        // padded K / 16
  int32_t pad;
};

struct TcTile {
  int64_t c_off;
  int32_t c_ld, m, n, npad;
  int32_t t0, t1;
  int16_t c_slot, accumulate;
  int32_t pad;
};

struct PackJob {
  int64_t src_off;
  int64_t dst_off;  // bf16 elements
  int32_t src_ld;
  int32_t trans;    // stored matrix is op()^T
  int32_t role;     // 0: A (rows = M), 1: B (rows = N)
  int32_t rows, k;  // valid rows of this tile slice, valid K
  int32_t rpad, kpad;
  int32_t r0;       // first row (A: m0, B: n0) of the slice
  int32_t slot;
  int32_t pad;
  double alpha;
};

// ------------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// bounded wait for the phase with the given parity; returns false on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  for (uint32_t i = 0; i < WAIT_LIMIT; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version (tcgen05)
  // base offset 0, LBO mode relative, layout type 0 = no swizzle
  return d;
}

// kind::f16 instruction descriptor: D fp32, A/B bf16, both K-major, N>>3 @17, M>>4 @24
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// ------------------------------------------------------------------ kernels
// One block row per job (blockIdx.x), grid-stride over the padded rpad x kpad operand.  The
// FP64 value is rounded once to FP32 and split there into hi + mid + lo BF16 terms: each
// difference xf - bf16(xf) is exact in FP32, so the three terms carry all 24 significand bits
// of xf (relative error 2^-24, the order of the dropped lo*lo-type products) while the FP64
// pipe, slow on this GPU, sees one conversion per element.  32-bit index arithmetic.
__global__ void pack_kernel(const PackJob* __restrict__ jobs, imps_dslots slots, __nv_bfloat16* __restrict__ out) {
  const PackJob jb = jobs[blockIdx.x];
  const double* S = slots.p[jb.slot] + jb.src_off;
  const int rpad = jb.rpad;
  const int total = rpad * jb.kpad;
  const float alpha = (float)jb.alpha;
  const int split_elems = rpad * 16;
  for (int t = threadIdx.x + blockIdx.y * blockDim.x; t < total; t += gridDim.y * blockDim.x) {
    const int k = t / rpad, r = t - k * rpad;
    float xf = 0.0f;
    const int gr = jb.r0 + r;
    if (r < jb.rows && k < jb.k) {
      double x;
      if (jb.role == 0)  // op(A)(gr, k)
        x = jb.trans ? S[k + (int64_t)gr * jb.src_ld] : S[gr + (int64_t)k * jb.src_ld];
      else  // op(B)(k, gr)
        x = jb.trans ? S[gr + (int64_t)k * jb.src_ld] : S[k + (int64_t)gr * jb.src_ld];
      xf = __double2float_rn(x) * alpha;
    }
    const __nv_bfloat16 hi = __float2bfloat16_rn(xf);
    const float x1 = xf - __bfloat162float(hi);
    const __nv_bfloat16 mid = __float2bfloat16_rn(x1);
    const float x2 = x1 - __bfloat162float(mid);
    const __nv_bfloat16 lo = __float2bfloat16_rn(x2);
    const int kstep = k >> 4, kk = k & 15, chunk = kk >> 3, e = kk & 7;
    const int rgi = r >> 3, rr = r & 7;
    const int64_t base = jb.dst_off + (int64_t)kstep * 3 * split_elems + (int64_t)chunk * rpad * 8 +
                         (int64_t)rgi * 64 + rr * 8 + e;
    out[base] = hi;
    out[base + split_elems] = mid;
    out[base + 2 * split_elems] = lo;
  }
}

__global__ void __launch_bounds__(TC_THREADS, 1)
tc_gemm_kernel(const TcTile* __restrict__ tiles, const TcTerm* __restrict__ terms,
               const __nv_bfloat16* __restrict__ packed, imps_dslots slots, int* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full_bar[TC_NSTAGE];
  __shared__ __align__(8) uint64_t empty_bar[TC_NSTAGE];
  __shared__ __align__(8) uint64_t done_bar;
  __shared__ uint32_t tmem_base_s;
  __shared__ int abort_s;
  const TcTile tl = tiles[blockIdx.x];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t ncols = 128;  // TMEM columns (power of two >= npad)
  if (threadIdx.x == 0) {
    for (int s = 0; s < TC_NSTAGE; ++s) { mbar_init(&full_bar[s], 1); mbar_init(&empty_bar[s], 1); }
    mbar_init(&done_bar, 1);
    abort_s = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_s)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_s;
  const int nterm = tl.t1 - tl.t0;
  const uint32_t idesc = idesc_bf16(TC_M, tl.npad);
  const uint32_t a_split_bytes = TC_M * 32;          // one split of one K-step (A)
  const uint32_t b_split_bytes = (uint32_t)tl.npad * 32;

  if (warp == 0 && lane == 0 && nterm > 0) {
    // ---------------- producer
    int it = 0;
    bool ok = true;
    for (int t = tl.t0; t < tl.t1 && ok; ++t) {
      const TcTerm tm = terms[t];
      for (int ks = 0; ks < tm.ksteps && ok; ks += TC_KSTAGE, ++it) {
        const int s = it % TC_NSTAGE;
        const uint32_t u = (uint32_t)(it / TC_NSTAGE);
        if (u > 0 && !mbar_wait(&empty_bar[s], (u & 1) ^ 1)) { ok = false; break; }
        if (*(volatile int*)&abort_s) { ok = false; break; }
        const int nk = min(TC_KSTAGE, tm.ksteps - ks);
        const uint32_t abytes = nk * 3 * a_split_bytes, bbytes = nk * 3 * b_split_bytes;
        uint8_t* sa = smem + s * STAGE_BYTES;
        uint8_t* sb = sa + A_STAGE_BYTES;
        mbar_expect_tx(&full_bar[s], abytes + bbytes);
        bulk_g2s(sa, packed + tm.a_off + (int64_t)ks * 3 * TC_M * 16, abytes, &full_bar[s]);
        bulk_g2s(sb, packed + tm.b_off + (int64_t)ks * 3 * tl.npad * 16, bbytes, &full_bar[s]);
      }
    }
    if (!ok) { atomicExch(err, 1); abort_s = 1; }
  } else if (warp == 1 && lane == 0 && nterm > 0) {
    // ---------------- MMA issuer
    int it = 0;
    uint32_t accum = 0;
    bool ok = true;
    for (int t = tl.t0; t < tl.t1 && ok; ++t) {
      const TcTerm tm = terms[t];
      for (int ks = 0; ks < tm.ksteps; ks += TC_KSTAGE, ++it) {
        const int s = it % TC_NSTAGE;
        const uint32_t u = (uint32_t)(it / TC_NSTAGE);
        if (!mbar_wait(&full_bar[s], u & 1) || *(volatile int*)&abort_s) { ok = false; break; }
        tc_fence_after();
        const int nk = min(TC_KSTAGE, tm.ksteps - ks);
        const uint32_t sa = smem_u32(smem + s * STAGE_BYTES);
        const uint32_t sb = sa + A_STAGE_BYTES;
        for (int k = 0; k < nk; ++k) {
          // split pairs (a, b): hh, hm, mh, hl, mm, lh
          const int pa[6] = {0, 0, 1, 0, 1, 2};
          const int pb[6] = {0, 1, 0, 2, 1, 0};
#pragma unroll
          for (int q = 0; q < 6; ++q) {
            const uint64_t ad = smem_desc(sa + (k * 3 + pa[q]) * a_split_bytes, TC_M * 16, 128);
            const uint64_t bd = smem_desc(sb + (k * 3 + pb[q]) * b_split_bytes, tl.npad * 16, 128);
            mma_bf16(tmem, ad, bd, idesc, accum);
            accum = 1;
          }
        }
        mma_commit(&empty_bar[s]);  // frees the stage once these MMAs have read it
      }
    }
    if (!ok) { atomicExch(err, 1); abort_s = 1; }
    mma_commit(&done_bar);  // arrives when every MMA issued above has completed
  }
  __syncthreads();  // role lanes rejoin their warps before the warp-collective TMEM loads
  // ---------------- epilogue
  double* C = slots.p[tl.c_slot] + tl.c_off;
  bool have = nterm > 0;
  if (have) {
    if (!mbar_wait(&done_bar, 0)) { atomicExch(err, 1); have = false; }
    tc_fence_after();
  }
  have = __all_sync(0xffffffffu, have);
  __syncwarp();
  const int row = warp * 32 + lane;
  for (int c0 = 0; c0 < tl.npad; c0 += 16) {
    float v[16];
    if (have) {
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
    } else {
#pragma unroll
      for (int i = 0; i < 16; ++i) v[i] = 0.f;
    }
    if (row < tl.m) {
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int col = c0 + i;
        if (col < tl.n) {
          double* p = C + row + (int64_t)col * tl.c_ld;
          *p = tl.accumulate ? *p + (double)v[i] : (double)v[i];
        }
      }
    }
  }
  // producer drains its copies if it aborted (bounded), then TMEM is released
  if (warp == 0 && lane == 0 && abort_s) {
    for (int s = 0; s < TC_NSTAGE; ++s) mbar_wait(&full_bar[s], 0);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
  }
}

}  // namespace

// ------------------------------------------------------------------ host side
struct TcStage {
  std::vector<TcTile> tiles;
  std::vector<TcTerm> terms;
  std::vector<PackJob> dyn_jobs;  // packed before every run of the stage
  TcTile* d_tiles = nullptr;
  TcTerm* d_terms = nullptr;
  PackJob* d_dyn = nullptr;
};

struct TcPlan {
  std::vector<TcStage> stages;         // parallel to Plan::stages
  std::vector<PackJob> static_jobs;    // packed at prepare time
  PackJob* d_static = nullptr;
  __nv_bfloat16* packed = nullptr;
  int64_t packed_elems = 0;
  int* d_err = nullptr;
  bool static_valid = false;
  std::vector<char> dynamic_slot;
  const Stage* first_stage = nullptr;
};

static int round_up(int x, int m) { return (x + m - 1) / m * m; }

int tc_create(TcPlan** out, const Plan& P, cudaStream_t st) {
  TcPlan* T = new TcPlan();
  T->dynamic_slot.assign(P.slots.size(), 0);
  T->dynamic_slot[P.n_in] = 1;
  for (const Stage& S : P.stages)
    for (const OutBlock& o : S.outs) T->dynamic_slot[o.c_slot] = 1;
  std::map<std::tuple<int, int64_t, int, int, int, int, int, int, double>, int64_t> seen;
  int64_t off = 0;
  bool too_large = false;  // the pack kernel indexes one operand slice with 32-bit integers
  auto pack_for = [&](int slot, int64_t src, int ld, int trans, int role, int r0, int rows, int k, int rpad,
                      double alpha, std::vector<PackJob>& jobs) -> int64_t {
    const int kpad = round_up(std::max(k, 1), 16);
    if ((int64_t)rpad * kpad * 3 >= ((int64_t)1 << 31)) too_large = true;
    auto key = std::make_tuple(slot, src, ld, trans, role, r0, rows, k, alpha);
    auto it = seen.find(key);
    if (it != seen.end()) return it->second;
    PackJob j{};
    j.src_off = src; j.dst_off = off; j.src_ld = ld; j.trans = trans; j.role = role;
    j.rows = rows; j.k = k; j.rpad = rpad; j.kpad = kpad; j.r0 = r0; j.slot = slot; j.alpha = alpha;
    jobs.push_back(j);
    seen[key] = off;
    const int64_t o = off;
    off += (int64_t)3 * rpad * kpad;
    return o;
  };
  for (const Stage& S : P.stages) {
    TcStage ts;
    for (const OutBlock& o : S.outs) {
      for (int m0 = 0; m0 < std::max(o.M, 1); m0 += TC_M)
        for (int n0 = 0; n0 < std::max(o.N, 1); n0 += TC_NMAX) {
          TcTile tl{};
          tl.c_off = o.c_off + m0 + (int64_t)n0 * o.c_ld;
          tl.c_ld = std::max(o.c_ld, 1);
          tl.m = std::min(TC_M, o.M - m0);
          tl.n = std::min(TC_NMAX, o.N - n0);
          tl.npad = std::max(16, round_up(tl.n, 16));
          tl.c_slot = o.c_slot;
          tl.accumulate = o.accumulate;
          tl.t0 = (int)ts.terms.size();
          if (tl.m <= 0 || tl.n <= 0) continue;
          for (int t = o.t0; t < o.t1; ++t) {
            const Term& tm = S.terms[t];
            if (tm.k <= 0) continue;
            std::vector<PackJob>& ja = T->dynamic_slot[tm.a_slot] ? ts.dyn_jobs : T->static_jobs;
            std::vector<PackJob>& jb = T->dynamic_slot[tm.b_slot] ? ts.dyn_jobs : T->static_jobs;
            TcTerm tt{};
            tt.a_off = pack_for(tm.a_slot, tm.a_off, tm.a_ld, tm.a_t, 0, m0, tl.m, tm.k, TC_M, tm.alpha, ja);
            tt.b_off = pack_for(tm.b_slot, tm.b_off, tm.b_ld, tm.b_t, 1, n0, tl.n, tm.k, tl.npad, 1.0, jb);
            tt.ksteps = round_up(tm.k, 16) / 16;
            ts.terms.push_back(tt);
          }
          tl.t1 = (int)ts.terms.size();
          ts.tiles.push_back(tl);
        }
    }
    T->stages.push_back(std::move(ts));
  }
  T->packed_elems = off;
  auto up = [&](void** d, const void* h, size_t bytes) -> int {
    if (bytes == 0) return IMPS_OK;
    if (cudaMalloc(d, bytes) != cudaSuccess) return IMPS_ERR_OOM;
    if (cudaMemcpy(*d, h, bytes, cudaMemcpyHostToDevice) != cudaSuccess) return IMPS_ERR_CUDA;
    return IMPS_OK;
  };
  int rc = too_large ? IMPS_ERR_TOO_LARGE : IMPS_OK;
  for (TcStage& ts : T->stages) {
    if (rc) break;
    if ((rc = up((void**)&ts.d_tiles, ts.tiles.data(), ts.tiles.size() * sizeof(TcTile)))) break;
    if ((rc = up((void**)&ts.d_terms, ts.terms.data(), ts.terms.size() * sizeof(TcTerm)))) break;
    if ((rc = up((void**)&ts.d_dyn, ts.dyn_jobs.data(), ts.dyn_jobs.size() * sizeof(PackJob)))) break;
  }
  if (!rc) rc = up((void**)&T->d_static, T->static_jobs.data(), T->static_jobs.size() * sizeof(PackJob));
  if (!rc && cudaMalloc(&T->packed, std::max<int64_t>(T->packed_elems, 8) * sizeof(__nv_bfloat16)) != cudaSuccess)
    rc = IMPS_ERR_OOM;
  if (!rc && cudaMalloc(&T->d_err, sizeof(int)) != cudaSuccess) rc = IMPS_ERR_OOM;
  if (!rc) cudaMemsetAsync(T->d_err, 0, sizeof(int), st);
  if (!rc) {
    cudaError_t e = cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) {
      fprintf(stderr, "imps_gb300: tcgen05 kernel setup failed: %s\n", cudaGetErrorString(e));
      rc = IMPS_ERR_CUDA;
    }
  }
  if (rc) { tc_destroy(T); return rc; }
  T->first_stage = P.stages.empty() ? nullptr : &P.stages[0];
  *out = T;
  return IMPS_OK;
}

int tc_destroy(TcPlan* T) {
  if (!T) return IMPS_OK;
  for (TcStage& ts : T->stages) { cudaFree(ts.d_tiles); cudaFree(ts.d_terms); cudaFree(ts.d_dyn); }
  cudaFree(T->d_static);
  cudaFree(T->packed);
  cudaFree(T->d_err);
  delete T;
  return IMPS_OK;
}

int tc_invalidate(TcPlan* T) {
  if (T) T->static_valid = false;
  return IMPS_OK;
}

static int launch_pack(const PackJob* d_jobs, int n, const imps_dslots& slots, __nv_bfloat16* out, cudaStream_t st) {
  if (n <= 0) return IMPS_OK;
  dim3 grid(n, 4);
  imps::count_launch();
  pack_kernel<<<grid, 256, 0, st>>>(d_jobs, slots, out);
  return cudaGetLastError() == cudaSuccess ? IMPS_OK : IMPS_ERR_CUDA;
}

int tc_run_stage(TcPlan* T, const Stage& S, const imps_dslots& slots, cudaStream_t st) {
  // locate the stage index by address (stages are stored in the same order)
  size_t si = (size_t)(&S - T->first_stage);
  if (!T->first_stage || si >= T->stages.size()) return IMPS_ERR_BAD_ARG;
  if (!T->static_valid) {
    int rc = launch_pack(T->d_static, (int)T->static_jobs.size(), slots, T->packed, st);
    if (rc) return rc;
    T->static_valid = true;
  }
  TcStage& ts = T->stages[si];
  int rc = launch_pack(ts.d_dyn, (int)ts.dyn_jobs.size(), slots, T->packed, st);
  if (rc) return rc;
  if (!ts.tiles.empty()) {
    imps::count_launch();
    tc_gemm_kernel<<<(int)ts.tiles.size(), TC_THREADS, SMEM_BYTES, st>>>(ts.d_tiles, ts.d_terms, T->packed, slots,
                                                                        T->d_err);
    if (cudaGetLastError() != cudaSuccess) return IMPS_ERR_CUDA;
  }
  return IMPS_OK;
}

int tc_error_flag(TcPlan* T, int* flag) {
  if (!T || !flag) return IMPS_ERR_BAD_ARG;
  if (cudaMemcpy(flag, T->d_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return IMPS_ERR_CUDA;
  return IMPS_OK;
}

}  // namespace imps
