// C ABI of imps_gb300: contexts, sector tables, compiled contraction plans, the
// reference-facing functors and the device Krylov solvers.
#include <cuda_runtime.h>

#include <array>
#include <mutex>
#include <unordered_map>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <limits>
#include <new>
#include <vector>

#include "../../include/imps_gb300.h"
#include "imps_decomp.h"
#include "imps_handles.h"
#include "imps_internal.h"
#include "imps_krylov.h"
#include "imps_tc.h"
#include "imps_nonsym.h"
#include "imps_tridiag.h"

using namespace imps;

struct imps_ctx {
  int device = 0;
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  KrylovWs ws;
  double* dscal = nullptr;  // 64 device scalars
  int* dflag = nullptr;     // 16 device flags
  char* arena = nullptr;
  size_t arena_bytes = 0;
  // a second arena for solvers whose operator is a caller's callback: the callback may run
  // solvers of its own on this context, which take the first arena
  char* arena_cb = nullptr;
  size_t arena_cb_bytes = 0;
  // pinned staging of solver convergence data (projected-matrix columns + flags), so that the
  // device-to-host copies are asynchronous and a check can be evaluated while the next
  // Krylov step runs
  double* hpin = nullptr;   // kPinDoubles doubles, then 16 ints
  // the GMRES core's own staging (its solves run inside eigensolver callbacks, between an
  // eigensolver's staging and its check)
  double* hpin_g = nullptr;  // kPinDoubles doubles, then 16 ints
  cudaEvent_t ev_check = nullptr;
};
constexpr size_t kPinDoubles = (size_t)(imps::kMaxCols + 1) * (imps::kMaxCols + 1);


struct imps_plan {
  imps_ctx* ctx = nullptr;
  Plan P;
  double* stage_in = nullptr;
  double* stage_out = nullptr;
  double* stage_aux[2] = {nullptr, nullptr};
  // in-layout tables (TM plans): block offsets / dims for traces
  int64_t* d_boff = nullptr;
  int32_t* d_bdim = nullptr;   // rows
  int32_t* d_bcols = nullptr;  // cols (mixed TM plans: general BlockMat input)
  int nb_in = 0;
  Layout in_layout;
  // gradient plan segments
  int64_t* d_soff = nullptr;
  int64_t* d_slen = nullptr;
  int nseg = 0;
  int64_t count_elems = 0;
  int prec = IMPS_PREC_FP64;
  TcPlan* tc = nullptr;
  DecompPlan* dc = nullptr;
};

std::atomic<long long>& imps::launch_counter() {
  static std::atomic<long long> n{0};
  return n;
}

constexpr int PLAN_DECOMP = 12;
constexpr double kMixedEigTol = 2e-7;    // Ritz-residual floor of split-BF16 applies
constexpr double kAttainableRes = 64.0;  // FP64 Lanczos residual floor, in units of eps |T|
constexpr int CGS_BATCH_GRID = 152;      // row blocks per system of kr_cgs2_step_batch (its CGRID)
constexpr double kMixedInnerTol = 1e-6;  // residual reduction per mixed GMRES cycle
constexpr double kDominantTolFloor = 1e-14;  // attainable residual of the fixed-point solve

namespace {

#define CK(x)                                                        \
  do {                                                               \
    cudaError_t e_ = (x);                                            \
    if (e_ != cudaSuccess) {                                         \
      fprintf(stderr, "imps_gb300: %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
      return e_ == cudaErrorMemoryAllocation ? IMPS_ERR_OOM : IMPS_ERR_CUDA;                   \
    }                                                                \
  } while (0)

#define RC(x)              \
  do {                     \
    int r_ = (x);          \
    if (r_ < 0) return r_; \
  } while (0)

std::vector<HNnz> make_h(int nnz, const int32_t* r, const int32_t* c, const double* v) {
  std::vector<HNnz> h;
  for (int i = 0; i < nnz; ++i) h.push_back({r[i], c[i], v[i]});
  return h;
}

// ---- FP64 grouped-GEMM launch shape per stage: tile size and split-K ----
// A stage's work is set by the histogram of its output blocks (rows, cols, summed K, terms).
// The autotuner (imps_plan_autotune) times every candidate shape of a stage once and caches the
// fastest under the hash of that histogram; stages of later plans with the same histogram take
// the cached shape, others the makespan estimate below.
struct TuneChoice {
  int T = 16, splits = 1;
  float us = 0.f;
};
static std::mutex g_tune_mu;
static std::unordered_map<uint64_t, TuneChoice> g_tune;

static uint64_t stage_key(const Stage& S) {
  std::vector<std::array<int64_t, 4>> h;
  h.reserve(S.outs.size());
  for (const OutBlock& o : S.outs) {
    int64_t k = 0;
    for (int t = o.t0; t < o.t1; ++t) k += S.terms[t].k;
    h.push_back({(int64_t)o.M, (int64_t)o.N, k, (int64_t)(o.t1 - o.t0)});
  }
  std::sort(h.begin(), h.end());
  uint64_t x = 1469598103934665603ull;  // FNV-1a over the sorted histogram
  auto mix = [&](uint64_t v) {
    for (int b = 0; b < 8; ++b) { x ^= (v >> (8 * b)) & 0xFF; x *= 1099511628211ull; }
  };
  mix(h.size());
  for (const auto& e : h)
    for (int64_t v : e) mix((uint64_t)v);
  return x;
}

// largest useful split for tile size T: at least one K chunk per K group of the kernel
static int max_splits(const Stage& S, int T) {
  int max_chunks = 0;
  for (const OutBlock& o : S.outs) {
    int ch = 0;
    for (int t = o.t0; t < o.t1; ++t) ch += (S.terms[t].k + 15) / 16;
    max_chunks = std::max(max_chunks, ch);
  }
  return std::max(1, std::min(8, max_chunks / (T == 16 ? 4 : 2)));
}

// (re)build the stage's tiles for shape (T, splits) and upload them.  Split-K in proportion to
// the work: the tile with the most K chunks is split over `splits` CTAs, every other tile over
// ceil(splits x its chunks / the most chunks), each share keeping at least one chunk per K group
// of the kernel, so that the CTAs of a launch carry about equal work; the CTA entries are ordered
// by decreasing work.
static int install_stage(Stage& S, int T, int splits) {
  cudaFree(S.d_tiles); cudaFree(S.d_ws); cudaFree(S.d_cnt);
  S.d_tiles = nullptr; S.d_ws = nullptr; S.d_cnt = nullptr;
  finalize_tiles(S, T, T);
  S.splits = splits;
  const int ks = T == 16 ? 4 : 2;  // K groups of the kernel for this tile size
  const size_t ntiles = S.tiles.size();
  std::vector<int> ch(ntiles, 0);
  int cmax = 1;
  for (size_t i = 0; i < ntiles; ++i) {
    for (int t = S.tiles[i].t0; t < S.tiles[i].t1; ++t) ch[i] += (S.terms[t].k + 15) / 16;
    cmax = std::max(cmax, ch[i]);
  }
  std::vector<Tile> units;
  int nws = 0;
  for (size_t i = 0; i < ntiles; ++i) {
    Tile t = S.tiles[i];
    int np = splits > 1 ? (int)(((int64_t)ch[i] * splits + cmax - 1) / cmax) : 1;
    np = std::max(1, std::min(np, ch[i] / ks));
    t.nparts = np;
    t.cnt_idx = (int)i;
    t.ws_unit = np > 1 ? nws : 0;
    if (np > 1) nws += np;
    for (int q = 0; q < np; ++q) {
      t.part = q;
      units.push_back(t);
    }
  }
  std::stable_sort(units.begin(), units.end(), [&](const Tile& a, const Tile& b) {
    return (int64_t)ch[a.cnt_idx] * b.nparts > (int64_t)ch[b.cnt_idx] * a.nparts;
  });
  S.tiles = std::move(units);
  if (!S.tiles.empty()) {
    CK(cudaMalloc(&S.d_tiles, S.tiles.size() * sizeof(Tile)));
    CK(cudaMemcpy(S.d_tiles, S.tiles.data(), S.tiles.size() * sizeof(Tile), cudaMemcpyHostToDevice));
    if (S.splits > 1) {
      CK(cudaMalloc(&S.d_ws, (size_t)std::max(nws, 1) * T * T * sizeof(double)));
      CK(cudaMalloc(&S.d_cnt, std::max<size_t>(ntiles, 1) * sizeof(int)));
      CK(cudaMemset(S.d_cnt, 0, std::max<size_t>(ntiles, 1) * sizeof(int)));
    }
  }
  return IMPS_OK;
}

int upload_stage(Stage& S) {
  // tile size and split-K: minimise the estimated makespan of the FP64-pipe-bound kernel, the
  // larger of the heaviest tile's share (a tile's K chunks split over `splits` CTAs) and the
  // total padded work spread over the 152 SMs
  constexpr int kSMs = 152, kMaxSplits = 8;
  auto plan_for = [&](int T, int* splits_out) {
    int64_t crit = 0, total = 0;
    int max_chunks = 0;
    for (const OutBlock& o : S.outs) {
      int64_t k = 0;
      int ch = 0;
      for (int t = o.t0; t < o.t1; ++t) {
        k += S.terms[t].k;
        ch += (S.terms[t].k + 15) / 16;
      }
      crit = std::max(crit, (int64_t)std::min(T, o.M) * std::min(T, o.N) * k);
      total += (int64_t)((o.M + T - 1) / T * T) * ((o.N + T - 1) / T * T) * k;
      max_chunks = std::max(max_chunks, ch);
    }
    const int64_t spread = std::max<int64_t>(total / kSMs, 1);
    int sp = (int)std::min<int64_t>((crit + spread - 1) / spread, kMaxSplits);
    sp = std::max(1, std::min(sp, max_chunks / (T == 16 ? 4 : 2)));  // at least one chunk per K group
    *splits_out = sp;
    return std::max(crit / sp, spread);
  };
  int s16 = 1, s32 = 1;
  const int64_t m16 = plan_for(16, &s16), m32 = plan_for(32, &s32);
  int T = m16 <= m32 ? 16 : 32;
  int sp = T == 16 ? s16 : s32;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(stage_key(S));
    if (it != g_tune.end()) { T = it->second.T; sp = it->second.splits; }
  }
  RC(install_stage(S, T, sp));
  if (!S.terms.empty()) {
    CK(cudaMalloc(&S.d_terms, S.terms.size() * sizeof(Term)));
    CK(cudaMemcpy(S.d_terms, S.terms.data(), S.terms.size() * sizeof(Term), cudaMemcpyHostToDevice));
  }
  return IMPS_OK;
}

int finish_plan(imps_ctx* ctx, Plan& P, imps_plan** out) {
  imps_plan* p = new (std::nothrow) imps_plan();
  if (!p) return IMPS_ERR_OOM;
  p->ctx = ctx;
  p->P = std::move(P);
  if (ctx->device < 0) {  // host-only context: tables are built, nothing is uploaded
    for (Stage& S : p->P.prep) finalize_tiles(S, 32, 32);
    for (Stage& S : p->P.stages) finalize_tiles(S, 32, 32);
    *out = p;
    return IMPS_OK;
  }
  for (Slot& s : p->P.slots) {
    if (s.kind == SLOT_INTERNAL && s.nelem > 0) {
      cudaError_t e = cudaMalloc(&s.dptr, s.nelem * sizeof(double));
      if (e != cudaSuccess) { imps_plan_destroy(p); return IMPS_ERR_OOM; }
      cudaMemsetAsync(s.dptr, 0, s.nelem * sizeof(double), ctx->stream);
    }
  }
  for (Stage& S : p->P.prep) { int r = upload_stage(S); if (r) { imps_plan_destroy(p); return r; } }
  for (Stage& S : p->P.stages) { int r = upload_stage(S); if (r) { imps_plan_destroy(p); return r; } }
  *out = p;
  return IMPS_OK;
}

int run_stages(imps_plan* p, std::vector<Stage>& stages) {
  if (p->ctx->device < 0) return IMPS_ERR_NO_DEVICE;
  imps_dslots sl{};
  for (size_t i = 0; i < p->P.slots.size() && i < (size_t)kMaxSlots; ++i) sl.p[i] = p->P.slots[i].dptr;
  // every slot the stages read or write must be bound
  for (const Stage& S : stages) {
    for (const Term& t : S.terms)
      if (!sl.p[t.a_slot] || !sl.p[t.b_slot]) return IMPS_ERR_BAD_ARG;
    for (const OutBlock& o : S.outs)
      if (!sl.p[o.c_slot]) return IMPS_ERR_BAD_ARG;
  }
  // operator-dependent prepare stages always run in FP64; only apply stages use tensor cores
  const bool tc = p->prec == IMPS_PREC_BF16X6 && p->tc && &stages == &p->P.stages;
  for (Stage& S : stages) {
    if (tc) {
      RC(tc_run_stage(p->tc, S, sl, p->ctx->stream));
    } else {
      RC(imps_launch_grouped_f64(S.d_tiles, (int)S.tiles.size(), S.d_terms, sl, S.tile_m, S.splits, S.d_ws,
                                 S.d_cnt, p->ctx->stream));
    }
  }
  return IMPS_OK;
}

// ---- arena (per-context scratch, grows; never shrinks) ----
int arena_reserve(imps_ctx* c, size_t bytes, bool callback_arena = false) {
  char*& a = callback_arena ? c->arena_cb : c->arena;
  size_t& ab = callback_arena ? c->arena_cb_bytes : c->arena_bytes;
  if (bytes <= ab) return IMPS_OK;
  if (a) { cudaStreamSynchronize(c->stream); cudaFree(a); a = nullptr; ab = 0; }
  size_t nb = std::max(bytes, (size_t)1 << 20);
  CK(cudaMalloc(&a, nb));
  ab = nb;
  return IMPS_OK;
}

struct Bump {
  char* base;
  size_t used = 0;
  double* take(size_t n) {
    double* p = (double*)(base + used);
    used += ((n * sizeof(double) + 255) / 256) * 256;
    return p;
  }
};

size_t round256(size_t b) { return ((b + 255) / 256) * 256; }

// IMPS_DEBUG=1 in the environment prints one line per solver call to stderr
int debug_level() {
  static const int lvl = [] {
    const char* e = getenv("IMPS_DEBUG");
    return e && e[0] ? atoi(e) : 0;
  }();
  return lvl;
}
bool debug_on() { return debug_level() > 0; }

int stage_host(imps_plan* p, double** buf, int64_t n) {
  if (!*buf) CK(cudaMalloc(buf, std::max<int64_t>(n, 1) * sizeof(double)));
  return IMPS_OK;
}

// apply the plan's operator: IN -> OUT with device pointers
int apply_dev(imps_plan* p, const double* in, double* out) {
  p->P.slots[p->P.n_in].dptr = const_cast<double*>(in);
  p->P.slots[p->P.n_out].dptr = out;
  return run_stages(p, p->P.stages);
}

}  // namespace

// =====================================================================================
extern "C" {

const char* imps_status_string(int s) {
  switch (s) {
    case IMPS_OK: return "ok";
    case IMPS_WARN_NOT_CONVERGED: return "not converged";
    case IMPS_ERR_BAD_ARG: return "bad argument";
    case IMPS_ERR_BAD_TABLE: return "inconsistent sector table";
    case IMPS_ERR_CUDA: return "CUDA error";
    case IMPS_ERR_NAN: return "NaN/Inf detected";
    case IMPS_ERR_TIMEOUT: return "timeout";
    case IMPS_ERR_NO_DEVICE: return "no CUDA device";
    case IMPS_ERR_OOM: return "out of device memory";
    case IMPS_ERR_UNSUPPORTED: return "unsupported";
    case IMPS_ERR_TOO_LARGE: return "problem exceeds the fixed scratch of the no-allocation entry point";
    default: return "unknown status";
  }
}

int imps_version(void) { return 100; }

int64_t imps_launch_count(void) { return (int64_t)imps::launch_counter().load(); }

int imps_ctx_create(int device, imps_ctx** out) {
  if (!out) return IMPS_ERR_BAD_ARG;
  if (device == -1) {  // host-only context: sector tables and plans, no execution
    imps_ctx* c = new (std::nothrow) imps_ctx();
    if (!c) return IMPS_ERR_OOM;
    c->device = -1;
    *out = c;
    return IMPS_OK;
  }
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= device || device < 0) return IMPS_ERR_NO_DEVICE;
  CK(cudaSetDevice(device));
  imps_ctx* c = new (std::nothrow) imps_ctx();
  if (!c) return IMPS_ERR_OOM;
  c->device = device;
  CK(cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking));
  c->stream = c->own;
  CK(cudaMalloc(&c->ws.partials, kr_partials_elems() * sizeof(double)));
  CK(cudaMalloc(&c->ws.counter, 256));
  CK(cudaMemset(c->ws.counter, 0, 256));
  CK(cudaMalloc(&c->dscal, 64 * sizeof(double)));
  CK(cudaMemset(c->dscal, 0, 64 * sizeof(double)));
  CK(cudaMalloc(&c->dflag, 16 * sizeof(int)));
  CK(cudaMemset(c->dflag, 0, 16 * sizeof(int)));
  c->ws.sync = c->ws.counter + 1;  // counter[0]: last-block reductions; [1], [2]: grid barrier
  c->ws.err = c->dflag + 4;
  CK(cudaMallocHost(&c->hpin, kPinDoubles * sizeof(double) + 16 * sizeof(int)));
  CK(cudaMallocHost(&c->hpin_g, kPinDoubles * sizeof(double) + 16 * sizeof(int)));
  CK(cudaEventCreateWithFlags(&c->ev_check, cudaEventDisableTiming));
  *out = c;
  return IMPS_OK;
}

int imps_ctx_destroy(imps_ctx* c) {
  if (!c) return IMPS_OK;
  if (c->device < 0) { delete c; return IMPS_OK; }
  cudaStreamSynchronize(c->stream);
  cudaFree(c->ws.partials);
  cudaFree(c->ws.counter);
  cudaFree(c->dscal);
  cudaFree(c->dflag);
  if (c->hpin) cudaFreeHost(c->hpin);
  if (c->hpin_g) cudaFreeHost(c->hpin_g);
  if (c->ev_check) cudaEventDestroy(c->ev_check);
  if (c->arena) cudaFree(c->arena);
  if (c->arena_cb) cudaFree(c->arena_cb);
  if (c->own) cudaStreamDestroy(c->own);
  delete c;
  return IMPS_OK;
}

int imps_ctx_set_stream(imps_ctx* c, void* s) {
  if (!c) return IMPS_ERR_BAD_ARG;
  c->stream = (cudaStream_t)s;  // used as given: NULL is the CUDA legacy default stream
  return IMPS_OK;
}

int imps_ctx_use_own_stream(imps_ctx* c) {
  if (!c) return IMPS_ERR_BAD_ARG;
  c->stream = c->own;
  return IMPS_OK;
}

int imps_ctx_synchronize(imps_ctx* c) {
  if (!c) return IMPS_ERR_BAD_ARG;
  if (c->device < 0) return IMPS_OK;
  CK(cudaStreamSynchronize(c->stream));
  return IMPS_OK;
}

// ---- layouts ----
int imps_layout_create(int nsym, int nblocks, const int32_t* qin, const int32_t* qout,
                       const int32_t* rows, const int32_t* cols, const int32_t* group,
                       imps_layout** out) {
  if (!out || (nblocks > 0 && (!qin || !qout || !rows || !cols))) return IMPS_ERR_BAD_ARG;
  imps_layout* L = new (std::nothrow) imps_layout();
  if (!L) return IMPS_ERR_OOM;
  int r = layout_build(L->L, nsym, nblocks, qin, qout, rows, cols, group);
  if (r) { delete L; return r; }
  *out = L;
  return IMPS_OK;
}

int imps_layout_destroy(imps_layout* L) { delete L; return IMPS_OK; }
int64_t imps_layout_nelem(const imps_layout* L) { return L ? L->L.nelem : -1; }
int imps_layout_nblocks(const imps_layout* L) { return L ? (int)L->L.blocks.size() : -1; }
int imps_layout_nsym(const imps_layout* L) { return L ? L->L.nsym : -1; }

int imps_layout_get(const imps_layout* L, int32_t* qin, int32_t* qout, int32_t* rows, int32_t* cols,
                    int32_t* group, int64_t* off) {
  if (!L) return IMPS_ERR_BAD_ARG;
  const int ns = L->L.nsym;
  for (size_t b = 0; b < L->L.blocks.size(); ++b) {
    const Block& B = L->L.blocks[b];
    for (int k = 0; k < ns; ++k) {
      if (qin) qin[b * ns + k] = B.qin[k];
      if (qout) qout[b * ns + k] = B.qout[k];
    }
    if (rows) rows[b] = B.rows;
    if (cols) cols[b] = B.cols;
    if (group) group[b] = B.group;
    if (off) off[b] = B.off;
  }
  return IMPS_OK;
}

int imps_layout_bond(const imps_layout* A, int side, imps_layout** out) {
  if (!A || !out) return IMPS_ERR_BAD_ARG;
  imps_layout* L = new (std::nothrow) imps_layout();
  if (!L) return IMPS_ERR_OOM;
  L->L = layout_bond(A->L, side);
  *out = L;
  return IMPS_OK;
}

// ---- plans ----
int imps_plan_hac(imps_ctx* ctx, const imps_layout* AC, const imps_layout* EHL, const imps_layout* EHR,
                  const imps_layout* HL, const imps_layout* HR, int d, imps_plan** out) {
  if (!ctx || !AC || !EHL || !EHR || !HL || !HR || !out || d <= 0) return IMPS_ERR_BAD_ARG;
  Plan P;
  RC(build_hac(P, AC->L, EHL->L, EHR->L, HL->L, HR->L, d));
  RC(finish_plan(ctx, P, out));
  (*out)->in_layout = AC->L;
  return IMPS_OK;
}

int imps_plan_hc(imps_ctx* ctx, const imps_layout* C, const imps_layout* EHL, const imps_layout* EHR,
                 const imps_layout* AL, const imps_layout* AR, int d, int nnz, const int32_t* hrow,
                 const int32_t* hcol, const double* hval, imps_plan** out) {
  if (!ctx || !C || !EHL || !EHR || !AL || !AR || !out || d <= 0 || nnz < 0) return IMPS_ERR_BAD_ARG;
  Plan P;
  RC(build_hc(P, C->L, EHL->L, EHR->L, AL->L, AR->L, d, make_h(nnz, hrow, hcol, hval)));
  RC(finish_plan(ctx, P, out));
  (*out)->in_layout = C->L;
  return IMPS_OK;
}

int imps_plan_tm(imps_ctx* ctx, int nsites, const imps_layout* const* A, int dir, const imps_layout* in,
                 const imps_layout* outl, imps_plan** out) {
  if (!ctx || !A || !in || !outl || !out || nsites < 1 || (dir != 0 && dir != 1)) return IMPS_ERR_BAD_ARG;
  std::vector<const Layout*> As;
  for (int k = 0; k < nsites; ++k) {
    if (!A[k]) return IMPS_ERR_BAD_ARG;
    As.push_back(&A[k]->L);
  }
  Plan P;
  RC(build_tm(P, As, dir, in->L, outl->L));
  RC(finish_plan(ctx, P, out));
  imps_plan* p = *out;
  p->in_layout = in->L;
  // block tables of the in layout for traces / identity
  std::vector<int64_t> bo;
  std::vector<int32_t> bd;
  for (const Block& b : in->L.blocks) { bo.push_back(b.off); bd.push_back(b.rows); }
  p->nb_in = (int)bo.size();
  if (p->nb_in && ctx->device >= 0) {
    CK(cudaMalloc(&p->d_boff, bo.size() * sizeof(int64_t)));
    CK(cudaMalloc(&p->d_bdim, bd.size() * sizeof(int32_t)));
    CK(cudaMemcpy(p->d_boff, bo.data(), bo.size() * sizeof(int64_t), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(p->d_bdim, bd.data(), bd.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
  }
  return IMPS_OK;
}

int imps_plan_tm_mixed(imps_ctx* ctx, int nsites, const imps_layout* const* A, const imps_layout* const* B,
                       int dir, const imps_layout* in, const imps_layout* outl, imps_plan** out) {
  if (!ctx || !A || !B || !in || !outl || !out || nsites < 1 || (dir != 0 && dir != 1)) return IMPS_ERR_BAD_ARG;
  std::vector<const Layout*> As, Bs;
  for (int k = 0; k < nsites; ++k) {
    if (!A[k] || !B[k]) return IMPS_ERR_BAD_ARG;
    As.push_back(&A[k]->L);
    Bs.push_back(&B[k]->L);
  }
  Plan P;
  RC(build_tm_mixed(P, As, Bs, dir, in->L, outl->L));
  RC(finish_plan(ctx, P, out));
  imps_plan* p = *out;
  p->in_layout = in->L;
  std::vector<int64_t> bo;
  std::vector<int32_t> br, bc;
  for (const Block& b : in->L.blocks) { bo.push_back(b.off); br.push_back(b.rows); bc.push_back(b.cols); }
  p->nb_in = (int)bo.size();
  if (p->nb_in && ctx->device >= 0) {
    CK(cudaMalloc(&p->d_boff, bo.size() * sizeof(int64_t)));
    CK(cudaMalloc(&p->d_bdim, br.size() * sizeof(int32_t)));
    CK(cudaMalloc(&p->d_bcols, bc.size() * sizeof(int32_t)));
    CK(cudaMemcpy(p->d_boff, bo.data(), bo.size() * sizeof(int64_t), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(p->d_bdim, br.data(), br.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(p->d_bcols, bc.data(), bc.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
  }
  return IMPS_OK;
}

// A grouped-GEMM program given as explicit tables (every slot external): used for
// contractions whose sector matching is compiled by a caller (the excitation effective
// Hamiltonian).  Every term's operands and every output region are bounds-checked against
// the slot sizes here, so a table can never make a kernel access memory outside its slots.
int imps_plan_replicate(const imps_plan* src, int copies, imps_plan** out) {
  if (!src || copies < 1 || !out) return IMPS_ERR_BAD_ARG;
  const Plan& S = src->P;
  if (!S.prep.empty()) return IMPS_ERR_UNSUPPORTED;  // operator-derived stages would need sharing rules
  Plan Q;
  Q.kind = PLAN_PROGRAM;
  // per copy: the input, the output and the plan's own scratch; shared: the operator slots
  std::vector<char> per(S.slots.size(), 0);
  for (size_t i = 0; i < S.slots.size(); ++i) {
    per[i] = S.slots[i].kind == SLOT_INTERNAL || (int)i == S.n_in || (int)i == S.n_out;
    Slot sl = S.slots[i];
    if (per[i]) sl.nelem *= copies;
    if (sl.kind == SLOT_INTERNAL || per[i]) sl.dptr = nullptr;  // operators keep their bindings
    Q.slots.push_back(sl);
  }
  Q.n_in = S.n_in;
  Q.n_out = S.n_out;
  for (const Stage& st : S.stages) {
    Stage R;
    for (int c = 0; c < copies; ++c) {
      for (const OutBlock& o : st.outs) {
        OutBlock ob = o;
        if (per[o.c_slot]) ob.c_off += (int64_t)c * S.slots[o.c_slot].nelem;
        ob.t0 = (int32_t)R.terms.size();
        for (int t = o.t0; t < o.t1; ++t) {
          Term tm = st.terms[t];
          if (per[tm.a_slot]) tm.a_off += (int64_t)c * S.slots[tm.a_slot].nelem;
          if (per[tm.b_slot]) tm.b_off += (int64_t)c * S.slots[tm.b_slot].nelem;
          R.terms.push_back(tm);
        }
        ob.t1 = (int32_t)R.terms.size();
        R.outs.push_back(ob);
      }
    }
    R.flops = st.flops * copies;
    Q.stages.push_back(std::move(R));
  }
  Q.flops_apply = S.flops_apply * copies;
  Q.dropped = S.dropped * copies;
  return finish_plan(src->ctx, Q, out);
}

int imps_plan_program(imps_ctx* ctx, int nslots, const int64_t* slot_nelem, int nstages,
                      const int32_t* stage_nouts, const int64_t* outs, const int64_t* terms,
                      const double* alphas, imps_plan** out) {
  if (!ctx || !slot_nelem || nslots < 1 || nslots > kMaxSlots || nstages < 0 || (nstages && !stage_nouts) || !out)
    return IMPS_ERR_BAD_ARG;
  Plan P;
  P.kind = PLAN_PROGRAM;
  for (int i = 0; i < nslots; ++i) {
    if (slot_nelem[i] < 0) return IMPS_ERR_BAD_ARG;
    Slot sl;
    sl.kind = SLOT_EXTERNAL;
    sl.nelem = slot_nelem[i];
    sl.name = "p";
    P.slots.push_back(sl);
  }
  P.n_in = 0;
  P.n_out = nslots > 1 ? 1 : 0;
  auto within = [&](int64_t slot, int64_t off, int64_t ld, int64_t r, int64_t c) {
    if (slot < 0 || slot >= nslots || off < 0 || r < 0 || c < 0) return false;
    if (r == 0 || c == 0) return true;
    if (ld < r) return false;
    return off + (r - 1) + (c - 1) * ld < slot_nelem[slot];
  };
  int64_t o = 0, t = 0;
  for (int sidx = 0; sidx < nstages; ++sidx) {
    P.stages.emplace_back();
    Stage& S = P.stages.back();
    for (int q = 0; q < stage_nouts[sidx]; ++q, ++o) {
      const int64_t* od = outs + 7 * o;
      const int64_t cs = od[0], coff = od[1], cld = od[2], M = od[3], N = od[4], acc = od[5], nt = od[6];
      if (!within(cs, coff, cld, M, N) || nt < 0 || M > INT32_MAX || N > INT32_MAX) return IMPS_ERR_BAD_TABLE;
      OutBlock ob{};
      ob.c_slot = (int16_t)cs;
      ob.c_off = coff;
      ob.c_ld = (int32_t)std::max<int64_t>(cld, 1);
      ob.M = (int32_t)M;
      ob.N = (int32_t)N;
      ob.accumulate = (int16_t)(acc ? 1 : 0);
      ob.tag = q;
      ob.t0 = (int32_t)S.terms.size();
      for (int64_t e = 0; e < nt; ++e, ++t) {
        const int64_t* td = terms + 9 * t;
        const int64_t as = td[0], aoff = td[1], ald = td[2], at = td[3], bs = td[4], boff = td[5], bld = td[6],
                      bt = td[7], k = td[8];
        // op(A) is M x k (stored k x M when transposed), op(B) is k x N (stored N x k)
        const bool okA = at ? within(as, aoff, ald, k, M) : within(as, aoff, ald, M, k);
        const bool okB = bt ? within(bs, boff, bld, N, k) : within(bs, boff, bld, k, N);
        if (!okA || !okB || k < 0 || k > INT32_MAX || ald > INT32_MAX || bld > INT32_MAX) return IMPS_ERR_BAD_TABLE;
        Term tm{};
        tm.a_slot = (int16_t)as;
        tm.a_off = aoff;
        tm.a_ld = (int32_t)std::max<int64_t>(ald, 1);
        tm.a_t = (int8_t)(at ? 1 : 0);
        tm.b_slot = (int16_t)bs;
        tm.b_off = boff;
        tm.b_ld = (int32_t)std::max<int64_t>(bld, 1);
        tm.b_t = (int8_t)(bt ? 1 : 0);
        tm.k = (int32_t)k;
        tm.alpha = alphas[t];
        S.terms.push_back(tm);
        S.flops += 2LL * M * N * k;
      }
      ob.t1 = (int32_t)S.terms.size();
      S.outs.push_back(ob);
    }
  }
  for (auto& st : P.stages) P.flops_apply += st.flops;
  return finish_plan(ctx, P, out);
}

int imps_plan_redop(imps_ctx* ctx, const imps_layout* A, int d, int nnz, const int32_t* hrow,
                    const int32_t* hcol, const double* hval, int dir, imps_plan** out) {
  if (!ctx || !A || !out || d <= 0 || nnz < 0) return IMPS_ERR_BAD_ARG;
  Plan P;
  RC(build_redop(P, A->L, d, make_h(nnz, hrow, hcol, hval), dir));
  return finish_plan(ctx, P, out);
}

int imps_plan_optm(imps_ctx* ctx, const imps_layout* A0, const imps_layout* A1, int d, int nnz,
                   const int32_t* hrow, const int32_t* hcol, const double* hval, int dir,
                   const imps_layout* outl, imps_plan** out) {
  if (!ctx || !A0 || !A1 || !outl || !out || d <= 0) return IMPS_ERR_BAD_ARG;
  Plan P;
  RC(build_optm(P, A0->L, A1->L, d, make_h(nnz, hrow, hcol, hval), dir, outl->L));
  return finish_plan(ctx, P, out);
}

int imps_plan_mps_bd(imps_ctx* ctx, const imps_layout* A, const imps_layout* X, int side, double alpha,
                     imps_plan** out) {
  if (!ctx || !A || !X || !out) return IMPS_ERR_BAD_ARG;
  Plan P;
  RC(build_mps_bd(P, A->L, X->L, side, alpha));
  return finish_plan(ctx, P, out);
}

int imps_plan_grad_right(imps_ctx* ctx, const imps_layout* Y, const imps_layout* AR, imps_plan** out) {
  if (!ctx || !Y || !AR || !out) return IMPS_ERR_BAD_ARG;
  Plan P;
  RC(build_grad_right(P, Y->L, AR->L));
  RC(finish_plan(ctx, P, out));
  imps_plan* p = *out;
  // segments: AR blocks whose left sector has a right null space (mr_tot > ml),
  // Nullspace(AR, r) of MPSBlockUtilities.hpp:299-321
  std::map<Key, std::pair<int64_t, int64_t>> sec;  // qin -> (ml, mr_tot)
  for (const Block& b : AR->L.blocks) {
    auto& e = sec[b.qin];
    e.first = b.rows;
    e.second += b.cols;
  }
  std::vector<int64_t> so, sl;
  int64_t count = 0;
  for (const Block& b : AR->L.blocks) {
    auto& e = sec[b.qin];
    if (e.second > e.first) { so.push_back(b.off); sl.push_back((int64_t)b.rows * b.cols); }
  }
  for (auto& kv : sec)
    if (kv.second.second > kv.second.first) count += kv.second.first * (kv.second.second - kv.second.first);
  p->nseg = (int)so.size();
  p->count_elems = count;
  if (p->nseg && ctx->device >= 0) {
    CK(cudaMalloc(&p->d_soff, so.size() * sizeof(int64_t)));
    CK(cudaMalloc(&p->d_slen, sl.size() * sizeof(int64_t)));
    CK(cudaMemcpy(p->d_soff, so.data(), so.size() * sizeof(int64_t), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(p->d_slen, sl.data(), sl.size() * sizeof(int64_t), cudaMemcpyHostToDevice));
  }
  return IMPS_OK;
}

int imps_plan_destroy(imps_plan* p) {
  if (!p) return IMPS_OK;
  if (p->ctx && p->ctx->device < 0) { delete p->dc; delete p; return IMPS_OK; }
  if (p->ctx) cudaStreamSynchronize(p->ctx->stream);
  for (Slot& s : p->P.slots)
    if (s.kind == SLOT_INTERNAL && s.dptr) cudaFree(s.dptr);
  for (auto* v : {&p->P.prep, &p->P.stages})
    for (Stage& S : *v) {
      if (S.d_tiles) cudaFree(S.d_tiles);
      if (S.d_terms) cudaFree(S.d_terms);
      if (S.d_ws) cudaFree(S.d_ws);
      if (S.d_cnt) cudaFree(S.d_cnt);
    }
  cudaFree(p->stage_in);
  cudaFree(p->stage_out);
  cudaFree(p->stage_aux[0]);
  cudaFree(p->stage_aux[1]);
  cudaFree(p->d_boff);
  cudaFree(p->d_bdim);
  cudaFree(p->d_bcols);
  cudaFree(p->d_soff);
  cudaFree(p->d_slen);
  if (p->tc) tc_destroy(p->tc);
  if (p->dc) {
    cudaFree(p->dc->d_ent); cudaFree(p->dc->d_mats); cudaFree(p->dc->dA); cudaFree(p->dc->dQ);
    cudaFree(p->dc->dR); cudaFree(p->dc->dV2); cudaFree(p->dc->dS); cudaFree(p->dc->dW);
    cudaFree(p->dc->dstatus);
    cudaFree(p->dc->dNS); cudaFree(p->dc->d_nent);
    delete p->dc;
  }
  delete p;
  return IMPS_OK;
}

int imps_plan_derived_layout(const imps_plan* p, int which, imps_layout** out) {
  if (!p || !out || which < 0 || which >= (int)p->P.derived.size()) return IMPS_ERR_BAD_ARG;
  imps_layout* L = new (std::nothrow) imps_layout();
  if (!L) return IMPS_ERR_OOM;
  L->L = p->P.derived[which];
  *out = L;
  return IMPS_OK;
}

int imps_plan_info(const imps_plan* p, int64_t* fa, int64_t* fp, int64_t* dropped, int* nslots, int* nstages) {
  if (!p) return IMPS_ERR_BAD_ARG;
  if (fa) *fa = p->P.flops_apply;
  if (fp) *fp = p->P.flops_prep;
  if (dropped) *dropped = p->P.dropped;
  if (nslots) *nslots = (int)p->P.slots.size();
  if (nstages) *nstages = (int)p->P.stages.size();
  return IMPS_OK;
}

int imps_plan_slot_info(const imps_plan* p, int slot, int* kind, int64_t* nelem) {
  if (!p || slot < 0 || slot >= (int)p->P.slots.size()) return IMPS_ERR_BAD_ARG;
  if (kind) *kind = p->P.slots[slot].kind;
  if (nelem) *nelem = p->P.slots[slot].nelem;
  return IMPS_OK;
}

int imps_plan_bind(imps_plan* p, int slot, double* ptr) {
  if (!p || slot < 0 || slot >= (int)p->P.slots.size()) return IMPS_ERR_BAD_ARG;
  if (p->P.slots[slot].kind != SLOT_EXTERNAL) return IMPS_ERR_BAD_ARG;
  // (re)binding an operator slot means its contents may have changed: the tensor-core
  // operand packs are rebuilt on the next run
  if (p->tc && slot != p->P.n_in && slot != p->P.n_out) tc_invalidate(p->tc);
  p->P.slots[slot].dptr = ptr;
  return IMPS_OK;
}

int imps_plan_prepare(imps_plan* p) {
  if (!p) return IMPS_ERR_BAD_ARG;
  RC(run_stages(p, p->P.prep));
  if (p->tc) RC(tc_invalidate(p->tc));
  return IMPS_OK;
}

int imps_plan_run(imps_plan* p) {
  if (!p) return IMPS_ERR_BAD_ARG;
  return run_stages(p, p->P.stages);
}

int imps_plan_table(const imps_plan* p, int prep, int stage, int64_t* n_outs, int64_t* n_terms,
                    int32_t* out_tag, int32_t* out_t0, int32_t* out_t1, int32_t* term_aslot,
                    int64_t* term_aoff, int32_t* term_bslot, int64_t* term_boff, int32_t* term_k,
                    double* term_alpha) {
  if (!p) return IMPS_ERR_BAD_ARG;
  const std::vector<Stage>& v = prep ? p->P.prep : p->P.stages;
  if (stage < 0 || stage >= (int)v.size()) return IMPS_ERR_BAD_ARG;
  const Stage& S = v[stage];
  if (n_outs) *n_outs = (int64_t)S.outs.size();
  if (n_terms) *n_terms = (int64_t)S.terms.size();
  for (size_t i = 0; i < S.outs.size(); ++i) {
    if (out_tag) out_tag[i] = S.outs[i].tag;
    if (out_t0) out_t0[i] = S.outs[i].t0;
    if (out_t1) out_t1[i] = S.outs[i].t1;
  }
  for (size_t i = 0; i < S.terms.size(); ++i) {
    const Term& t = S.terms[i];
    if (term_aslot) term_aslot[i] = t.a_slot;
    if (term_aoff) term_aoff[i] = t.a_off;
    if (term_bslot) term_bslot[i] = t.b_slot;
    if (term_boff) term_boff[i] = t.b_off;
    if (term_k) term_k[i] = t.k;
    if (term_alpha) term_alpha[i] = t.alpha;
  }
  return IMPS_OK;
}

int imps_plan_autotune(imps_plan* p, int reps, int* n_tuned) {
  if (!p) return IMPS_ERR_BAD_ARG;
  if (p->ctx->device < 0) return IMPS_ERR_NO_DEVICE;
  if (reps < 1) reps = 5;
  cudaStream_t st = p->ctx->stream;
  // the candidates run on zero-filled stand-ins of the caller's slots (the plan's own scratch
  // slots are used as they are), so no bound buffer is read or written
  imps_dslots sl{};
  std::vector<double*> temps;
  auto free_temps = [&]() { for (double* t : temps) cudaFree(t); };
  for (size_t i = 0; i < p->P.slots.size() && i < (size_t)kMaxSlots; ++i) {
    const Slot& sd = p->P.slots[i];
    if (sd.kind == SLOT_INTERNAL) { sl.p[i] = sd.dptr; continue; }
    if (sd.nelem <= 0) continue;
    double* t = nullptr;
    if (cudaMalloc(&t, sd.nelem * sizeof(double)) != cudaSuccess) { free_temps(); return IMPS_ERR_OOM; }
    temps.push_back(t);
    if (cudaMemsetAsync(t, 0, sd.nelem * sizeof(double), st) != cudaSuccess) { free_temps(); return IMPS_ERR_CUDA; }
    sl.p[i] = t;
  }
  for (const Stage& S : p->P.stages) {
    for (const Term& t : S.terms)
      if (!sl.p[t.a_slot] || !sl.p[t.b_slot]) { free_temps(); return IMPS_ERR_BAD_TABLE; }
    for (const OutBlock& o : S.outs)
      if (!sl.p[o.c_slot]) { free_temps(); return IMPS_ERR_BAD_TABLE; }
  }
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) { free_temps(); return IMPS_ERR_CUDA; }
  if (cudaEventCreate(&e1) != cudaSuccess) { cudaEventDestroy(e0); free_temps(); return IMPS_ERR_CUDA; }
  int tuned = 0, rc = IMPS_OK;
  for (Stage& S : p->P.stages) {
    if (S.outs.empty() || S.terms.empty()) continue;
    const uint64_t key = stage_key(S);
    TuneChoice best;
    bool have = false;
    {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      auto it = g_tune.find(key);
      if (it != g_tune.end()) { best = it->second; have = true; }
    }
    if (!have) {
      best.us = std::numeric_limits<float>::infinity();
      for (int T : {16, 32}) {
        const int smax = max_splits(S, T);
        for (int sp = 1; sp <= smax && !rc; sp *= 2) {
          if ((rc = install_stage(S, T, sp))) break;
          auto launch = [&]() {
            return imps_launch_grouped_f64(S.d_tiles, (int)S.tiles.size(), S.d_terms, sl, S.tile_m, S.splits,
                                           S.d_ws, S.d_cnt, st);
          };
          if ((rc = launch())) break;  // warm-up
          std::vector<float> ts;
          for (int r = 0; r < reps && !rc; ++r) {
            if (cudaEventRecord(e0, st) != cudaSuccess) { rc = IMPS_ERR_CUDA; break; }
            rc = launch();
            if (rc || cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
              if (!rc) rc = IMPS_ERR_CUDA;
              break;
            }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            ts.push_back(ms * 1e3f);
          }
          if (rc) break;
          std::sort(ts.begin(), ts.end());
          const float us = ts[ts.size() / 2];
          if (us < best.us) { best.T = T; best.splits = sp; best.us = us; }
        }
        if (rc) break;
      }
      if (rc) break;
      std::lock_guard<std::mutex> lk(g_tune_mu);
      g_tune[key] = best;
      ++tuned;
    }
    if (S.tile_m != best.T || S.splits != best.splits)
      if ((rc = install_stage(S, best.T, best.splits))) break;
  }
  if (cudaStreamSynchronize(st) != cudaSuccess && !rc) rc = IMPS_ERR_CUDA;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  free_temps();
  if (n_tuned) *n_tuned = tuned;
  return rc;
}

int imps_plan_stage_shape(const imps_plan* p, int stage, int* tile, int* splits, uint64_t* key) {
  if (!p || stage < 0 || stage >= (int)p->P.stages.size()) return IMPS_ERR_BAD_ARG;
  const Stage& S = p->P.stages[stage];
  if (tile) *tile = S.tile_m;
  if (splits) *splits = S.splits;
  if (key) *key = stage_key(S);
  return IMPS_OK;
}

int imps_autotune_clear(void) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune.clear();
  return IMPS_OK;
}

int imps_plan_set_precision(imps_plan* p, int prec) {
  if (!p) return IMPS_ERR_BAD_ARG;
  if (prec == IMPS_PREC_FP64) { p->prec = prec; return IMPS_OK; }
  if (prec != IMPS_PREC_BF16X6) return IMPS_ERR_BAD_ARG;
  if (!p->tc) RC(tc_create(&p->tc, p->P, p->ctx->stream));
  p->prec = prec;
  return IMPS_OK;
}

// ---- functors ----
static int apply_mem(imps_plan* p, const double* in, double* out, int mem) {
  if (!p || !in || !out) return IMPS_ERR_BAD_ARG;
  const int64_t nin = p->P.slots[p->P.n_in].nelem, nout = p->P.slots[p->P.n_out].nelem;
  cudaStream_t st = p->ctx->stream;
  if (mem == IMPS_MEM_DEVICE) return apply_dev(p, in, out);
  RC(stage_host(p, &p->stage_in, nin));
  RC(stage_host(p, &p->stage_out, nout));
  CK(cudaMemcpyAsync(p->stage_in, in, nin * sizeof(double), cudaMemcpyHostToDevice, st));
  RC(apply_dev(p, p->stage_in, p->stage_out));
  CK(cudaMemcpyAsync(out, p->stage_out, nout * sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return IMPS_OK;
}

int imps_hac_apply(imps_plan* p, const double* in, double* out, int mem) {
  if (!p || p->P.kind != PLAN_HAC) return IMPS_ERR_BAD_ARG;
  return apply_mem(p, in, out, mem);
}

int imps_hc_apply(imps_plan* p, const double* in, double* out, int mem) {
  if (!p || p->P.kind != PLAN_HC) return IMPS_ERR_BAD_ARG;
  return apply_mem(p, in, out, mem);
}

static bool is_mixed_tm(const imps_plan* p) {
  return p && (p->P.kind == PLAN_TMMIXED_L || p->P.kind == PLAN_TMMIXED_R);
}

int imps_tm_apply(imps_plan* p, const double* in, double* out, int mem) {
  if (!p || (p->P.kind != PLAN_TM && !is_mixed_tm(p))) return IMPS_ERR_BAD_ARG;
  return apply_mem(p, in, out, mem);
}

// device-side InvEfun_proj: y = x - T(x) + tr(x*rho_in) * rho_out (tmp: n doubles)
static int proj_apply_dev(imps_plan* p, const double* x, const double* rho_in, const double* rho_out,
                          double* y, double* tmp, double* dtr) {
  imps_ctx* c = p->ctx;
  const int64_t n = p->P.slots[0].nelem;
  RC(kr_trace_prod(c->ws, x, rho_in, p->d_boff, p->d_bdim, p->nb_in, dtr, c->stream));
  RC(apply_dev(p, x, tmp));
  RC(kr_proj_epilogue(x, tmp, dtr, rho_out, y, n, c->stream));
  return IMPS_OK;
}

int imps_tm_proj_apply(imps_plan* p, const double* in, const double* rho_in, const double* rho_out,
                       double* out, int mem) {
  if (!p || p->P.kind != PLAN_TM || !in || !rho_in || !rho_out || !out) return IMPS_ERR_BAD_ARG;
  imps_ctx* c = p->ctx;
  const int64_t n = p->P.slots[0].nelem;
  if (p->P.slots[1].nelem != n) return IMPS_ERR_BAD_ARG;
  RC(arena_reserve(c, round256(n * 8) * 5));
  Bump bp{c->arena};
  double* tmp = bp.take(n);
  if (mem == IMPS_MEM_DEVICE) return proj_apply_dev(p, in, rho_in, rho_out, out, tmp, c->dscal);
  double* x = bp.take(n);
  double* ri = bp.take(n);
  double* ro = bp.take(n);
  double* y = bp.take(n);
  CK(cudaMemcpyAsync(x, in, n * 8, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(ri, rho_in, n * 8, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(ro, rho_out, n * 8, cudaMemcpyHostToDevice, c->stream));
  RC(proj_apply_dev(p, x, ri, ro, y, tmp, c->dscal));
  CK(cudaMemcpyAsync(out, y, n * 8, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return IMPS_OK;
}

int imps_dot(imps_ctx* c, const double* x, const double* y, int64_t n, double* result) {
  if (!c || !x || !y || !result) return IMPS_ERR_BAD_ARG;
  RC(kr_multidot(c->ws, x, n, 1, y, n, c->dscal, 0, nullptr, c->stream));
  CK(cudaMemcpyAsync(result, c->dscal, 8, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return IMPS_OK;
}

// ---- Lanczos: eigs_rs("SA") for the nev lowest eigenpairs of a symmetric operator ----
using DevApply = std::function<int(const double* in, double* out)>;

// p (optional): the plan whose precision the ladder may switch; op applies the operator on
// device vectors; x: start vector (mem), on return the normalised lowest Ritz vector;
// evecs (device, n x nev, optional): the nev Ritz vectors; evals (host, nev).
static int eigs_impl(imps_ctx* c, imps_plan* p, int64_t n, const DevApply& op, double* x, int mem, int nev,
                     double tol, int ncv, int maxit, double* evals, double* evecs, int* n_applies) {
  cudaStream_t st = c->stream;
  if (n < 2 || nev < 1 || nev > 16 || nev >= n) return IMPS_ERR_BAD_ARG;
  int m = ncv > 0 ? ncv : std::max(20, 2 * nev);  // eigs.cpp:4, 390: max(std_ncv, 2*nev) capped at N
  if (m > n) m = (int)n;
  if (m > kMaxCols - 2) m = kMaxCols - 2;
  if (m < nev + 3) m = (int)std::min<int64_t>(nev + 3, n);
  if (m < 2) m = 2;
  // maxit counts restart cycles, as ARPACK's IPARAM(3) (eigs.cpp:384, 399)
  if (maxit <= 0) maxit = (int)std::min<int64_t>(n, 100000);
  const int64_t max_applies = (int64_t)maxit * m;
  const int ld = m + 1;
  const int kk = std::max(nev, std::max(1, std::min(m / 2, m - 3)));  // Ritz vectors kept at a thick restart
  if (kk >= m) return IMPS_ERR_BAD_ARG;
  const bool cb_arena = p == nullptr;  // operator is a callback: keep clear of its solvers
  RC(arena_reserve(c, round256(n * 8) * (m + 4 + kk) + round256((size_t)ld * ld * 8) +
                          round256((size_t)m * kk * 8) + 4096, cb_arena));
  Bump bp{cb_arena ? c->arena_cb : c->arena};
  double* V = bp.take((size_t)n * (m + 1));
  double* Wk = bp.take((size_t)n * kk);
  double* w = bp.take(n);
  double* xr = bp.take(n);
  double* Hd = bp.take((size_t)ld * ld);
  double* Wrot = bp.take((size_t)m * kk);
  double* tmp = bp.take(ld);
  double* nrm = c->dscal + 8;
  int* bflag = c->dflag;
  if (mem == IMPS_MEM_HOST) CK(cudaMemcpyAsync(xr, x, n * 8, cudaMemcpyHostToDevice, st));
  else CK(cudaMemcpyAsync(xr, x, n * 8, cudaMemcpyDeviceToDevice, st));

  // The device keeps full CGS2 columns h = V^T A v_j; the host keeps the tridiagonal part
  // (alpha_j = h_j, beta_j = |w_j|), exact up to rounding because the basis is kept
  // orthonormal and a thick restart re-tridiagonalises the kept block (arrow_tridiag).
  std::vector<double> H((size_t)ld * ld, 0.0);
  std::vector<double> ta(m + 1, 0.0), tb(m + 1, 0.0), z(m, 0.0), thv(nev, 0.0), Zv((size_t)m * nev, 0.0);
  std::vector<double> th(kk), Z((size_t)m * kk), sv(kk), Q((size_t)kk * kk), qa(kk), qb(kk),
      Wr((size_t)m * kk);
  int applies = 0;
  double theta = 0.0, last_res = 0.0;
  const int chk = 4;
  // ARPACK's Ritz test (dsconv): |beta * y_k| <= tol * max(eps^(2/3), |theta|)
  const double eps23 = std::cbrt(kEps * kEps);

  // One thick-restart Lanczos run started from xr, at most `budget` applies; leaves the
  // (unnormalised) lowest Ritz vector in xr.  With stall_exit the run also ends (not
  // converged) once the Ritz residual has not halved over ~3 restart cycles: the floor of an
  // inexact operator.
  auto lanczos = [&](double tol_eff, int64_t budget, bool stall_exit) -> int {
    CK(cudaMemsetAsync(bflag, 0, sizeof(int), st));
    CK(cudaMemsetAsync(Hd, 0, (size_t)ld * ld * 8, st));
    RC(kr_multidot(c->ws, xr, n, 1, xr, n, tmp, 0, nrm, st));
    RC(kr_scale_inv(xr, nrm, V, n, bflag, st));
    int jstart = 0, jpulled = 0, status = IMPS_WARN_NOT_CONVERGED, kfinal = 0, pending = -1;
    int64_t used = 0, best_at = 0;
    double best = std::numeric_limits<double>::infinity();
    const int64_t stall_window = 3 * (int64_t)(m - kk) + m;
    bool done = false, pre_applied = false;
    int* pin_flags = (int*)(c->hpin + kPinDoubles);
    // queue the copies of columns jpulled..j and the flags into pinned memory, then an event
    auto stage = [&](int j) -> int {
      CK(cudaMemcpyAsync(c->hpin, Hd + (size_t)jpulled * ld, (size_t)(j + 1 - jpulled) * ld * 8,
                         cudaMemcpyDeviceToHost, st));
      CK(cudaMemcpyAsync(pin_flags, bflag, sizeof(int), cudaMemcpyDeviceToHost, st));
      CK(cudaMemcpyAsync(pin_flags + 1, c->ws.err, sizeof(int), cudaMemcpyDeviceToHost, st));
      CK(cudaEventRecord(c->ev_check, st));
      return IMPS_OK;
    };
    // convergence test of step j from the staged data: 1 = finished, 0 = go on, < 0 error
    auto evaluate = [&](int j) -> int {
      CK(cudaEventSynchronize(c->ev_check));
      if (pin_flags[1]) {  // a grid-barrier wait of the CGS2 step ran out: report, re-arm
        CK(cudaMemsetAsync(c->ws.err, 0, sizeof(int), st));
        return IMPS_ERR_TIMEOUT;
      }
      for (int q = jpulled; q <= j; ++q) {
        ta[q] = c->hpin[(size_t)(q - jpulled) * ld + q];
        tb[q] = c->hpin[(size_t)(q - jpulled) * ld + q + 1];
      }
      jpulled = j + 1;
      const int k = j + 1;
      const int nw = std::min(nev, k);
      tri_lowest_pairs(k, ta.data(), tb.data(), nw, thv.data(), Zv.data());
      theta = thv[0];
      if (!std::isfinite(theta)) return IMPS_ERR_NAN;
      std::copy(Zv.begin(), Zv.begin() + k, z.begin());
      // every wanted Ritz pair must pass the test (ARPACK counts nconv >= nev)
      double res = 0.0;
      bool all = nw == nev;
      for (int i = 0; i < nw; ++i) {
        const double ri = std::fabs(tb[k - 1] * Zv[(size_t)(k - 1) + (size_t)i * k]);
        res = std::max(res, i == 0 ? ri : 0.0);
        all = all && ri <= tol_eff * std::max(std::fabs(thv[i]), eps23);
      }
      last_res = res;
      kfinal = k;
      if (all || pin_flags[0]) {
        status = IMPS_OK;
        return 1;
      }
      if (used >= budget) return 1;
      if (res < 0.5 * best) {
        best = res;
        best_at = used;
      } else if (used - best_at > stall_window) {
        if (stall_exit) return 1;
        // A tolerance below what FP64 resolves for this operator: the Ritz residual cannot fall
        // below ~eps |H| (|H| bounded by the Gershgorin radius of T), where it only fluctuates.
        // Once it has stopped halving there, the solve ends converged to that accuracy.
        double normT = 0.0;
        for (int q = 0; q < k; ++q)
          normT = std::max(normT, std::fabs(ta[q]) + std::fabs(tb[q]) + (q ? std::fabs(tb[q - 1]) : 0.0));
        if (res <= kAttainableRes * kEps * normT) {
          status = IMPS_OK;
          return 1;
        }
      }
      return 0;
    };
    while (!done) {
      for (int j = jstart; j < m; ++j) {
        if (!(pre_applied && j == jstart)) RC(op(V + (size_t)j * n, w));
        pre_applied = false;
        ++applies;
        ++used;
        // the kept block is rotated at every restart so that the projected matrix stays
        // tridiagonal: w couples to v_j and v_{j-1} only, the first CGS pass takes those two
        RC(kr_cgs2_step(c->ws, V, n, j + 1, w, n, Hd + (size_t)j * ld, tmp, V + (size_t)(j + 1) * n, bflag, st,
                        2));
        if (pending >= 0) {  // the check of an earlier step, evaluated while step j runs
          const int r = evaluate(pending);
          pending = -1;
          if (r < 0) return r;
          if (r) { done = true; break; }
        }
        const bool last_step = j == m - 1 || used >= budget;
        if (!(((j + 1 - jstart) % chk == 0) || last_step)) continue;
        RC(stage(j));
        if (!last_step) { pending = j; continue; }
        // restart point: the first apply of the next cycle (on the residual direction v_m)
        // runs on the device while the host evaluates the check and computes the restart
        if (j == m - 1) {
          RC(op(V + (size_t)m * n, w));
          pre_applied = true;
        }
        const int r = evaluate(j);
        if (r < 0) return r;
        if (r) { done = true; break; }
      }
      if (done) break;
      // Thick restart (Wu & Simon): keep the kk lowest Ritz pairs of T_m and the residual
      // direction v_m.  The kept block is rotated so that T stays tridiagonal, with only its
      // last vector coupled to v_m (coupling |s|, s_i = beta_{m-1} * y_i[m-1]).
      tri_lowest_pairs(m, ta.data(), tb.data(), kk, th.data(), Z.data());
      for (int i = 0; i < kk; ++i) sv[i] = tb[m - 1] * Z[(size_t)(m - 1) + (size_t)i * m];
      arrow_tridiag(kk, th.data(), sv.data(), Q.data(), qa.data(), qb.data());
      double sn = 0.0;
      for (int i = 0; i < kk; ++i) sn += sv[i] * sv[i];
      sn = std::sqrt(sn);
      // new kept column p = Z * Q[:, kk-1-p], so that column kk-1 is the one coupled to v_m
      for (int pc = 0; pc < kk; ++pc) {
        const double* q = Q.data() + (size_t)(kk - 1 - pc) * kk;
        for (int r = 0; r < m; ++r) {
          double acc = 0.0;
          for (int i = 0; i < kk; ++i) acc += Z[(size_t)r + (size_t)i * m] * q[i];
          Wr[(size_t)r + (size_t)pc * m] = acc;
        }
      }
      std::copy(Wr.begin(), Wr.end(), c->hpin);  // pinned: the upload is asynchronous
      CK(cudaMemcpyAsync(Wrot, c->hpin, (size_t)m * kk * 8, cudaMemcpyHostToDevice, st));
      RC(kr_basis_rotate(V, n, m, Wrot, kk, Wk, n, n, st));
      CK(cudaMemcpyAsync(V, Wk, (size_t)kk * n * 8, cudaMemcpyDeviceToDevice, st));
      CK(cudaMemcpyAsync(V + (size_t)kk * n, V + (size_t)m * n, n * 8, cudaMemcpyDeviceToDevice, st));
      for (int pc = 0; pc < kk; ++pc) ta[pc] = qa[kk - 1 - pc];
      for (int pc = 0; pc + 1 < kk; ++pc) tb[pc] = qb[kk - 2 - pc];
      tb[kk - 1] = sn;
      jstart = jpulled = kk;
    }
    // the staging buffer is reused below: wait for the rotation upload to be consumed
    CK(cudaStreamSynchronize(st));
    // Ritz vectors: x = V[:, 0..k-1] z (lowest); all nev into evecs
    std::copy(z.begin(), z.begin() + kfinal, c->hpin);
    CK(cudaMemcpyAsync(tmp, c->hpin, kfinal * 8, cudaMemcpyHostToDevice, st));
    RC(kr_gemv(V, n, kfinal, tmp, xr, n, st));
    if (evecs && kfinal >= nev) {
      CK(cudaStreamSynchronize(st));
      std::copy(Zv.begin(), Zv.begin() + (size_t)kfinal * nev, c->hpin);
      CK(cudaMemcpyAsync(Wrot, c->hpin, (size_t)kfinal * nev * 8, cudaMemcpyHostToDevice, st));
      RC(kr_basis_rotate(V, n, kfinal, Wrot, nev, evecs, n, n, st));
    }
    CK(cudaStreamSynchronize(st));
    return status;
  };

  // Precision ladder.  Splitting operands into BF16 terms rounds, so the split-BF16 operator is
  // linear only to ~1e-7 |H| and its Lanczos residual floors there.  A tolerance at or above
  // that floor runs on the tensor cores (FP64 applies finish only if the mixed run stalls); a
  // tolerance below it runs in FP64 from the start — a mixed run followed by an FP64 run that
  // restarts from its Ritz vector costs more than the FP64 run alone.
  const int prec_saved = p ? p->prec : IMPS_PREC_FP64;
  const bool mixed = p && p->prec == IMPS_PREC_BF16X6 && tol >= kMixedEigTol;
  if (p) p->prec = mixed ? IMPS_PREC_BF16X6 : IMPS_PREC_FP64;
  int status = lanczos(tol, max_applies, mixed);
  const int applies_mixed = mixed ? applies : 0;
  if (status >= 0 && mixed && status != IMPS_OK && applies < max_applies) {
    p->prec = IMPS_PREC_FP64;
    status = lanczos(tol, std::max<int64_t>(max_applies - applies, m), false);
  }
  if (p) p->prec = prec_saved;
  if (status < 0) return status;
  // normalise
  RC(kr_multidot(c->ws, xr, n, 1, xr, n, tmp, 0, nrm, st));
  if (mem == IMPS_MEM_HOST) {
    RC(kr_scale_inv(xr, nrm, w, n, bflag, st));
    CK(cudaMemcpyAsync(x, w, n * 8, cudaMemcpyDeviceToHost, st));
  } else {
    RC(kr_scale_inv(xr, nrm, x, n, bflag, st));
  }
  CK(cudaStreamSynchronize(st));
  if (evals) {
    evals[0] = theta;
    for (int i = 1; i < nev; ++i) evals[i] = thv[i];
  }
  if (n_applies) *n_applies = applies;
  if (debug_on())
    fprintf(stderr,
            "[imps eigs_rs] n=%lld prec=%d applies=%d (split-bf16 %d) theta=%.15g res=%.3e tol=%.1e status=%d\n",
            (long long)n, prec_saved, applies, applies_mixed, theta, last_res, tol, status);
  return status;
}

int imps_eigs_rs(imps_plan* p, double* x, int mem, double tol, int ncv, int maxit, double* eval,
                 int* n_applies) {
  if (!p || !x || (p->P.kind != PLAN_HAC && p->P.kind != PLAN_HC)) return IMPS_ERR_BAD_ARG;
  const int64_t n = p->P.slots[p->P.n_in].nelem;
  DevApply op = [p](const double* in, double* out) { return apply_dev(p, in, out); };
  return eigs_impl(p->ctx, p, n, op, x, mem, 1, tol, ncv, maxit, eval, nullptr, n_applies);
}

int imps_eigs_rs_op(imps_ctx* c, int64_t n, imps_apply_fn fn, void* user, double* x, int mem, int nev, double tol,
                    int ncv, int maxit, double* evals, double* evecs, int* n_applies) {
  if (!c || !fn || !x || !evals) return IMPS_ERR_BAD_ARG;
  if (c->device < 0) return IMPS_ERR_NO_DEVICE;
  DevApply op = [fn, user](const double* in, double* out) {
    const int rc = fn(user, in, out);
    return rc < 0 ? rc : IMPS_OK;
  };
  return eigs_impl(c, nullptr, n, op, x, mem, nev, tol, ncv, maxit, evals, evecs, n_applies);
}

// ---- Lanczos over P independent symmetric systems in lockstep ----
// Every step applies the operator of all P systems at once (one callback on P x n vectors,
// system-major), then runs each system's CGS step on its own basis.  Per system: thick restart
// (Wu & Simon) with the kept block rotated to keep the projected matrix tridiagonal, ARPACK's
// Ritz test on the nev lowest pairs, and the attainable-accuracy exit of eigs_impl.  The systems
// restart together (they advance in lockstep); a converged system stops taking CGS steps (its
// slot of the batched apply is then unused).  Convergence is checked every 4 steps, synchronously.
int imps_eigs_rs_batch_op(imps_ctx* c, int P, int64_t n, imps_apply_fn fn, void* user, double* X, int nev,
                          double tol, int ncv, int maxit, double* evals, int* n_applies, int* converged) {
  if (!c || P < 1 || !fn || !X || !evals || n < 2 || nev < 1 || nev > 16 || nev >= n) return IMPS_ERR_BAD_ARG;
  if (c->device < 0) return IMPS_ERR_NO_DEVICE;
  cudaStream_t st = c->stream;
  int m = ncv > 0 ? ncv : std::max(20, 2 * nev);
  if (m > n) m = (int)n;
  if (m > kMaxCols - 2) m = kMaxCols - 2;
  if (m < nev + 3) m = (int)std::min<int64_t>(nev + 3, n);
  if (maxit <= 0) maxit = (int)std::min<int64_t>(n, 100000);
  const int64_t max_applies = (int64_t)maxit * m;
  const int ld = m + 1;
  const int kk = std::max(nev, std::max(1, std::min(m / 2, m - 3)));
  if (kk >= m) return IMPS_ERR_BAD_ARG;
  // the callback's own solves use the context's main arena: the bases live in the callback arena
  RC(arena_reserve(c, round256((size_t)P * n * 8) * (m + 1) + round256(n * 8) * (kk + 1) +
                          round256((size_t)P * n * 8) * 2 + round256((size_t)P * ld * ld * 8) +
                          round256((size_t)m * kk * 8) + round256(ld * 8) + 2 * round256((size_t)P * 8) +
                          round256((size_t)P * kMaxCols * 8) + round256((size_t)P * CGS_BATCH_GRID * kMaxCols * 8) +
                          4096, true));
  Bump bp{c->arena_cb};
  double* V = bp.take((size_t)P * n * (m + 1));  // system s: V + s * n * (m + 1), column j at + j * n
  double* Wk = bp.take((size_t)n * kk);
  double* IN = bp.take((size_t)P * n);
  double* OUT = bp.take((size_t)P * n);
  double* Hd = bp.take((size_t)P * ld * ld);
  double* Wrot = bp.take((size_t)m * kk);
  double* tmp = bp.take(ld);
  int* bflag = (int*)bp.take((P + 1) / 2 + 1);
  double* h2 = bp.take((size_t)P * kMaxCols);
  double* parts = bp.take((size_t)P * CGS_BATCH_GRID * kMaxCols);
  unsigned int* counters = (unsigned int*)bp.take((P + 1) / 2 + 1);
  double* nrm = c->dscal + 8;
  auto Vs = [&](int sy) { return V + (size_t)sy * n * (m + 1); };
  CK(cudaMemsetAsync(Hd, 0, (size_t)P * ld * ld * 8, st));
  CK(cudaMemsetAsync(bflag, 0, P * sizeof(int), st));
  CK(cudaMemsetAsync(counters, 0, P * sizeof(unsigned int), st));
  CK(cudaMemsetAsync(IN, 0, (size_t)P * n * 8, st));
  for (int sy = 0; sy < P; ++sy) {
    RC(kr_multidot(c->ws, X + (size_t)sy * n, n, 1, X + (size_t)sy * n, n, tmp, 0, nrm, st));
    RC(kr_scale_inv(X + (size_t)sy * n, nrm, Vs(sy), n, bflag + sy, st));
  }
  struct Sys {
    std::vector<double> ta, tb, z, thv, Zv;
    bool active = true, ok = false, final = false;
    int kfinal = 0, jpulled = 0;
    double best = std::numeric_limits<double>::infinity(), res = 0.0;
    int64_t best_at = 0;
  };
  std::vector<Sys> sys(P);
  for (Sys& q : sys) {
    q.ta.assign(m + 1, 0.0); q.tb.assign(m + 1, 0.0); q.z.assign(m, 0.0);
    q.thv.assign(nev, 0.0); q.Zv.assign((size_t)m * nev, 0.0);
  }
  std::vector<double> th(kk), Z((size_t)m * kk), sv(kk), Q((size_t)kk * kk), qa(kk), qb(kk), Wr((size_t)m * kk);
  std::vector<int> hflags(P);
  const double eps23 = std::cbrt(kEps * kEps);
  const int64_t stall_window = 3 * (int64_t)(m - kk) + m;
  int64_t applies = 0;
  int jstart = 0;
  const int chk = 4;
  auto n_active = [&]() { int a = 0; for (const Sys& q : sys) a += q.active; return a; };
  // convergence test of every active system at step j (columns jpulled..j come to the host)
  auto evaluate = [&](int j) -> int {
    CK(cudaMemcpyAsync(hflags.data(), bflag, P * sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    for (int sy = 0; sy < P; ++sy) {
      Sys& q = sys[sy];
      if (!q.active) continue;
      const int cols = j + 1 - q.jpulled;
      CK(cudaMemcpy(c->hpin, Hd + (size_t)sy * ld * ld + (size_t)q.jpulled * ld, (size_t)cols * ld * 8,
                    cudaMemcpyDeviceToHost));
      for (int r = q.jpulled; r <= j; ++r) {
        q.ta[r] = c->hpin[(size_t)(r - q.jpulled) * ld + r];
        q.tb[r] = c->hpin[(size_t)(r - q.jpulled) * ld + r + 1];
      }
      q.jpulled = j + 1;
      const int k = j + 1, nw = std::min(nev, k);
      tri_lowest_pairs(k, q.ta.data(), q.tb.data(), nw, q.thv.data(), q.Zv.data());
      if (!std::isfinite(q.thv[0])) return IMPS_ERR_NAN;
      std::copy(q.Zv.begin(), q.Zv.begin() + k, q.z.begin());
      q.kfinal = k;
      bool all = nw == nev;
      double res = 0.0;
      for (int i = 0; i < nw; ++i) {
        const double ri = std::fabs(q.tb[k - 1] * q.Zv[(size_t)(k - 1) + (size_t)i * k]);
        res = std::max(res, ri);
        all = all && ri <= tol * std::max(std::fabs(q.thv[i]), eps23);
      }
      q.res = res;
      if (all || hflags[sy]) { q.ok = true; q.active = false; continue; }
      if (res < 0.5 * q.best) {
        q.best = res;
        q.best_at = applies;
      } else if (applies - q.best_at > stall_window) {
        double normT = 0.0;
        for (int r = 0; r < k; ++r)
          normT = std::max(normT, std::fabs(q.ta[r]) + std::fabs(q.tb[r]) + (r ? std::fabs(q.tb[r - 1]) : 0.0));
        if (res <= kAttainableRes * kEps * normT) { q.ok = true; q.active = false; }
      }
    }
    return IMPS_OK;
  };
  // the lowest Ritz vector of system sy into X (normalised) and its Ritz values into evals; done
  // as soon as a system stops, because the batched CGS steps go on writing its unused columns
  auto finalize = [&](int sy) -> int {
    Sys& q = sys[sy];
    if (q.final) return IMPS_OK;
    q.final = true;
    for (int i = 0; i < nev; ++i) evals[(size_t)sy * nev + i] = i < q.kfinal ? q.thv[i] : 0.0;
    if (converged) converged[sy] = q.ok ? 1 : 0;
    if (q.kfinal < 1) return IMPS_OK;
    CK(cudaStreamSynchronize(st));
    CK(cudaMemcpy(tmp, q.z.data(), q.kfinal * 8, cudaMemcpyHostToDevice));
    RC(kr_gemv(Vs(sy), n, q.kfinal, tmp, X + (size_t)sy * n, n, st));
    RC(kr_multidot(c->ws, X + (size_t)sy * n, n, 1, X + (size_t)sy * n, n, tmp, 0, nrm, st));
    RC(kr_scale_inv(X + (size_t)sy * n, nrm, X + (size_t)sy * n, n, nullptr, st));
    CK(cudaStreamSynchronize(st));
    return IMPS_OK;
  };
  bool done = false;
  while (!done) {
    for (int j = jstart; j < m; ++j) {
      for (int sy = 0; sy < P; ++sy)
        if (sys[sy].active)
          CK(cudaMemcpyAsync(IN + (size_t)sy * n, Vs(sy) + (size_t)j * n, n * 8, cudaMemcpyDeviceToDevice, st));
      const int frc = fn(user, IN, OUT);
      if (frc < 0) return frc;
      ++applies;
      // every system's CGS step in one set of launches (converged systems work on their own
      // columns, which are no longer read)
      RC(kr_cgs2_step_batch(parts, counters, P, V, n * (m + 1), n, j + 1, OUT, n, n, Hd + (size_t)j * ld,
                            (int64_t)ld * ld, h2, V + (size_t)(j + 1) * n, bflag, st));
      const bool last = j == m - 1 || applies >= max_applies;
      if (((j + 1 - jstart) % chk == 0) || last) {
        RC(evaluate(j));
        for (int sy = 0; sy < P; ++sy)
          if (!sys[sy].active) RC(finalize(sy));
        if (n_active() == 0 || applies >= max_applies) { done = true; break; }
      }
    }
    if (done) break;
    // thick restart of every active system
    for (int sy = 0; sy < P; ++sy) {
      Sys& q = sys[sy];
      if (!q.active) continue;
      tri_lowest_pairs(m, q.ta.data(), q.tb.data(), kk, th.data(), Z.data());
      for (int i = 0; i < kk; ++i) sv[i] = q.tb[m - 1] * Z[(size_t)(m - 1) + (size_t)i * m];
      arrow_tridiag(kk, th.data(), sv.data(), Q.data(), qa.data(), qb.data());
      double sn = 0.0;
      for (int i = 0; i < kk; ++i) sn += sv[i] * sv[i];
      sn = std::sqrt(sn);
      for (int pc = 0; pc < kk; ++pc) {
        const double* qq = Q.data() + (size_t)(kk - 1 - pc) * kk;
        for (int r = 0; r < m; ++r) {
          double acc = 0.0;
          for (int i = 0; i < kk; ++i) acc += Z[(size_t)r + (size_t)i * m] * qq[i];
          Wr[(size_t)r + (size_t)pc * m] = acc;
        }
      }
      CK(cudaMemcpy(Wrot, Wr.data(), (size_t)m * kk * 8, cudaMemcpyHostToDevice));
      RC(kr_basis_rotate(Vs(sy), n, m, Wrot, kk, Wk, n, n, st));
      CK(cudaMemcpyAsync(Vs(sy), Wk, (size_t)kk * n * 8, cudaMemcpyDeviceToDevice, st));
      CK(cudaMemcpyAsync(Vs(sy) + (size_t)kk * n, Vs(sy) + (size_t)m * n, n * 8, cudaMemcpyDeviceToDevice, st));
      CK(cudaStreamSynchronize(st));  // Wrot and Wk are reused by the next system
      for (int pc = 0; pc < kk; ++pc) q.ta[pc] = qa[kk - 1 - pc];
      for (int pc = 0; pc + 1 < kk; ++pc) q.tb[pc] = qb[kk - 2 - pc];
      q.tb[kk - 1] = sn;
      q.jpulled = kk;
    }
    jstart = kk;
  }
  // systems still running at the apply limit: their current lowest Ritz vectors
  for (int sy = 0; sy < P; ++sy) RC(finalize(sy));
  if (n_applies) *n_applies = (int)applies;
  if (debug_on())
    fprintf(stderr, "[imps eigs_rs_batch] P=%d n=%lld applies=%lld converged=%d\n", P, (long long)n,
            (long long)applies, P - n_active());
  int allok = 1;
  for (const Sys& q : sys) allok &= q.ok;
  return allok ? IMPS_OK : IMPS_WARN_NOT_CONVERGED;
}

// ---- Arnoldi: eigs_n for the nev wanted eigenpairs of a real nonsymmetric operator ----
// Restart of Krylov-Schur type (Stewart, SIAM J. Matrix Anal. Appl. 23 (2001) 601): at the end
// of a cycle the kept Ritz vectors of the projected matrix G = V^T A V span an invariant
// subspace of G; with an orthonormal basis Q of it (real and imaginary parts of complex pairs)
// the kept basis is V Q, the kept block Q^T G Q and the coupling row h_m Q[m-1, :] to the
// residual direction v_m, which becomes the next basis vector.  The full CGS2 columns keep
// G = V^T A V exact up to rounding.  Convergence as ARPACK's dnconv (used by dnaupd):
// |h_m y[m-1]| <= tol max(eps^(2/3), |theta|) for each of the nev wanted Ritz pairs.
static int eign_impl(imps_ctx* c, imps_plan* p, int64_t n, const DevApply& op, const double* x0, int mem,
                     int nev, int which, double tol, int ncv, int maxit, double* evals, double* evecs_re,
                     double* evecs_im, int* n_applies) {
  cudaStream_t st = c->stream;
  if (n < 3 || nev < 1 || nev > 32 || nev > n - 2 || which < 0 || which > 2 || !evals) return IMPS_ERR_BAD_ARG;
  int m = ncv > 0 ? ncv : std::max(20, 2 * nev + 1);  // eigs.cpp: NCV = min(max(20, 2 NEV + 1), N)
  if (m > n) m = (int)n;
  if (m > kMaxCols - 2) m = kMaxCols - 2;
  if (m < nev + 2) return IMPS_ERR_BAD_ARG;  // dnaupd needs NCV - NEV >= 2
  if (maxit <= 0) maxit = (int)std::min<int64_t>(n, 100000);  // restart cycles (eigs.cpp: MAXIT = N)
  if (tol <= 0.0) tol = kEps;                                   // dnaupd: TOL <= 0 means machine precision
  const int ld = m + 1;
  const bool cb_arena = p == nullptr;
  RC(arena_reserve(c, round256(n * 8) * (2 * (size_t)m + 3) + round256((size_t)ld * ld * 8) +
                          round256((size_t)m * m * 8) + 4096, cb_arena));
  Bump bp{cb_arena ? c->arena_cb : c->arena};
  double* V = bp.take((size_t)n * (m + 1));
  double* Wk = bp.take((size_t)n * m);
  double* w = bp.take(n);
  double* Hd = bp.take((size_t)ld * ld);
  double* Qd = bp.take((size_t)m * m);
  double* tmp = bp.take(ld);
  double* nrm = c->dscal + 8;
  int* bflag = c->dflag;
  int* pin_flags = (int*)(c->hpin + kPinDoubles);
  // the operator runs in FP64 unless the tolerance is above the split-BF16 floor
  const int prec_saved = p ? p->prec : IMPS_PREC_FP64;
  if (p && tol < kMixedEigTol) p->prec = IMPS_PREC_FP64;
  struct Restore {
    imps_plan* p;
    int prec;
    ~Restore() { if (p) p->prec = prec; }
  } restore{p, prec_saved};

  if (x0) {
    CK(cudaMemcpyAsync(w, x0, n * 8, mem == IMPS_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, st));
  } else {
    RC(kr_fill_random(w, n, 0x5EED0F1A4D0C0DEull, st));  // dnaupd starts from a random vector
  }
  CK(cudaMemsetAsync(bflag, 0, sizeof(int), st));
  RC(kr_multidot(c->ws, w, n, 1, w, n, tmp, 0, nrm, st));
  RC(kr_scale_inv(w, nrm, V, n, bflag, st));

  std::vector<double> G((size_t)m * m, 0.0), Gs((size_t)m * m), wr(m), wi(m), Qh((size_t)m * m), B((size_t)m * m);
  std::vector<imps::cplx> Y((size_t)m * m);  // Ritz vectors of G, column i for order[i]
  std::vector<int> order;
  const double eps23 = std::cbrt(kEps * kEps);
  int kept = 0, applies = 0, cycles = 0, status = IMPS_WARN_NOT_CONVERGED, k = m;
  double hm = 0.0, worst = 0.0;
  while (true) {
    for (int j = kept; j < m; ++j) {
      RC(op(V + (size_t)j * n, w));
      ++applies;
      RC(kr_cgs2_step(c->ws, V, n, j + 1, w, n, Hd + (size_t)j * ld, tmp, V + (size_t)(j + 1) * n, bflag, st));
    }
    ++cycles;
    CK(cudaMemcpyAsync(c->hpin, Hd + (size_t)kept * ld, (size_t)(m - kept) * ld * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(pin_flags + 1, c->ws.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (pin_flags[1]) {  // a grid-barrier wait of the CGS2 step ran out: report, re-arm
      CK(cudaMemsetAsync(c->ws.err, 0, sizeof(int), st));
      return IMPS_ERR_TIMEOUT;
    }
    double gscale = 0.0;
    for (int j = kept; j < m; ++j) {
      const double* hc = c->hpin + (size_t)(j - kept) * ld;
      for (int i = 0; i < m; ++i) G[i + (size_t)j * m] = i <= j + 1 && i < m ? hc[i] : 0.0;
    }
    hm = c->hpin[(size_t)(m - 1 - kept) * ld + m];
    for (double g : G) {
      if (!std::isfinite(g)) return IMPS_ERR_NAN;
      gscale = std::max(gscale, std::fabs(g));
    }
    if (!std::isfinite(hm)) return IMPS_ERR_NAN;
    // breakdown: an exactly invariant Krylov subspace of size k < m (later columns are void)
    k = m;
    for (int j = kept; j + 1 < m; ++j)
      if (!(std::fabs(G[j + 1 + (size_t)j * m]) > 1e-14 * gscale)) {
        k = j + 1;
        break;
      }
    if (k < m) hm = 0.0;
    for (int j = 0; j < k; ++j)
      for (int i = 0; i < k; ++i) Gs[i + (size_t)j * k] = G[i + (size_t)j * m];
    if (!imps::dense_eigvals(k, Gs.data(), wr.data(), wi.data())) return IMPS_ERR_NAN;
    order = imps::order_ritz(k, wr.data(), wi.data(), which);
    // kept set (real dimension), never splitting a conjugate pair
    const int target = std::min(k, std::max(nev + 1, std::min(m - 2, nev + (m - nev) / 2)));
    int nk = 0, nsel = 0;  // real dimension kept, Ritz values selected
    while (nsel < k && nk < target) {
      const int i = order[nsel];
      nk += wi[i] != 0.0 ? 2 : 1;
      nsel += wi[i] != 0.0 ? 2 : 1;
    }
    nsel = std::max(nsel, std::min(k, nev + (wi[order[std::min(nev, k) - 1]] > 0.0 ? 1 : 0)));
    for (int s = 0; s < nsel; ++s) {
      const int i = order[s];
      imps::cplx* y = Y.data() + (size_t)s * m;
      if (wi[i] < 0.0 && s > 0 && order[s - 1] >= 0 && wi[order[s - 1]] == -wi[i] && wr[order[s - 1]] == wr[i]) {
        for (int r = 0; r < k; ++r) y[r] = std::conj(Y[(size_t)(s - 1) * m + r]);
      } else {
        imps::dense_eigvec(k, Gs.data(), gscale * k, imps::cplx(wr[i], wi[i]), y);
      }
    }
    // convergence of the nev wanted pairs
    int nconv = 0;
    worst = 0.0;
    for (int s = 0; s < std::min(nev, k); ++s) {
      const int i = order[s];
      const double res = std::fabs(hm) * std::abs(Y[(size_t)s * m + (k - 1)]);
      worst = std::max(worst, res);
      if (res <= tol * std::max(eps23, std::hypot(wr[i], wi[i]))) ++nconv;
    }
    if (nconv >= nev && k >= nev) {
      status = IMPS_OK;
      break;
    }
    if (k < m || cycles >= maxit) break;
    // restart: orthonormal real basis of the kept invariant subspace (two MGS passes)
    int q = 0;
    for (int s = 0; s < nsel && q < m - 1; ++s) {
      const int i = order[s];
      if (wi[i] < 0.0) continue;  // the conjugate partner adds nothing new
      for (int part = 0; part < (wi[i] > 0.0 ? 2 : 1); ++part) {
        double* col = Qh.data() + (size_t)q * m;
        for (int r = 0; r < k; ++r) col[r] = part ? Y[(size_t)s * m + r].imag() : Y[(size_t)s * m + r].real();
        double n0 = 0.0;
        for (int r = 0; r < k; ++r) n0 += col[r] * col[r];
        n0 = std::sqrt(n0);
        for (int pass = 0; pass < 2; ++pass)
          for (int t = 0; t < q; ++t) {
            const double* qt = Qh.data() + (size_t)t * m;
            double d = 0.0;
            for (int r = 0; r < k; ++r) d += qt[r] * col[r];
            for (int r = 0; r < k; ++r) col[r] -= d * qt[r];
          }
        double n1 = 0.0;
        for (int r = 0; r < k; ++r) n1 += col[r] * col[r];
        n1 = std::sqrt(n1);
        if (!(n1 > 1e-8 * n0)) continue;  // dependent (a defective cluster): drop
        for (int r = 0; r < k; ++r) col[r] /= n1;
        ++q;
        if (q >= m - 1) break;
      }
    }
    if (q < 1) break;
    // kept block B = Q^T G Q and coupling row g = h_m Q[m-1, :]
    for (int b = 0; b < q; ++b) {
      std::vector<double> gq(k, 0.0);
      const double* qb = Qh.data() + (size_t)b * m;
      for (int j = 0; j < k; ++j)
        for (int i = 0; i < k; ++i) gq[i] += G[i + (size_t)j * m] * qb[j];
      for (int a = 0; a < q; ++a) {
        const double* qa = Qh.data() + (size_t)a * m;
        double acc = 0.0;
        for (int i = 0; i < k; ++i) acc += qa[i] * gq[i];
        B[a + (size_t)b * q] = acc;
      }
    }
    for (int b = 0; b < q; ++b)
      for (int r = 0; r < k; ++r) c->hpin[r + (size_t)b * k] = Qh[r + (size_t)b * m];
    CK(cudaMemcpyAsync(Qd, c->hpin, (size_t)k * q * 8, cudaMemcpyHostToDevice, st));
    RC(kr_basis_rotate(V, n, k, Qd, q, Wk, n, n, st));
    CK(cudaMemcpyAsync(V, Wk, (size_t)q * n * 8, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(V + (size_t)q * n, V + (size_t)m * n, n * 8, cudaMemcpyDeviceToDevice, st));
    std::fill(G.begin(), G.end(), 0.0);
    for (int b = 0; b < q; ++b) {
      for (int a = 0; a < q; ++a) G[a + (size_t)b * m] = B[a + (size_t)b * q];
      G[q + (size_t)b * m] = hm * Qh[(size_t)(k - 1) + (size_t)b * m];
    }
    kept = q;
  }
  // the staging buffer is reused below: wait for any rotation upload to be consumed
  CK(cudaStreamSynchronize(st));
  const int nout = std::min(nev, k);
  for (int s = 0; s < nev; ++s) {
    evals[2 * s] = s < nout ? wr[order[s]] : std::numeric_limits<double>::quiet_NaN();
    evals[2 * s + 1] = s < nout ? wi[order[s]] : std::numeric_limits<double>::quiet_NaN();
  }
  if (evecs_re && nout > 0) {
    for (int part = 0; part < 2; ++part) {
      double* dst = part ? evecs_im : evecs_re;
      if (!dst) continue;
      for (int s = 0; s < nout; ++s)
        for (int r = 0; r < k; ++r) {
          const imps::cplx y = Y[(size_t)s * m + r];
          c->hpin[r + (size_t)s * k] = part ? y.imag() : y.real();
        }
      CK(cudaMemcpyAsync(Qd, c->hpin, (size_t)k * nout * 8, cudaMemcpyHostToDevice, st));
      if (mem == IMPS_MEM_HOST) {
        RC(kr_basis_rotate(V, n, k, Qd, nout, Wk, n, n, st));
        CK(cudaMemcpyAsync(dst, Wk, (size_t)nout * n * 8, cudaMemcpyDeviceToHost, st));
      } else {
        RC(kr_basis_rotate(V, n, k, Qd, nout, dst, n, n, st));
      }
      CK(cudaStreamSynchronize(st));
    }
  }
  if (n_applies) *n_applies = applies;
  if (debug_on())
    fprintf(stderr, "[imps eigs_n] n=%lld which=%d nev=%d ncv=%d applies=%d cycles=%d theta0=%.15g%+.3gi res=%.3e status=%d\n",
            (long long)n, which, nev, m, applies, cycles, evals[0], evals[1], worst, status);
  return status;
}

int imps_eigs_n(imps_plan* p, const double* x0, int mem, int nev, int which, double tol, int ncv, int maxit,
                double* evals, double* evecs_re, double* evecs_im, int* n_applies) {
  if (!p || !evals) return IMPS_ERR_BAD_ARG;
  const int kd = p->P.kind;
  if (kd != PLAN_TM && !is_mixed_tm(p) && kd != PLAN_HAC && kd != PLAN_HC) return IMPS_ERR_BAD_ARG;
  if (p->ctx->device < 0) return IMPS_ERR_NO_DEVICE;
  const int64_t n = p->P.slots[p->P.n_in].nelem;
  if (p->P.slots[p->P.n_out].nelem != n) return IMPS_ERR_BAD_ARG;
  DevApply op = [p](const double* in, double* out) { return apply_dev(p, in, out); };
  return eign_impl(p->ctx, p, n, op, x0, mem, nev, which, tol, ncv, maxit, evals, evecs_re, evecs_im, n_applies);
}

int imps_eigs_n_op(imps_ctx* c, int64_t n, imps_apply_fn fn, void* user, const double* x0, int mem, int nev,
                   int which, double tol, int ncv, int maxit, double* evals, double* evecs_re, double* evecs_im,
                   int* n_applies) {
  if (!c || !fn || !evals) return IMPS_ERR_BAD_ARG;
  if (c->device < 0) return IMPS_ERR_NO_DEVICE;
  DevApply op = [fn, user](const double* in, double* out) {
    const int rc = fn(user, in, out);
    return rc < 0 ? rc : IMPS_OK;
  };
  return eign_impl(c, nullptr, n, op, x0, mem, nev, which, tol, ncv, maxit, evals, evecs_re, evecs_im, n_applies);
}

// ---- device GMRES (generic operator) ----
// Operator of a device GMRES: out = A(in) on device vectors; `fp64` asks for the FP64 engine
// (the residual of a mixed-precision solve), otherwise the operator's own precision.
using DevOp = std::function<int(const double* in, double* out, bool fp64)>;

// Restarted GMRES(krylov) on the device for A y = b (y holds y0 on entry): CGS2 Arnoldi,
// Givens rotations on the device, the residual recomputed (in FP64) at every restart.
static int gmres_dev(imps_ctx* c, int64_t n, const DevOp& A, bool mixed, const double* b, double* y,
                     double tol, int maxit, int krylov, int* iters, double* relres, Bump& bp) {
  cudaStream_t st = c->stream;
  int m = krylov > 0 ? krylov : kGmresKrylov;
  if (m > kMaxCols - 2) m = kMaxCols - 2;
  if (m > n) m = (int)n;
  const int ld = m + 1;
  double* V = bp.take((size_t)n * (m + 1));
  double* w = bp.take(n);
  double* t = bp.take(n);
  double* Hd = bp.take((size_t)ld * m);  // Hessenberg columns (CGS2 projections), column j at j*ld
  double* tmp = bp.take(ld);
  double* ys = bp.take(ld);
  double* dsc = c->dscal;  // 0: trace, 1: |r|, 2: |b|
  int* bflag = c->dflag + 1;
  int* pin_flags = (int*)(c->hpin_g + kPinDoubles);
  // |b|
  RC(kr_multidot(c->ws, b, n, 1, b, n, tmp, 0, dsc + 2, st));
  double bnorm = 0.0;
  CK(cudaMemcpyAsync(&bnorm, dsc + 2, 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (!std::isfinite(bnorm)) return IMPS_ERR_NAN;
  int it = 0;
  double rel = 0.0;
  int status = IMPS_WARN_NOT_CONVERGED;
  if (bnorm == 0.0) {
    CK(cudaMemsetAsync(y, 0, n * 8, st));
    if (iters) *iters = 0;
    if (relres) *relres = 0.0;
    return IMPS_OK;
  }
  // Givens rotations of the Hessenberg columns (IterativeSolvers.hpp:79-85, 103-115), on the
  // host at the residual checks: the columns of the steps since the last check arrive in one
  // copy, so the device runs no serial rotation kernel per iteration
  std::vector<double> Rh((size_t)ld * ld), gh(ld), yh(ld), csh(ld), snh(ld), col(ld + 1);
  // Mixed precision: every restart recomputes the true residual with the FP64 engine and the
  // inner Krylov cycle (split-BF16 applies) only has to reduce it by kMixedInnerTol, i.e.
  // restarted GMRES acts as iterative refinement with FP64 residuals.
  int stall = 0;
  double rn_prev = 0.0;
  bool inner_hit = false;  // the last cycle ended on its Krylov residual estimate
  for (int outer = 0; it < maxit; ++outer) {
    // r = b - A(y)  (FP64 residual)
    RC(A(y, w, true));
    RC(kr_axpby(1.0, b, -1.0, w, n, st));
    RC(kr_multidot(c->ws, w, n, 1, w, n, tmp, 0, dsc + 1, st));
    double rn = 0.0;
    CK(cudaMemcpyAsync(&rn, dsc + 1, 8, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (!std::isfinite(rn)) return IMPS_ERR_NAN;
    rel = rn / bnorm;
    if (debug_level() > 1)
      fprintf(stderr, "[imps gmres]   outer=%d it=%d relres=%.3e\n", outer, it, rel);
    if (rn < tol * bnorm) { status = IMPS_OK; break; }
    // At the attainable accuracy (~eps * |A| |y| / |b|) the Krylov estimate of a cycle reaches
    // its target while the recomputed residual stops falling.  Three such cycles in a row that
    // gain < 10% each end the solve (not converged, result returned) instead of running into
    // maxit; cycles that used their whole Krylov space (slow but steady) never count.
    stall = outer > 0 && inner_hit && rn > 0.9 * rn_prev ? stall + 1 : 0;
    rn_prev = rn;
    if (stall >= 3) break;
    inner_hit = false;
    CK(cudaMemsetAsync(bflag, 0, sizeof(int), st));
    RC(kr_scale_inv(w, dsc + 1, V, n, bflag, st));
    std::fill(gh.begin(), gh.end(), 0.0);
    gh[0] = rn;
    int kdim = 0, jpulled = 0;
    for (int j = 0; j < m && it < maxit; ++j) {
      double* vj = V + (size_t)j * n;
      RC(A(vj, w, false));
      ++it;
      RC(kr_cgs2_step(c->ws, V, n, j + 1, w, n, Hd + (size_t)j * ld, tmp, V + (size_t)(j + 1) * n, nullptr, st));
      kdim = j + 1;
      if ((j + 1) % 4 == 0 || j == m - 1 || it >= maxit) {
        CK(cudaMemcpyAsync(c->hpin_g, Hd + (size_t)jpulled * ld, (size_t)(j + 1 - jpulled) * ld * 8,
                           cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(pin_flags, c->ws.err, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (pin_flags[0]) {  // a grid-barrier wait of the CGS2 step ran out: report, re-arm
          CK(cudaMemsetAsync(c->ws.err, 0, sizeof(int), st));
          return IMPS_ERR_TIMEOUT;
        }
        double res = 0.0;
        bool brk = false;
        for (int q = jpulled; q <= j; ++q) {
          const double* hc = c->hpin_g + (size_t)(q - jpulled) * ld;
          for (int i = 0; i <= q + 1; ++i) col[i] = hc[i];
          for (int i = 0; i < q; ++i) {
            const double h1 = col[i], h2 = col[i + 1];
            col[i] = csh[i] * h1 + snh[i] * h2;
            col[i + 1] = -snh[i] * h1 + csh[i] * h2;
          }
          const double hqq = col[q], hq1 = col[q + 1];
          const double beta = std::sqrt(hqq * hqq + hq1 * hq1);
          if (!std::isfinite(beta)) return IMPS_ERR_NAN;
          if (!(beta >= 2e-16)) {  // flag -2 of the reference: column q adds nothing
            brk = true;
            kdim = q;
            break;
          }
          const double habs = std::fabs(hqq);
          const double phase = habs > 0.0 ? hqq / habs : 1.0;
          snh[q] = phase * hq1 / beta;
          csh[q] = habs / beta;
          col[q] = phase * beta;
          gh[q + 1] = -snh[q] * gh[q];
          gh[q] *= csh[q];
          for (int i = 0; i <= q; ++i) Rh[i + (size_t)q * ld] = col[i];
          res = std::fabs(gh[q + 1]);
        }
        jpulled = j + 1;
        if (brk) break;  // invariant subspace
        if (res < std::max(tol * bnorm, mixed ? kMixedInnerTol * rn : 0.0)) {
          inner_hit = true;
          break;
        }
      }
    }
    // y += V[:, :kdim] * R^{-1} gamma (R and gamma are on the host; checks pulled every column
    // up to kdim, since a cycle ends only at a check)
    if (kdim > 0) {
      for (int i = kdim - 1; i >= 0; --i) {
        double s = gh[i];
        for (int q = i + 1; q < kdim; ++q) s -= Rh[i + (size_t)q * ld] * yh[q];
        yh[i] = s / Rh[i + (size_t)i * ld];
      }
      CK(cudaMemcpyAsync(ys, yh.data(), kdim * 8, cudaMemcpyHostToDevice, st));
      RC(kr_gemv(V, n, kdim, ys, t, n, st));
      RC(kr_axpby(1.0, t, 1.0, y, n, st));
    }
  }
  if (status != IMPS_OK) {
    // final explicit residual (FP64)
    RC(A(y, w, true));
    RC(kr_axpby(1.0, b, -1.0, w, n, st));
    RC(kr_multidot(c->ws, w, n, 1, w, n, tmp, 0, dsc + 1, st));
    double rn = 0.0;
    CK(cudaMemcpyAsync(&rn, dsc + 1, 8, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    rel = rn / bnorm;
    if (rn < tol * bnorm) status = IMPS_OK;
  }
  if (iters) *iters = it;
  if (debug_on())
    fprintf(stderr, "[imps gmres] n=%lld mixed=%d iters=%d relres=%.3e tol=%.1e status=%d\n", (long long)n,
            (int)mixed, it, rel, tol, status);
  if (relres) *relres = rel;
  return status;
}

// GMRES on the projected operator A(v) = v - T(v) + tr(v*rho_in)*rho_out of a TM plan
static int gmres_proj(imps_plan* p, const double* b, double* y, const double* rho_in,
                      const double* rho_out, double tol, int maxit, int krylov, int* iters,
                      double* relres, Bump& bp) {
  imps_ctx* c = p->ctx;
  const int64_t n = p->P.slots[0].nelem;
  double* t = bp.take(n);
  const int prec_saved = p->prec;
  DevOp A = [&](const double* in, double* out, bool fp64) -> int {
    if (fp64) p->prec = IMPS_PREC_FP64;
    const int rc = proj_apply_dev(p, in, rho_in, rho_out, out, t, c->dscal);
    p->prec = prec_saved;
    return rc;
  };
  return gmres_dev(c, n, A, prec_saved == IMPS_PREC_BF16X6, b, y, tol, maxit, krylov, iters, relres, bp);
}

int imps_invert_e_proj(imps_plan* p, const double* x, const double* L, const double* R, int dir,
                       double* y, int mem, double tol, int maxit, int krylov, int* iters, double* relres) {
  if (!p || p->P.kind != PLAN_TM || !x || !L || !R || !y || (dir != 0 && dir != 1)) return IMPS_ERR_BAD_ARG;
  imps_ctx* c = p->ctx;
  cudaStream_t st = c->stream;
  const int64_t n = p->P.slots[0].nelem;
  if (p->P.slots[1].nelem != n) return IMPS_ERR_BAD_ARG;
  int m = krylov > 0 ? std::min(krylov, kMaxCols - 2) : kGmresKrylov;
  if (maxit <= 0) maxit = (int)std::min<int64_t>(n, 100000);
  RC(arena_reserve(c, round256(n * 8) * (m + 12) + round256((size_t)(m + 1) * (m + 1) * 8) + 16 * 4096));
  Bump bp{c->arena};
  double *dx = (double*)x, *dL = (double*)L, *dR = (double*)R, *dy = y;
  if (mem == IMPS_MEM_HOST) {
    dx = bp.take(n); dL = bp.take(n); dR = bp.take(n); dy = bp.take(n);
    CK(cudaMemcpyAsync(dx, x, n * 8, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dL, L, n * 8, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dR, R, n * 8, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dy, y, n * 8, cudaMemcpyHostToDevice, st));
  }
  // rho_in / rho_out: dir l -> (R, L), dir r -> (L, R)  (InvEBlockFunctions.hpp:239-257)
  const double* rin = dir == 0 ? dR : dL;
  const double* rout = dir == 0 ? dL : dR;
  // b = x - tr(x*rho_in) * rho_out
  double* b = bp.take(n);
  RC(kr_trace_prod(c->ws, dx, rin, p->d_boff, p->d_bdim, p->nb_in, c->dscal + 4, st));
  CK(cudaMemsetAsync(b, 0, n * 8, st));
  RC(kr_proj_epilogue(dx, b, c->dscal + 4, rout, b, n, st));  // b = x + s*rho_out - 0
  // flip sign of the projector part: b = x - s*rho_out  ->  compute b2 = 2x - b
  RC(kr_axpby(2.0, dx, -1.0, b, n, st));
  int rc = gmres_proj(p, b, dy, rin, rout, tol, maxit, m, iters, relres, bp);
  if (rc < 0) return rc;
  if (mem == IMPS_MEM_HOST) {
    CK(cudaMemcpyAsync(y, dy, n * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
  }
  return rc;
}

__global__ void imps_set_identity_kernel(double* X, const int64_t* boff, const int32_t* bdim, int nb) {
  const int b = blockIdx.x;
  if (b >= nb) return;
  const int m = bdim[b];
  double* x = X + boff[b];
  for (int64_t e = threadIdx.x; e < (int64_t)m * m; e += blockDim.x) x[e] = (e % (m + 1) == 0) ? 1.0 : 0.0;
}

// ---- InvertE_fac / InvertE_proj_fac on split complex planes ----
// Solves (1 - fac T) y = x (InvEBlockFunctions.hpp:413-451 with InvEfun_fac :166-197) or,
// with rho, the projected (1 - fac T + |rho_out)(rho_in|) y = x - tr(x rho_in) rho_out
// (:277-330 with InvEfun_proj_fac :90-125).  x, y complex as separate real and imaginary
// planes; T is the real mixed transfer matrix of the plan, so the complex system is the real
// system on the stacked vector [re; im] and the device GMRES solves it in FP64.
static int invert_fac_impl(imps_plan* p, const double* xre, const double* xim, const double* L,
                           const double* R, int dir, bool proj, double fre, double fim, double* yre,
                           double* yim, int mem, double tol, int maxit, int krylov, int* iters, double* relres) {
  if (!is_mixed_tm(p) || !xre || !xim || !yre || !yim || (proj && (!L || !R))) return IMPS_ERR_BAD_ARG;
  imps_ctx* c = p->ctx;
  if (c->device < 0) return IMPS_ERR_NO_DEVICE;
  cudaStream_t st = c->stream;
  const int64_t n = p->P.slots[p->P.n_in].nelem;
  if (p->P.slots[p->P.n_out].nelem != n) return IMPS_ERR_BAD_ARG;
  int m = krylov > 0 ? std::min(krylov, kMaxCols - 2) : kGmresKrylov;
  if (maxit <= 0) maxit = (int)std::min<int64_t>(2 * n, 100000);
  RC(arena_reserve(c, round256(2 * n * 8) * (m + 12) + round256((size_t)(m + 1) * (m + 1) * 8) + 16 * 4096));
  Bump bp{c->arena};
  double* x = bp.take(2 * n);
  double* y = bp.take(2 * n);
  double* t = bp.take(2 * n);
  double* b = bp.take(2 * n);
  double *dL = nullptr, *dR = nullptr;
  const cudaMemcpyKind k_in = mem == IMPS_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  CK(cudaMemcpyAsync(x, xre, n * 8, k_in, st));
  CK(cudaMemcpyAsync(x + n, xim, n * 8, k_in, st));
  CK(cudaMemcpyAsync(y, yre, n * 8, k_in, st));
  CK(cudaMemcpyAsync(y + n, yim, n * 8, k_in, st));
  if (proj) {
    dL = bp.take(n);
    dR = bp.take(n);
    CK(cudaMemcpyAsync(dL, L, n * 8, k_in, st));
    CK(cudaMemcpyAsync(dR, R, n * 8, k_in, st));
  }
  // rho_in / rho_out: dir l -> (R, L), dir r -> (L, R) (InvEBlockFunctions.hpp:313-328)
  const double* rin = proj ? (dir == 0 ? dR : dL) : nullptr;
  const double* rout = proj ? (dir == 0 ? dL : dR) : nullptr;
  double* tau = c->dscal + 16;  // (re, im) of tr(v rho_in)
  auto traces = [&](const double* v) -> int {
    RC(kr_trace_prod(c->ws, v, rin, p->d_boff, p->d_bdim, p->nb_in, tau, st, p->d_bcols));
    RC(kr_trace_prod(c->ws, v + n, rin, p->d_boff, p->d_bdim, p->nb_in, tau + 1, st, p->d_bcols));
    return IMPS_OK;
  };
  // b = x - tr(x rho_in) rho_out  (x unchanged without projection)
  if (proj) {
    RC(traces(x));
    CK(cudaMemsetAsync(t, 0, 2 * n * 8, st));
    // b = x - 0 + tau rho_out, then flip the projector's sign: b = 2x - b
    RC(kr_fac_epilogue(x, x + n, t, t + n, 0.0, 0.0, tau, rout, b, b + n, n, st));
    RC(kr_axpby(2.0, x, -1.0, b, 2 * n, st));
  } else {
    CK(cudaMemcpyAsync(b, x, 2 * n * 8, cudaMemcpyDeviceToDevice, st));
  }
  DevOp A = [&](const double* u, double* out, bool) -> int {
    RC(apply_dev(p, u, t));
    RC(apply_dev(p, u + n, t + n));
    if (proj) RC(traces(u));
    return kr_fac_epilogue(u, u + n, t, t + n, fre, fim, proj ? tau : nullptr, rout, out, out + n, n, st);
  };
  const int prec_saved = p->prec;
  p->prec = IMPS_PREC_FP64;
  int rc = gmres_dev(c, 2 * n, A, false, b, y, tol, maxit, m, iters, relres, bp);
  p->prec = prec_saved;
  if (rc < 0) return rc;
  const cudaMemcpyKind k_out = mem == IMPS_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  CK(cudaMemcpyAsync(yre, y, n * 8, k_out, st));
  CK(cudaMemcpyAsync(yim, y + n, n * 8, k_out, st));
  CK(cudaStreamSynchronize(st));
  return rc;
}

int imps_invert_e_fac(imps_plan* p, const double* x_re, const double* x_im, double fac_re, double fac_im,
                      double* y_re, double* y_im, int mem, double tol, int maxit, int krylov, int* iters,
                      double* relres) {
  return invert_fac_impl(p, x_re, x_im, nullptr, nullptr, 0, false, fac_re, fac_im, y_re, y_im, mem, tol,
                         maxit, krylov, iters, relres);
}

int imps_invert_e_proj_fac(imps_plan* p, const double* x_re, const double* x_im, const double* L,
                           const double* R, int dir, double fac_re, double fac_im, double* y_re, double* y_im,
                           int mem, double tol, int maxit, int krylov, int* iters, double* relres) {
  if ((dir != 0 && dir != 1) || !is_mixed_tm(p) || dir != (p->P.kind == PLAN_TMMIXED_L ? 0 : 1))
    return IMPS_ERR_BAD_ARG;  // the plan's direction and the projector's roles must agree
  return invert_fac_impl(p, x_re, x_im, L, R, dir, true, fac_re, fac_im, y_re, y_im, mem, tol, maxit, krylov,
                         iters, relres);
}

// Restarted GMRES on P independent systems in lockstep.  Every iteration applies the operators
// of all systems at once (Ab: stacked input -> stacked output, system s at s * n), then runs each
// system's CGS step on its own Krylov basis; the Givens rotations of every system run on the
// host at the checks (every 4 iterations), as in gmres_dev.  A system whose cycle met its
// tolerance stops extending its basis while the others go on; every system restarts from its
// recomputed residual.  Returns the largest iteration count and relative residual.
using BatchOp = std::function<int(const double* in, double* out)>;
static int gmres_batch(imps_ctx* c, int P, int64_t n, const BatchOp& Ab, const double* b, double* y, double tol,
                       int maxit, int krylov, int* iters, double* relres, Bump& bp) {
  cudaStream_t st = c->stream;
  int m = krylov > 0 ? krylov : kGmresKrylov;
  if (m > kMaxCols - 2) m = kMaxCols - 2;
  if (m > n) m = (int)n;
  const int ld = m + 1;
  const int64_t ntot = (int64_t)P * n;
  double* V = bp.take((size_t)ntot * (m + 1));  // system s: V + s * n * (m + 1)
  double* U = bp.take(ntot);
  double* W = bp.take(ntot);
  double* Tm = bp.take(n);
  double* Hd = bp.take((size_t)P * ld * m);
  double* tmp = bp.take(ld);
  double* ys = bp.take(ld);
  double* nrm = bp.take(P);
  double* h2 = bp.take((size_t)P * kMaxCols);
  double* parts = bp.take((size_t)P * CGS_BATCH_GRID * kMaxCols);
  unsigned int* counters = (unsigned int*)bp.take((P + 1) / 2 + 1);
  CK(cudaMemsetAsync(counters, 0, P * sizeof(unsigned int), st));
  CK(cudaMemsetAsync(U, 0, ntot * 8, st));
  auto Vs = [&](int sy) { return V + (size_t)sy * n * (m + 1); };
  struct Sys {
    std::vector<double> Rh, gh, yh, csh, snh;
    double bnorm = 0.0, rn = 0.0, rn_prev = 0.0;
    int stall = 0, kdim = 0, jpulled = 0, it = 0;
    bool done = false, in_cycle = false, inner_hit = false;
  };
  std::vector<Sys> sys(P);
  std::vector<double> hnorm(P), col(ld + 1);
  for (Sys& q : sys) {
    q.Rh.assign((size_t)ld * ld, 0.0); q.gh.assign(ld, 0.0); q.yh.assign(ld, 0.0);
    q.csh.assign(ld, 0.0); q.snh.assign(ld, 0.0);
  }
  auto norms = [&](const double* X, std::vector<double>& out) -> int {
    for (int sy = 0; sy < P; ++sy) RC(kr_multidot(c->ws, X + (size_t)sy * n, n, 1, X + (size_t)sy * n, n, tmp, 0,
                                                  nrm + sy, st));
    CK(cudaMemcpyAsync(out.data(), nrm, P * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return IMPS_OK;
  };
  RC(norms(b, hnorm));
  for (int sy = 0; sy < P; ++sy) {
    sys[sy].bnorm = hnorm[sy];
    if (!std::isfinite(hnorm[sy])) return IMPS_ERR_NAN;
    if (hnorm[sy] == 0.0) {
      CK(cudaMemsetAsync(y + (size_t)sy * n, 0, n * 8, st));
      sys[sy].done = true;
    }
  }
  int it = 0;
  auto any_open = [&]() { for (const Sys& q : sys) if (!q.done) return true; return false; };
  for (int outer = 0; any_open() && it < maxit; ++outer) {
    // r = b - A(y) for every system
    RC(Ab(y, W));
    RC(kr_axpby(1.0, b, -1.0, W, ntot, st));
    RC(norms(W, hnorm));
    for (int sy = 0; sy < P; ++sy) {
      Sys& q = sys[sy];
      q.in_cycle = false;
      if (q.done) continue;
      q.rn = hnorm[sy];
      if (!std::isfinite(q.rn)) return IMPS_ERR_NAN;
      if (q.rn < tol * q.bnorm) { q.done = true; continue; }
      // the stagnation rule of gmres_dev, per system
      q.stall = outer > 0 && q.inner_hit && q.rn > 0.9 * q.rn_prev ? q.stall + 1 : 0;
      q.rn_prev = q.rn;
      if (q.stall >= 3) { q.done = true; continue; }
      q.inner_hit = false;
      q.in_cycle = true;
      q.kdim = 0;
      q.jpulled = 0;
      std::fill(q.gh.begin(), q.gh.end(), 0.0);
      q.gh[0] = q.rn;
      RC(kr_scale_inv(W + (size_t)sy * n, nrm + sy, Vs(sy), n, nullptr, st));
    }
    for (int j = 0; j < m && it < maxit; ++j) {
      bool any = false;
      for (int sy = 0; sy < P; ++sy)
        if (sys[sy].in_cycle) {
          any = true;
          CK(cudaMemcpyAsync(U + (size_t)sy * n, Vs(sy) + (size_t)j * n, n * 8, cudaMemcpyDeviceToDevice, st));
        }
      if (!any) break;
      RC(Ab(U, W));
      ++it;
      // every system's CGS step in one set of launches (systems outside their cycle work on
      // their own unused columns)
      RC(kr_cgs2_step_batch(parts, counters, P, V, n * (m + 1), n, j + 1, W, n, n, Hd + (size_t)j * ld,
                            (int64_t)ld * m, h2, V + (size_t)(j + 1) * n, nullptr, st));
      for (int sy = 0; sy < P; ++sy) {
        Sys& q = sys[sy];
        if (!q.in_cycle) continue;
        q.kdim = j + 1;
        ++q.it;
      }
      if (!((j + 1) % 4 == 0 || j == m - 1 || it >= maxit)) continue;
      CK(cudaStreamSynchronize(st));
      for (int sy = 0; sy < P; ++sy) {
        Sys& q = sys[sy];
        if (!q.in_cycle) continue;
        CK(cudaMemcpy(c->hpin_g, Hd + (size_t)sy * ld * m + (size_t)q.jpulled * ld,
                      (size_t)(j + 1 - q.jpulled) * ld * 8, cudaMemcpyDeviceToHost));
        double res = 0.0;
        bool brk = false;
        for (int qq = q.jpulled; qq <= j; ++qq) {
          const double* hc = c->hpin_g + (size_t)(qq - q.jpulled) * ld;
          for (int i = 0; i <= qq + 1; ++i) col[i] = hc[i];
          for (int i = 0; i < qq; ++i) {
            const double h1 = col[i], h2 = col[i + 1];
            col[i] = q.csh[i] * h1 + q.snh[i] * h2;
            col[i + 1] = -q.snh[i] * h1 + q.csh[i] * h2;
          }
          const double hqq = col[qq], hq1 = col[qq + 1];
          const double beta = std::sqrt(hqq * hqq + hq1 * hq1);
          if (!std::isfinite(beta)) return IMPS_ERR_NAN;
          if (!(beta >= 2e-16)) { brk = true; q.kdim = qq; break; }
          const double habs = std::fabs(hqq);
          const double phase = habs > 0.0 ? hqq / habs : 1.0;
          q.snh[qq] = phase * hq1 / beta;
          q.csh[qq] = habs / beta;
          col[qq] = phase * beta;
          q.gh[qq + 1] = -q.snh[qq] * q.gh[qq];
          q.gh[qq] *= q.csh[qq];
          for (int i = 0; i <= qq; ++i) q.Rh[i + (size_t)qq * ld] = col[i];
          res = std::fabs(q.gh[qq + 1]);
        }
        q.jpulled = j + 1;
        if (brk) { q.in_cycle = false; continue; }
        if (res < tol * q.bnorm) { q.inner_hit = true; q.in_cycle = false; }
      }
    }
    // y_s += V_s[:, :kdim] R^{-1} gamma for every system that extended its basis this cycle
    for (int sy = 0; sy < P; ++sy) {
      Sys& q = sys[sy];
      if (q.done || q.kdim <= 0) continue;
      for (int i = q.kdim - 1; i >= 0; --i) {
        double sacc = q.gh[i];
        for (int qq = i + 1; qq < q.kdim; ++qq) sacc -= q.Rh[i + (size_t)qq * ld] * q.yh[qq];
        q.yh[i] = sacc / q.Rh[i + (size_t)i * ld];
      }
      CK(cudaMemcpy(ys, q.yh.data(), q.kdim * 8, cudaMemcpyHostToDevice));
      RC(kr_gemv(Vs(sy), n, q.kdim, ys, Tm, n, st));
      RC(kr_axpby(1.0, Tm, 1.0, y + (size_t)sy * n, n, st));
      CK(cudaStreamSynchronize(st));  // ys and Tm are reused by the next system
      q.kdim = 0;
    }
  }
  // final residuals
  RC(Ab(y, W));
  RC(kr_axpby(1.0, b, -1.0, W, ntot, st));
  RC(norms(W, hnorm));
  double worst = 0.0;
  bool ok = true;
  for (int sy = 0; sy < P; ++sy) {
    const Sys& q = sys[sy];
    const double r = q.bnorm > 0.0 ? hnorm[sy] / q.bnorm : 0.0;
    worst = std::max(worst, r);
    ok = ok && r < tol;
  }
  if (iters) *iters = it;
  if (relres) *relres = worst;
  if (debug_on())
    fprintf(stderr, "[imps gmres_batch] P=%d n=%lld iters=%d worst relres=%.3e tol=%.1e\n", P, (long long)n, it,
            worst, tol);
  return ok ? IMPS_OK : IMPS_WARN_NOT_CONVERGED;
}

int imps_invert_e_fac_batch(imps_plan* rep, int P, const double* const* x_re, const double* const* x_im,
                            const double* fac_re, const double* fac_im, double* const* y_re, double* const* y_im,
                            double tol, int maxit, int krylov, int* iters, double* relres) {
  if (!rep || P < 1 || !x_re || !x_im || !fac_re || !fac_im || !y_re || !y_im) return IMPS_ERR_BAD_ARG;
  imps_ctx* c = rep->ctx;
  if (c->device < 0) return IMPS_ERR_NO_DEVICE;
  const int64_t ntot = rep->P.slots[rep->P.n_in].nelem;
  if (ntot % (2 * (int64_t)P) || rep->P.slots[rep->P.n_out].nelem != ntot) return IMPS_ERR_BAD_ARG;
  const int64_t n = ntot / (2 * (int64_t)P);  // one plane; a system is [re | im], 2n
  cudaStream_t st = c->stream;
  int m = krylov > 0 ? std::min(krylov, kMaxCols - 2) : kGmresKrylov;
  if (maxit <= 0) maxit = (int)std::min<int64_t>(2 * n, 100000);
  RC(arena_reserve(c, round256(ntot * 8) * (m + 6) + round256(2 * n * 8) + round256((size_t)P * (m + 1) * (m + 1) * 8) +
                          4 * round256((size_t)P * 8) + round256((size_t)P * kMaxCols * 8) +
                          round256((size_t)P * CGS_BATCH_GRID * kMaxCols * 8) + 16 * 4096));
  Bump bp{c->arena};
  double* b = bp.take(ntot);
  double* y = bp.take(ntot);
  double* t = bp.take(ntot);
  double* dfr = bp.take(P);
  double* dfi = bp.take(P);
  CK(cudaMemcpyAsync(dfr, fac_re, P * 8, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(dfi, fac_im, P * 8, cudaMemcpyHostToDevice, st));
  for (int j = 0; j < P; ++j) {  // stack [re_j | im_j]
    CK(cudaMemcpyAsync(b + 2 * j * n, x_re[j], n * 8, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(b + (2 * j + 1) * n, x_im[j], n * 8, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(y + 2 * j * n, y_re[j], n * 8, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(y + (2 * j + 1) * n, y_im[j], n * 8, cudaMemcpyDeviceToDevice, st));
  }
  // one apply of the replicated transfer matrix takes every plane of every system
  BatchOp A = [&](const double* u, double* out) -> int {
    RC(apply_dev(rep, u, t));
    return kr_fac_epilogue_batch(u, t, dfr, dfi, out, n, P, st);
  };
  const int prec_saved = rep->prec;
  rep->prec = IMPS_PREC_FP64;
  const int rc = gmres_batch(c, P, 2 * n, A, b, y, tol, maxit, m, iters, relres, bp);
  rep->prec = prec_saved;
  if (rc < 0) return rc;
  for (int j = 0; j < P; ++j) {
    CK(cudaMemcpyAsync(y_re[j], y + 2 * j * n, n * 8, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(y_im[j], y + (2 * j + 1) * n, n * 8, cudaMemcpyDeviceToDevice, st));
  }
  CK(cudaStreamSynchronize(st));
  return rc;
}

int imps_tm_dominant(imps_plan* p, const double* x0, double* V, int mem, double tol, int maxit,
                     double* eval, int* iters) {
  if (!p || p->P.kind != PLAN_TM || !V) return IMPS_ERR_BAD_ARG;
  imps_ctx* c = p->ctx;
  cudaStream_t st = c->stream;
  const int64_t n = p->P.slots[0].nelem;
  if (p->P.slots[1].nelem != n) return IMPS_ERR_BAD_ARG;
  const int m = kGmresKrylov;
  if (maxit <= 0) maxit = (int)std::min<int64_t>(n, 100000);
  RC(arena_reserve(c, round256(n * 8) * (m + 14) + round256((size_t)(m + 1) * (m + 1) * 8) + 16 * 4096));
  Bump bp{c->arena};
  double* eye = bp.take(n);
  double* r0 = bp.take(n);
  double* v = bp.take(n);
  imps::count_launch();
  imps_set_identity_kernel<<<std::max(p->nb_in, 1), 256, 0, st>>>(eye, p->d_boff, p->d_bdim, p->nb_in);
  if (x0) {
    CK(cudaMemcpyAsync(r0, x0, n * 8, mem == IMPS_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, st));
  } else {
    CK(cudaMemcpyAsync(r0, eye, n * 8, cudaMemcpyDeviceToDevice, st));
  }
  // normalise the seed to unit trace: r0 /= tr(r0)
  RC(kr_trace_prod(c->ws, r0, eye, p->d_boff, p->d_bdim, p->nb_in, c->dscal + 5, st));
  RC(kr_scale_inv(r0, c->dscal + 5, r0, n, nullptr, st));
  CK(cudaMemcpyAsync(v, r0, n * 8, cudaMemcpyDeviceToDevice, st));
  // (1 - T + |r0)(1|) v = r0.  The residual of this linear system floors near 1e-15 in FP64,
  // so tolerances below kDominantTolFloor are raised to it (ARPACK's Ritz criterion, used by
  // the reference with tol = 1e-15, is met at that level).
  int rc = gmres_proj(p, r0, v, eye, r0, std::max(tol, kDominantTolFloor), maxit, m, iters, nullptr, bp);
  if (rc < 0) return rc;
  // normalise by the trace (EigsBlockFunctions.hpp:162) and estimate the eigenvalue
  RC(kr_trace_prod(c->ws, v, eye, p->d_boff, p->d_bdim, p->nb_in, c->dscal + 5, st));
  RC(kr_scale_inv(v, c->dscal + 5, v, n, nullptr, st));
  double* tv = bp.take(n);
  RC(apply_dev(p, v, tv));
  RC(kr_trace_prod(c->ws, tv, eye, p->d_boff, p->d_bdim, p->nb_in, c->dscal + 6, st));
  double lam = 0.0;
  CK(cudaMemcpyAsync(&lam, c->dscal + 6, 8, cudaMemcpyDeviceToHost, st));
  if (mem == IMPS_MEM_HOST) CK(cudaMemcpyAsync(V, v, n * 8, cudaMemcpyDeviceToHost, st));
  else CK(cudaMemcpyAsync(V, v, n * 8, cudaMemcpyDeviceToDevice, st));
  CK(cudaStreamSynchronize(st));
  if (eval) *eval = lam;
  return rc;
}

int imps_grad_norm_right(imps_plan* p, double* F) {
  if (!p || p->P.kind != PLAN_GRAD || !F) return IMPS_ERR_BAD_ARG;
  imps_ctx* c = p->ctx;
  cudaStream_t st = c->stream;
  Slot& Y = p->P.slots[0];
  Slot& G = p->P.slots[2];
  if (!Y.dptr || !G.dptr || !p->P.slots[1].dptr) return IMPS_ERR_BAD_ARG;
  CK(cudaMemcpyAsync(G.dptr, Y.dptr, Y.nelem * 8, cudaMemcpyDeviceToDevice, st));
  RC(run_stages(p, p->P.stages));
  if (p->nseg == 0 || p->count_elems == 0) { *F = 0.0; return IMPS_OK; }
  RC(kr_segsq(c->ws, G.dptr, p->d_soff, p->d_slen, p->nseg, c->dscal + 7, st));
  double s = 0.0;
  CK(cudaMemcpyAsync(&s, c->dscal + 7, 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  *F = std::sqrt(s) / std::sqrt((double)p->count_elems);
  return IMPS_OK;
}

// ---- per-sector decompositions ----
int imps_plan_decomp(imps_ctx* ctx, const imps_layout* A, int dir, imps_plan** out) {
  if (!ctx || !A || !out || (dir != 0 && dir != 1)) return IMPS_ERR_BAD_ARG;
  DecompPlan* D = new (std::nothrow) DecompPlan();
  if (!D) return IMPS_ERR_OOM;
  int rc = build_decomp(*D, A->L, dir);
  if (rc) { delete D; return rc; }
  imps_plan* p = new (std::nothrow) imps_plan();
  if (!p) { delete D; return IMPS_ERR_OOM; }
  p->ctx = ctx;
  p->P.kind = PLAN_DECOMP;
  p->P.derived.push_back(A->L);
  p->P.derived.push_back(D->rlayout);
  p->P.derived.push_back(D->nslayout);  // left null space (dir l; empty for dir r)
  p->dc = D;
  *out = p;
  if (ctx->device < 0) return IMPS_OK;
  auto alloc = [&](double** ptr, int64_t n) -> int {
    CK(cudaMalloc(ptr, std::max<int64_t>(n, 1) * sizeof(double)));
    return IMPS_OK;
  };
  if (!D->ent.empty()) {
    CK(cudaMalloc(&D->d_ent, D->ent.size() * sizeof(GatherEntry)));
    CK(cudaMemcpy(D->d_ent, D->ent.data(), D->ent.size() * sizeof(GatherEntry), cudaMemcpyHostToDevice));
  }
  if (!D->mats.empty()) {
    CK(cudaMalloc(&D->d_mats, D->mats.size() * sizeof(DenseMat)));
    CK(cudaMemcpy(D->d_mats, D->mats.data(), D->mats.size() * sizeof(DenseMat), cudaMemcpyHostToDevice));
  }
  RC(alloc(&D->dA, D->dense_elems));
  RC(alloc(&D->dQ, D->dense_elems));
  RC(alloc(&D->dR, D->r_elems));
  RC(alloc(&D->dV2, D->r_elems));
  RC(alloc(&D->dS, D->s_elems));
  RC(alloc(&D->dW, D->w_elems));
  RC(alloc(&D->dNS, D->ns_elems));
  if (!D->nent.empty()) {
    CK(cudaMalloc(&D->d_nent, D->nent.size() * sizeof(GatherEntry)));
    CK(cudaMemcpy(D->d_nent, D->nent.data(), D->nent.size() * sizeof(GatherEntry), cudaMemcpyHostToDevice));
  }
  CK(cudaMalloc(&D->dstatus, sizeof(int)));
  return IMPS_OK;
}

// Nullspace(A, l) (MPSBlockUtilities.hpp:247-300): N_L with A_s^T-orthogonal, orthonormal columns
// per right sector; layout: derived layout 2 of the plan.  A must be left-isometric (full
// column rank per sector); the basis is the Householder complement (the reference's SVD basis
// spans the same space).
int imps_sector_nullspace(imps_plan* p, const double* A, double* NL, int mem) {
  if (!p || p->P.kind != PLAN_DECOMP || !A || !NL || mem != IMPS_MEM_DEVICE) return IMPS_ERR_BAD_ARG;
  if (p->ctx->device < 0) return IMPS_ERR_NO_DEVICE;
  DecompPlan* D = p->dc;
  if (D->dir != 0 || !D->tall) return IMPS_ERR_UNSUPPORTED;
  cudaStream_t st = p->ctx->stream;
  RC(dc_gather(D->d_ent, (int)D->ent.size(), A, D->dA, st));
  RC(dc_nullspace(D->d_mats, (int)D->mats.size(), D->dA, D->dNS, st));
  RC(dc_scatter(D->d_nent, (int)D->nent.size(), D->dNS, NL, st));
  return IMPS_OK;
}

int imps_sector_qr(imps_plan* p, const double* A, double* Q, double* R, int mem) {
  if (!p || p->P.kind != PLAN_DECOMP || !A || !Q || !R || mem != IMPS_MEM_DEVICE) return IMPS_ERR_BAD_ARG;
  if (p->ctx->device < 0) return IMPS_ERR_NO_DEVICE;
  DecompPlan* D = p->dc;
  if (!D->tall) return IMPS_ERR_UNSUPPORTED;
  cudaStream_t st = p->ctx->stream;
  RC(dc_gather(D->d_ent, (int)D->ent.size(), A, D->dA, st));
  RC(dc_qr(D->d_mats, (int)D->mats.size(), D->dA, D->dQ, R, D->dir == 1, st));
  RC(dc_scatter(D->d_ent, (int)D->ent.size(), D->dQ, Q, st));
  return IMPS_OK;
}

int imps_sector_svd(imps_plan* p, const double* A, double* U, double* S, double* Viso, int mem) {
  if (!p || p->P.kind != PLAN_DECOMP || !A || mem != IMPS_MEM_DEVICE) return IMPS_ERR_BAD_ARG;
  if (p->ctx->device < 0) return IMPS_ERR_NO_DEVICE;
  DecompPlan* D = p->dc;
  if (!D->tall) return IMPS_ERR_UNSUPPORTED;
  cudaStream_t st = p->ctx->stream;
  CK(cudaMemsetAsync(D->dstatus, 0, sizeof(int), st));
  RC(dc_gather(D->d_ent, (int)D->ent.size(), A, D->dA, st));
  int maxN = 0;
  int64_t maxMN = 0;
  for (const DenseMat& m : D->mats) {
    maxN = std::max(maxN, (int)m.N);
    maxMN = std::max(maxMN, (int64_t)m.M * m.N);
  }
  RC(dc_svd(D->d_mats, (int)D->mats.size(), maxN, maxMN, D->dA, S ? S : D->dS, D->dR, D->dW, D->dstatus, st));
  if (U) RC(dc_scatter(D->d_ent, (int)D->ent.size(), D->dA, U, st));
  if (Viso) {
    if (D->dir == 0) RC(dc_transpose_sq(D->d_mats, (int)D->mats.size(), D->dR, Viso, st));  // V^T
    else CK(cudaMemcpyAsync(Viso, D->dR, D->r_elems * 8, cudaMemcpyDeviceToDevice, st));   // V
  }
  int status = 0;
  CK(cudaMemcpyAsync(&status, D->dstatus, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return status ? IMPS_WARN_NOT_CONVERGED : IMPS_OK;
}

int imps_sector_svd_batch(int np, imps_plan* const* plans, const double* const* A, double* const* U,
                          double* const* S, double* const* Viso, int mem) {
  if (np < 1 || np > kSvdSets || !plans || !A || mem != IMPS_MEM_DEVICE) return IMPS_ERR_BAD_ARG;
  imps_ctx* c = plans[0] ? plans[0]->ctx : nullptr;
  if (!c) return IMPS_ERR_BAD_ARG;
  if (c->device < 0) return IMPS_ERR_NO_DEVICE;
  cudaStream_t st = c->stream;
  SvdSets sets{};
  sets.nsets = np;
  int maxN = 0;
  int64_t maxMN = 0;
  for (int k = 0; k < np; ++k) {
    imps_plan* p = plans[k];
    if (!p || p->P.kind != PLAN_DECOMP || p->ctx != c || !A[k] || !p->dc->tall) return IMPS_ERR_BAD_ARG;
    DecompPlan* D = p->dc;
    for (const DenseMat& m : D->mats) {
      maxN = std::max(maxN, (int)m.N);
      maxMN = std::max(maxMN, (int64_t)m.M * m.N);
    }
    RC(dc_gather(D->d_ent, (int)D->ent.size(), A[k], D->dA, st));
    sets.s[k] = SvdSet{D->d_mats, D->dA, (S && S[k]) ? S[k] : D->dS, D->dR, D->dW, (int)D->mats.size()};
  }
  int* status = plans[0]->dc->dstatus;
  CK(cudaMemsetAsync(status, 0, sizeof(int), st));
  RC(dc_svd_sets(sets, maxN, maxMN, status, st));
  for (int k = 0; k < np; ++k) {
    DecompPlan* D = plans[k]->dc;
    if (U && U[k]) RC(dc_scatter(D->d_ent, (int)D->ent.size(), D->dA, U[k], st));
    if (Viso && Viso[k]) {
      if (D->dir == 0) RC(dc_transpose_sq(D->d_mats, (int)D->mats.size(), D->dR, Viso[k], st));
      else CK(cudaMemcpyAsync(Viso[k], D->dR, D->r_elems * 8, cudaMemcpyDeviceToDevice, st));
    }
  }
  int stat = 0;
  CK(cudaMemcpyAsync(&stat, status, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return stat ? IMPS_WARN_NOT_CONVERGED : IMPS_OK;
}

int imps_sector_colscale(imps_plan* p, double* X, const double* S, double power, int mem) {
  if (!p || p->P.kind != PLAN_DECOMP || !X || !S || mem != IMPS_MEM_DEVICE) return IMPS_ERR_BAD_ARG;
  if (p->ctx->device < 0) return IMPS_ERR_NO_DEVICE;
  DecompPlan* D = p->dc;
  for (const DenseMat& m : D->mats)
    if (m.M != m.N) return IMPS_ERR_BAD_ARG;  // BlockDiagMat plans only
  return dc_colscale(D->d_mats, (int)D->mats.size(), X, S, power, p->ctx->stream);
}

// ---- device-vector helpers for drivers ----
int imps_bd_trace_prod(imps_ctx* c, imps_layout* L, const double* X, const double* Y, double* result) {
  if (!c || !L || !X || !Y || !result) return IMPS_ERR_BAD_ARG;
  if (!L->d_boff && !L->L.blocks.empty()) {
    std::vector<int64_t> bo;
    std::vector<int32_t> bd;
    for (const Block& b : L->L.blocks) { bo.push_back(b.off); bd.push_back(b.rows); }
    CK(cudaMalloc(&L->d_boff, bo.size() * 8));
    CK(cudaMalloc(&L->d_bdim, bd.size() * 4));
    CK(cudaMemcpy(L->d_boff, bo.data(), bo.size() * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(L->d_bdim, bd.data(), bd.size() * 4, cudaMemcpyHostToDevice));
  }
  RC(kr_trace_prod(c->ws, X, Y, L->d_boff, L->d_bdim, (int)L->L.blocks.size(), c->dscal + 16, c->stream));
  CK(cudaMemcpyAsync(result, c->dscal + 16, 8, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return IMPS_OK;
}

int imps_absmax(imps_ctx* c, const double* x, int64_t n, double* result) {
  if (!c || !x || !result) return IMPS_ERR_BAD_ARG;
  RC(kr_absmax(c->ws, x, n, c->dscal + 17, c->stream));
  CK(cudaMemcpyAsync(result, c->dscal + 17, 8, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return IMPS_OK;
}

int imps_axpby(imps_ctx* c, double a, const double* x, double b, double* y, int64_t n) {
  if (!c || !x || !y) return IMPS_ERR_BAD_ARG;
  return kr_axpby(a, x, b, y, n, c->stream);
}

// x /= sign(x[0])  (VUMPS_main.cpp:201-202; sign(0) is taken as +1)
int imps_sign_normalize(imps_ctx* c, double* x, int64_t n) {
  if (!c || !x || n < 1) return IMPS_ERR_BAD_ARG;
  RC(kr_sign_of_first(x, c->dscal + 18, c->stream));
  RC(kr_scale_inv(x, c->dscal + 18, x, n, nullptr, c->stream));
  return IMPS_OK;
}

}  // extern "C"
