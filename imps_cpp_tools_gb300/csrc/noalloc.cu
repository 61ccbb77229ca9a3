// Single-site transfer-matrix apply that allocates no device memory.
//
// Who needs it: callers that cannot call cudaMalloc at the point where they apply the
// transfer matrix -- e.g. a host application whose GPU memory is fully reserved up front by
// another allocator (a framework's caching pool that owns the device), or a latency-critical
// loop that must not pay cudaMalloc's implicit device synchronisation.  The regular path
// (imps_plan_tm + imps_tm_apply) allocates its intermediate W = X*A_s and its task tables
// when the plan is created; this entry point instead keeps both in file-scope device arrays
// of fixed size that every GPU loading the library holds until the process exits.
//
// Limits (checked on every call, IMPS_ERR_TOO_LARGE beyond them):
//   intermediate W (the MPS tensor's element count) <= kNoAllocMaxScratch doubles (8 MiB),
//   output tiles per stage <= kNoAllocMaxTiles, GEMM terms per stage <= kNoAllocMaxTerms.
// Sharing: every call uses the same arrays and leaves its contents behind.  Each stage
// overwrites every element it later reads (no part of the scratch has to start at zero),
// but calls whose work overlaps on the GPU race on the scratch: issue them on one stream or
// otherwise serialise them.  The host-side staging of the task tables is also shared, so
// calls must not run concurrently from several host threads.
// Task tables: built on the host for every call and copied to the device (a copy from
// pageable host memory) only when they differ from the last ones copied to this device, so
// a loop over one set of layouts copies them once.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>

#include "../../include/imps_gb300.h"
#include "imps_handles.h"
#include "imps_internal.h"

namespace {

constexpr int64_t kNoAllocMaxScratch = 1 << 20;  // doubles
constexpr int kNoAllocMaxTiles = 8192;
constexpr int kNoAllocMaxTerms = 8192;
constexpr int kMaxDevices = 64;
constexpr int kTile = 32;

struct TableImage {
  imps::Tile tiles[2][kNoAllocMaxTiles];
  imps::Term terms[2][kNoAllocMaxTerms];
};

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocMaxScratch];
static __device__ __align__(256) unsigned char g_noalloc_tables[sizeof(TableImage)];

// host-side staging of the task tables (static, so that building them allocates nothing)
static TableImage h_img;
static double* d_scratch[kMaxDevices];
static unsigned char* d_tables[kMaxDevices];
static bool ready[kMaxDevices];

struct StageOut {
  int ntiles = 0, nterms = 0;
  bool overflow = false;
};

// the tables last copied to a device (one record: the device and the stage contents)
static TableImage h_last;
static int last_dev = -1;
static StageOut last_stage[2];

bool same_as_last(int dev, const StageOut* so) {
  if (dev != last_dev) return false;
  for (int s = 0; s < 2; ++s) {
    if (so[s].ntiles != last_stage[s].ntiles || so[s].nterms != last_stage[s].nterms) return false;
    if (memcmp(h_img.tiles[s], h_last.tiles[s], so[s].ntiles * sizeof(imps::Tile)) ||
        memcmp(h_img.terms[s], h_last.terms[s], so[s].nterms * sizeof(imps::Term)))
      return false;
  }
  return true;
}

void remember(int dev, const StageOut* so) {
  for (int s = 0; s < 2; ++s) {
    memcpy(h_last.tiles[s], h_img.tiles[s], so[s].ntiles * sizeof(imps::Tile));
    memcpy(h_last.terms[s], h_img.terms[s], so[s].nterms * sizeof(imps::Term));
    last_stage[s] = so[s];
  }
  last_dev = dev;
}

// every block of a BlockDiagMat layout must be square (the products below assume it)
bool square_blocks(const imps::Layout& L) {
  for (const imps::Block& b : L.blocks)
    if (b.rows != b.cols) return false;
  return true;
}

// emit an output block's tiles (all sharing the block's term range [t0, t1))
void emit_tiles(StageOut& so, imps::Tile* tiles, int c_slot, int64_t c_off, int ld, int M, int N, int t0, int t1) {
  for (int n0 = 0; n0 < N; n0 += kTile)
    for (int m0 = 0; m0 < M; m0 += kTile) {
      if (so.ntiles >= kNoAllocMaxTiles) { so.overflow = true; return; }
      imps::Tile& t = tiles[so.ntiles++];
      t.c_off = c_off;
      t.c_ld = ld > 0 ? ld : 1;
      t.m0 = m0;
      t.n0 = n0;
      t.mt = M - m0 < kTile ? M - m0 : kTile;
      t.nt = N - n0 < kTile ? N - n0 : kTile;
      t.t0 = t0;
      t.t1 = t1;
      t.c_slot = (int16_t)c_slot;
      t.accumulate = 0;
      t.part = 0;
      t.nparts = 1;
      t.ws_unit = 0;
      t.cnt_idx = 0;
    }
}

void push_term(StageOut& so, imps::Term* terms, int a_slot, int64_t a_off, int a_ld, int a_t, int b_slot,
               int64_t b_off, int b_ld, int b_t, int k) {
  if (so.nterms >= kNoAllocMaxTerms) { so.overflow = true; return; }
  imps::Term& t = terms[so.nterms++];
  t = imps::Term{};
  t.a_slot = (int16_t)a_slot; t.a_off = a_off; t.a_ld = a_ld > 0 ? a_ld : 1; t.a_t = (int8_t)a_t;
  t.b_slot = (int16_t)b_slot; t.b_off = b_off; t.b_ld = b_ld > 0 ? b_ld : 1; t.b_t = (int8_t)b_t;
  t.k = k;
  t.alpha = 1.0;
}

}  // namespace

extern "C" int imps_tm_apply_noalloc(const imps_layout* A, const imps_layout* in, const imps_layout* out, int dir,
                                     const double* dA, const double* dX, double* dY, void* stream) {
  if (!A || !in || !out || !dA || !dX || !dY || (dir != 0 && dir != 1)) return IMPS_ERR_BAD_ARG;
  const imps::Layout& LA = A->L;
  const imps::Layout& LI = in->L;
  const imps::Layout& LO = out->L;
  if (!square_blocks(LI) || !square_blocks(LO)) {
    fprintf(stderr, "imps_tm_apply_noalloc: in and out must be BlockDiagMat layouts (square blocks)\n");
    return IMPS_ERR_BAD_TABLE;
  }
  if (LA.nelem > kNoAllocMaxScratch) {
    fprintf(stderr, "imps_tm_apply_noalloc: MPS tensor has %lld elements, the static scratch holds %lld\n",
            (long long)LA.nelem, (long long)kNoAllocMaxScratch);
    return IMPS_ERR_TOO_LARGE;
  }
  // once per device, with that device current: the device address of the static arrays
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return IMPS_ERR_NO_DEVICE;
  if (!ready[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      fprintf(stderr, "imps_tm_apply_noalloc: cudaGetSymbolAddress(scratch): %s\n", cudaGetErrorString(e));
      return IMPS_ERR_CUDA;
    }
    d_scratch[dev] = (double*)p;
    e = cudaGetSymbolAddress(&p, g_noalloc_tables);
    if (e != cudaSuccess) {
      fprintf(stderr, "imps_tm_apply_noalloc: cudaGetSymbolAddress(tables): %s\n", cudaGetErrorString(e));
      return IMPS_ERR_CUDA;
    }
    d_tables[dev] = (unsigned char*)p;
    ready[dev] = true;
  }
  // slots: 0 X (in), 1 Y (out), 2 A, 3 W (static scratch, A's layout)
  enum { SX = 0, SY = 1, SA = 2, SW = 3 };
  StageOut s1, s2;
  // stage 1: W_b = X(qin) A_b (left) or A_b X(qout) (right); blocks without an X sector -> 0
  for (const imps::Block& b : LA.blocks) {
    const int t0 = s1.nterms;
    const int x = LI.find_in(0, dir == 0 ? b.qin : b.qout);
    if (x >= 0) {
      const imps::Block& X = LI.blocks[x];
      const int m = dir == 0 ? b.rows : b.cols;
      if (X.rows != m || X.cols != m) return IMPS_ERR_BAD_TABLE;
      if (dir == 0) push_term(s1, h_img.terms[0], SX, X.off, m, 0, SA, b.off, b.rows, 0, b.rows);
      else push_term(s1, h_img.terms[0], SA, b.off, b.rows, 0, SX, X.off, m, 0, b.cols);
    }
    emit_tiles(s1, h_img.tiles[0], SW, b.off, b.rows, b.rows, b.cols, t0, s1.nterms);
  }
  // stage 2: Y(q) = sum_b A_b^T W_b (left, Qout(b) = q) or W_b A_b^T (right, Qin(b) = q)
  for (const imps::Block& o : LO.blocks) {
    const int t0 = s2.nterms;
    for (int g = 0; g < LA.ngroups; ++g) {
      const int bi = dir == 0 ? LA.find_out(g, o.qin) : LA.find_in(g, o.qin);
      if (bi < 0) continue;
      const imps::Block& b = LA.blocks[bi];
      if (LI.find_in(0, dir == 0 ? b.qin : b.qout) < 0) continue;
      if (dir == 0) {
        if (b.cols != o.rows) return IMPS_ERR_BAD_TABLE;
        push_term(s2, h_img.terms[1], SA, b.off, b.rows, 1, SW, b.off, b.rows, 0, b.rows);
      } else {
        if (b.rows != o.rows) return IMPS_ERR_BAD_TABLE;
        push_term(s2, h_img.terms[1], SW, b.off, b.rows, 0, SA, b.off, b.rows, 1, b.cols);
      }
    }
    emit_tiles(s2, h_img.tiles[1], SY, o.off, o.rows, o.rows, o.cols, t0, s2.nterms);
  }
  if (s1.overflow || s2.overflow) {
    fprintf(stderr, "imps_tm_apply_noalloc: more than %d tiles or %d terms per stage\n", kNoAllocMaxTiles,
            kNoAllocMaxTerms);
    return IMPS_ERR_TOO_LARGE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  TableImage* dimg = (TableImage*)d_tables[dev];
  const StageOut stages[2] = {s1, s2};
  if (!same_as_last(dev, stages)) {
    last_dev = -1;  // a failed copy leaves the device tables unknown
    // pageable-host copies return once the staging buffer has been consumed
    for (int s = 0; s < 2; ++s) {
      const StageOut& so = stages[s];
      if (so.ntiles && cudaMemcpyAsync(dimg->tiles[s], h_img.tiles[s], so.ntiles * sizeof(imps::Tile),
                                       cudaMemcpyHostToDevice, st) != cudaSuccess)
        return IMPS_ERR_CUDA;
      if (so.nterms && cudaMemcpyAsync(dimg->terms[s], h_img.terms[s], so.nterms * sizeof(imps::Term),
                                       cudaMemcpyHostToDevice, st) != cudaSuccess)
        return IMPS_ERR_CUDA;
    }
    remember(dev, stages);
  }
  imps_dslots sl{};
  sl.p[SX] = const_cast<double*>(dX);
  sl.p[SY] = dY;
  sl.p[SA] = const_cast<double*>(dA);
  sl.p[SW] = d_scratch[dev];
  int rc = imps_launch_grouped_f64(dimg->tiles[0], s1.ntiles, dimg->terms[0], sl, kTile, 1, nullptr, nullptr, stream);
  if (rc) return rc;
  return imps_launch_grouped_f64(dimg->tiles[1], s2.ntiles, dimg->terms[1], sl, kTile, 1, nullptr, nullptr, stream);
}
