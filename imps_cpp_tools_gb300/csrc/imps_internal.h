// Internal declarations shared by the planner (host C++) and the CUDA kernels.
//
// Architecture: every block-sparse contraction of the hot path (H_AC, H_C, transfer
// matrices, reduced operators, ...) is compiled on the host into "stages".  A stage is a
// grouped GEMM: a list of output tiles, each owning a contiguous range of terms
// C_tile (+)= sum_t alpha_t * op(A_t) * op(B_t).  Sector matching (the std::map lookups
// the reference performs in every apply) happens once, here, as integer tables; the GPU
// only ever sees flat offsets into a few device buffers ("slots").
#pragma once
#include <atomic>
#include <cstdint>
#include <map>
#include <string>
#include <vector>

namespace imps {

// process-wide count of kernel launches issued by this library (imps_launch_count)
std::atomic<long long>& launch_counter();
inline void count_launch(int k = 1) { launch_counter().fetch_add(k, std::memory_order_relaxed); }

using Key = std::vector<int32_t>;

struct Block {
  Key qin, qout;
  int32_t rows = 0, cols = 0;
  int32_t group = 0;  // physical index s for an MPS tensor, i*d+j for a RedOp grid, 0 otherwise
  int64_t off = 0;    // element offset in the vectorised object (reference Vectorize order)
};

struct Layout {
  int nsym = 0;
  std::vector<Block> blocks;
  int64_t nelem = 0;
  int ngroups = 1;
  std::map<std::pair<int, Key>, int> by_in;   // (group, qin)  -> block index
  std::map<std::pair<int, Key>, int> by_out;  // (group, qout) -> block index (first one)
  int find_in(int g, const Key& k) const {
    auto it = by_in.find({g, k});
    return it == by_in.end() ? -1 : it->second;
  }
  int find_out(int g, const Key& k) const {
    auto it = by_out.find({g, k});
    return it == by_out.end() ? -1 : it->second;
  }
};

// One GEMM term: alpha * op(A) (MxK) * op(B) (KxN), A and B column-major blocks inside a
// slot; trans=1 means the stored matrix is op()^T.  Layout shared with the device (POD).
struct Term {
  int64_t a_off, b_off;
  int32_t a_ld, b_ld;
  int32_t k;
  int16_t a_slot, b_slot;
  int8_t a_t, b_t;
  int8_t pad[6];
  double alpha;
};
static_assert(sizeof(Term) == 48, "Term layout");

// One output tile (a rectangle of an output block); tiles of one block share its term range.
struct Tile {
  int64_t c_off;
  int32_t c_ld;
  int32_t m0, n0, mt, nt;
  int32_t t0, t1;
  int16_t c_slot;
  int16_t accumulate;  // 1: C += sum, 0: C = sum
  // split-K: the CTA of this entry takes share `part` of `nparts` equal shares of the tile's K
  // chunks; with nparts > 1 it stores its partial tile at workspace tile ws_unit + part, and the
  // ticket counter cnt_idx picks the CTA that sums the tile's partials
  int32_t part, nparts, ws_unit, cnt_idx;
};
static_assert(sizeof(Tile) == 56, "Tile layout");

// Logical output block with its terms (kept on the host for table export and for the
// tensor-core packer).
struct OutBlock {
  int64_t c_off;
  int32_t c_ld, M, N;
  int32_t t0, t1;
  int16_t c_slot;
  int16_t accumulate;
  int32_t tag;  // index of the output block in the output layout
};

struct Stage {
  std::vector<OutBlock> outs;
  std::vector<Term> terms;
  std::vector<Tile> tiles;
  void* d_tiles = nullptr;
  void* d_terms = nullptr;
  int64_t flops = 0;  // useful flops: sum over terms of 2*M*N*K
  int tile_m = 32, tile_n = 32;
  // split-K over CTAs (FP64 engine): `splits` CTAs per tile write partial tiles to d_ws and the
  // last one to finish (ticket in d_cnt, reset by it) sums them in a fixed order
  int splits = 1;
  double* d_ws = nullptr;
  int* d_cnt = nullptr;
};

enum SlotKind { SLOT_EXTERNAL = 0, SLOT_INTERNAL = 1 };

struct Slot {
  int kind = SLOT_EXTERNAL;
  int64_t nelem = 0;
  double* dptr = nullptr;  // bound pointer (external) or owned buffer (internal)
  std::string name;
};

constexpr int kMaxSlots = 16;

enum PlanKind {
  PLAN_HAC = 1, PLAN_HC = 2, PLAN_TM = 3, PLAN_REDOP = 4, PLAN_OPTM = 5, PLAN_MPS_BD = 6,
  PLAN_GRAD = 7, PLAN_AA = 8, PLAN_BD_MPS = 9, PLAN_TMMIXED_R = 10, PLAN_TMMIXED_L = 11,
  PLAN_PROGRAM = 12
};

// A compiled contraction: slots + prepare stages (operator-dependent precomputation,
// run when operators change) + apply stages (run per apply).
struct Plan {
  int kind = 0;
  std::vector<Slot> slots;
  std::vector<Stage> prep;
  std::vector<Stage> stages;
  std::vector<Layout> derived;  // layouts the plan derived (outputs / scratch), by role
  int64_t flops_apply = 0, flops_prep = 0;
  int64_t dropped = 0;          // products whose output sector is absent (reference: lost)
  int n_in = 0, n_out = 1;      // slot indices of the apply input / output
};

// ----- planner (planner.cpp) -----
int layout_build(Layout& L, int nsym, int nblocks, const int32_t* qin, const int32_t* qout,
                 const int32_t* rows, const int32_t* cols, const int32_t* group);
void layout_index(Layout& L);
Layout layout_bond(const Layout& A, int side);  // side 0: GetMl, 1: GetMr (as BlockDiag)

struct HNnz { int r, c; double v; };

int build_hac(Plan& P, const Layout& AC, const Layout& EHL, const Layout& EHR,
              const Layout& HL, const Layout& HR, int d);
int build_hc(Plan& P, const Layout& C, const Layout& EHL, const Layout& EHR,
             const Layout& AL, const Layout& AR, int d, const std::vector<HNnz>& h);
int build_tm(Plan& P, const std::vector<const Layout*>& A, int dir, const Layout& in,
             const Layout& out);
int build_tm_mixed(Plan& P, const std::vector<const Layout*>& A, const std::vector<const Layout*>& B,
                   int dir, const Layout& in, const Layout& out);
int build_redop(Plan& P, const Layout& A, int d, const std::vector<HNnz>& h, int dir);
int build_optm(Plan& P, const Layout& A0, const Layout& A1, int d, const std::vector<HNnz>& h,
               int dir, const Layout& out);
int build_mps_bd(Plan& P, const Layout& A, const Layout& X, int side, double alpha);
int build_grad_right(Plan& P, const Layout& Y, const Layout& AR);
void finalize_tiles(Stage& S, int tm, int tn);

}  // namespace imps

// ----- kernel launchers (kernels_f64.cu) -----
struct imps_dslots { double* p[imps::kMaxSlots]; };
// ntiles: table entries, one CTA each; splits: the largest share count of a tile (> 1 needs the
// workspace ws and the ticket counters cnt)
int imps_launch_grouped_f64(const void* d_tiles, int ntiles, const void* d_terms, imps_dslots slots,
                            int tile_m, int splits, double* ws, int* cnt, void* stream);
