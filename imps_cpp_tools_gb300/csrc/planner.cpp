// Host-side sector planner: turns the reference's per-apply std::map sector matching into
// integer GEMM term tables, once per structure.
//
// Each builder restates, as a table, which block pairs the reference multiplies and where
// the product lands.  Semantics follow MPShelpers/include/Block/BlockObj.hpp:2557-2625
// (BlockMat/BlockDiagMat products: lhs iterated in key order, rhs found by key),
// MPSBlockMat.hpp:934-1043 (MPS products), TMBlockFunctions.hpp (transfer matrices) and
// VUMPS/VUMPS_helpers.hpp (H_AC / H_C).  A product whose output sector is absent from the
// output object is dropped: in the reference it is inserted into a std::map of non-owning
// views and never reaches the caller's buffer (VUMPS_helpers.hpp:69-87).
#include <algorithm>
#include <cstring>

#include "imps_internal.h"
#include "imps_status.h"

namespace imps {

int layout_build(Layout& L, int nsym, int nblocks, const int32_t* qin, const int32_t* qout,
                 const int32_t* rows, const int32_t* cols, const int32_t* group) {
  if (nsym <= 0 || nsym > 8 || nblocks < 0) return IMPS_ERR_BAD_TABLE;
  L = Layout();
  L.nsym = nsym;
  L.blocks.resize(nblocks);
  int64_t off = 0;
  int maxg = 0;
  for (int b = 0; b < nblocks; ++b) {
    Block& B = L.blocks[b];
    B.qin.assign(qin + (int64_t)b * nsym, qin + (int64_t)(b + 1) * nsym);
    B.qout.assign(qout + (int64_t)b * nsym, qout + (int64_t)(b + 1) * nsym);
    B.rows = rows[b];
    B.cols = cols[b];
    B.group = group ? group[b] : 0;
    if (B.rows < 0 || B.cols < 0 || B.group < 0) return IMPS_ERR_BAD_TABLE;
    // std::map order: groups ascending, keys strictly increasing inside a group
    if (b > 0) {
      const Block& P = L.blocks[b - 1];
      if (B.group < P.group) return IMPS_ERR_BAD_TABLE;
      if (B.group == P.group && !(P.qin < B.qin)) return IMPS_ERR_BAD_TABLE;
    }
    B.off = off;
    off += (int64_t)B.rows * B.cols;
    maxg = std::max(maxg, B.group);
  }
  L.nelem = off;
  L.ngroups = maxg + 1;
  layout_index(L);
  return IMPS_OK;
}

void layout_index(Layout& L) {
  L.by_in.clear();
  L.by_out.clear();
  for (int b = 0; b < (int)L.blocks.size(); ++b) {
    const Block& B = L.blocks[b];
    L.by_in[{B.group, B.qin}] = b;
    L.by_out.emplace(std::make_pair(B.group, B.qout), b);
  }
}

// GetMl / GetMr of an MPS tensor as a BlockDiag layout (MPSBlockMat.hpp:281-326).
Layout layout_bond(const Layout& A, int side) {
  std::map<Key, int32_t> dims;
  for (const Block& B : A.blocks) {
    if (side == 0) dims.emplace(B.qin, B.rows);
    else dims.emplace(B.qout, B.cols);
  }
  Layout L;
  L.nsym = A.nsym;
  int64_t off = 0;
  for (auto& kv : dims) {
    Block B;
    B.qin = B.qout = kv.first;
    B.rows = B.cols = kv.second;
    B.off = off;
    off += (int64_t)B.rows * B.cols;
    L.blocks.push_back(B);
  }
  L.nelem = off;
  layout_index(L);
  return L;
}

namespace {

struct StageBuilder {
  Stage& S;
  OutBlock cur{};
  explicit StageBuilder(Stage& s) : S(s) {}
  void begin(int c_slot, int64_t c_off, int c_ld, int M, int N, int acc, int tag) {
    cur = OutBlock{};
    cur.c_slot = (int16_t)c_slot;
    cur.c_off = c_off;
    cur.c_ld = c_ld;
    cur.M = M;
    cur.N = N;
    cur.accumulate = (int16_t)acc;
    cur.tag = tag;
    cur.t0 = (int32_t)S.terms.size();
  }
  void term(int a_slot, int64_t a_off, int a_ld, int a_t, int b_slot, int64_t b_off, int b_ld,
            int b_t, int k, double alpha) {
    Term t{};
    t.a_off = a_off;
    t.b_off = b_off;
    t.a_ld = std::max(a_ld, 1);
    t.b_ld = std::max(b_ld, 1);
    t.k = k;
    t.a_slot = (int16_t)a_slot;
    t.b_slot = (int16_t)b_slot;
    t.a_t = (int8_t)a_t;
    t.b_t = (int8_t)b_t;
    t.alpha = alpha;
    S.terms.push_back(t);
    S.flops += 2LL * cur.M * cur.N * k;
  }
  void end() {
    cur.t1 = (int32_t)S.terms.size();
    S.outs.push_back(cur);
  }
};

int add_slot(Plan& P, int kind, int64_t nelem, const char* name) {
  Slot s;
  s.kind = kind;
  s.nelem = nelem;
  s.name = name;
  P.slots.push_back(s);
  return (int)P.slots.size() - 1;
}

bool square(const Block& B, int m) { return B.rows == m && B.cols == m; }

}  // namespace

void finalize_tiles(Stage& S, int tm, int tn) {
  S.tiles.clear();
  S.tile_m = tm;
  S.tile_n = tn;
  for (const OutBlock& o : S.outs) {
    for (int n0 = 0; n0 < o.N; n0 += tn)
      for (int m0 = 0; m0 < o.M; m0 += tm) {
        Tile t{};
        t.c_off = o.c_off;
        t.c_ld = std::max(o.c_ld, 1);
        t.m0 = m0;
        t.n0 = n0;
        t.mt = std::min(tm, o.M - m0);
        t.nt = std::min(tn, o.N - n0);
        t.t0 = o.t0;
        t.t1 = o.t1;
        t.c_slot = o.c_slot;
        t.accumulate = o.accumulate;
        t.nparts = 1;
        S.tiles.push_back(t);
      }
  }
}

// H_AC apply, ApplyHA (VUMPS_helpers.hpp:38-53) on the ApplyHAvec layout (:55-88):
//   out[i] = EHL*in[i] + in[i]*EHR + sum_j HL[i][j]*in[j] + in[j]*HR[i][j].
// Slots: 0 in, 1 out, 2 EHL, 3 EHR, 4 HL (RedOp, group i*d+j), 5 HR (RedOp).
int build_hac(Plan& P, const Layout& AC, const Layout& EHL, const Layout& EHR, const Layout& HL,
              const Layout& HR, int d) {
  P = Plan();
  P.kind = PLAN_HAC;
  int IN = add_slot(P, SLOT_EXTERNAL, AC.nelem, "in");
  int OUT = add_slot(P, SLOT_EXTERNAL, AC.nelem, "out");
  int SEHL = add_slot(P, SLOT_EXTERNAL, EHL.nelem, "EHL");
  int SEHR = add_slot(P, SLOT_EXTERNAL, EHR.nelem, "EHR");
  int SHL = add_slot(P, SLOT_EXTERNAL, HL.nelem, "HL");
  int SHR = add_slot(P, SLOT_EXTERNAL, HR.nelem, "HR");
  P.n_in = IN;
  P.n_out = OUT;
  P.stages.emplace_back();
  StageBuilder sb(P.stages.back());
  for (int bi = 0; bi < (int)AC.blocks.size(); ++bi) {
    const Block& b = AC.blocks[bi];
    const int s = b.group, ml = b.rows, mr = b.cols;
    if (s >= d) return IMPS_ERR_BAD_TABLE;
    sb.begin(OUT, b.off, ml, ml, mr, 0, bi);
    int e = EHL.find_in(0, b.qin);  // BlockDiagMat * BlockMat (BlockObj.hpp:2591-2610)
    if (e >= 0) {
      if (!square(EHL.blocks[e], ml)) return IMPS_ERR_BAD_TABLE;
      sb.term(SEHL, EHL.blocks[e].off, ml, 0, IN, b.off, ml, 0, ml, 1.0);
    }
    e = EHR.find_in(0, b.qout);  // BlockMat * BlockDiagMat (BlockObj.hpp:2570-2589)
    if (e >= 0) {
      if (!square(EHR.blocks[e], mr)) return IMPS_ERR_BAD_TABLE;
      sb.term(IN, b.off, ml, 0, SEHR, EHR.blocks[e].off, mr, 0, mr, 1.0);
    }
    for (int j = 0; j < d; ++j) {
      // HL[i][j]*in[j]: HL block keyed Qin=ql, in[j] block found by HL's Qout
      int h = HL.find_in(s * d + j, b.qin);
      if (h >= 0) {
        const Block& H = HL.blocks[h];
        int x = AC.find_in(j, H.qout);
        if (x >= 0) {
          const Block& X = AC.blocks[x];
          if (X.qout != b.qout) {
            ++P.dropped;
          } else {
            if (H.rows != ml || H.cols != X.rows || X.cols != mr) return IMPS_ERR_BAD_TABLE;
            sb.term(SHL, H.off, H.rows, 0, IN, X.off, X.rows, 0, H.cols, 1.0);
          }
        }
      }
      // in[j]*HR[i][j]: in[j] block keyed Qin=ql, HR block found by in[j]'s Qout
      int x = AC.find_in(j, b.qin);
      if (x >= 0) {
        const Block& X = AC.blocks[x];
        int hr = HR.find_in(s * d + j, X.qout);
        if (hr >= 0) {
          const Block& H = HR.blocks[hr];
          if (H.qout != b.qout) {
            ++P.dropped;
          } else {
            if (X.rows != ml || H.rows != X.cols || H.cols != mr) return IMPS_ERR_BAD_TABLE;
            sb.term(IN, X.off, ml, 0, SHR, H.off, H.rows, 0, X.cols, 1.0);
          }
        }
      }
    }
    sb.end();
  }
  (void)SHR;
  P.flops_apply = P.stages[0].flops;
  return IMPS_OK;
}

// Transfer-matrix chain over a unit cell (TMBlockFunctions.hpp:33-56, 155-177, chains
// :557-563 / :600-606).  dir 0 = left (sites in order, out = sum_s A_s^T X A_s),
// dir 1 = right (sites reversed, out = sum_s A_s X A_s^T).  Each site is two stages:
// W_b = X*A_b (left) or A_b*X (right), then the per-sector reduction into the next bond.
// Slots: 0 in, 1 out, 2..2+n-1 A[k]; internal scratch W_k and intermediate bonds.
int build_tm(Plan& P, const std::vector<const Layout*>& A, int dir, const Layout& in,
             const Layout& out) {
  P = Plan();
  P.kind = PLAN_TM;
  const int n = (int)A.size();
  if (n < 1) return IMPS_ERR_BAD_ARG;
  int IN = add_slot(P, SLOT_EXTERNAL, in.nelem, "in");
  int OUT = add_slot(P, SLOT_EXTERNAL, out.nelem, "out");
  std::vector<int> SA(n), SW(n);
  for (int k = 0; k < n; ++k) SA[k] = add_slot(P, SLOT_EXTERNAL, A[k]->nelem, "A");
  for (int k = 0; k < n; ++k) SW[k] = add_slot(P, SLOT_INTERNAL, A[k]->nelem, "W");
  P.n_in = IN;
  P.n_out = OUT;
  // intermediate bonds
  std::vector<Layout> mids;
  std::vector<int> SM;
  for (int step = 0; step < n - 1; ++step) {
    int k = dir == 0 ? step : n - 1 - step;
    mids.push_back(layout_bond(*A[k], dir == 0 ? 1 : 0));
    SM.push_back(add_slot(P, SLOT_INTERNAL, mids.back().nelem, "Y"));
  }
  const Layout* cur = &in;
  int cur_slot = IN;
  for (int step = 0; step < n; ++step) {
    const int k = dir == 0 ? step : n - 1 - step;
    const Layout& Ak = *A[k];
    const Layout* O = step == n - 1 ? &out : &mids[step];
    const int o_slot = step == n - 1 ? OUT : SM[step];
    // stage 1: W_b
    P.stages.emplace_back();
    {
      StageBuilder sb(P.stages.back());
      for (int bi = 0; bi < (int)Ak.blocks.size(); ++bi) {
        const Block& b = Ak.blocks[bi];
        sb.begin(SW[k], b.off, b.rows, b.rows, b.cols, 0, bi);
        if (dir == 0) {
          int x = cur->find_in(0, b.qin);
          if (x >= 0) {
            if (!square(cur->blocks[x], b.rows)) return IMPS_ERR_BAD_TABLE;
            sb.term(cur_slot, cur->blocks[x].off, b.rows, 0, SA[k], b.off, b.rows, 0, b.rows, 1.0);
          }
        } else {
          int x = cur->find_in(0, b.qout);
          if (x >= 0) {
            if (!square(cur->blocks[x], b.cols)) return IMPS_ERR_BAD_TABLE;
            sb.term(SA[k], b.off, b.rows, 0, cur_slot, cur->blocks[x].off, b.cols, 0, b.cols, 1.0);
          }
        }
        sb.end();
      }
    }
    // stage 2: reduction into the output bond
    P.stages.emplace_back();
    {
      StageBuilder sb(P.stages.back());
      for (int oi = 0; oi < (int)O->blocks.size(); ++oi) {
        const Block& o = O->blocks[oi];
        sb.begin(o_slot, o.off, o.rows, o.rows, o.cols, 0, oi);
        for (int g = 0; g < Ak.ngroups; ++g) {
          if (dir == 0) {
            int bi = Ak.find_out(g, o.qin);
            if (bi < 0) continue;
            const Block& b = Ak.blocks[bi];
            if (cur->find_in(0, b.qin) < 0) continue;
            if (b.cols != o.rows) return IMPS_ERR_BAD_TABLE;
            sb.term(SA[k], b.off, b.rows, 1, SW[k], b.off, b.rows, 0, b.rows, 1.0);
          } else {
            int bi = Ak.find_in(g, o.qin);
            if (bi < 0) continue;
            const Block& b = Ak.blocks[bi];
            if (cur->find_in(0, b.qout) < 0) continue;
            if (b.rows != o.rows) return IMPS_ERR_BAD_TABLE;
            sb.term(SW[k], b.off, b.rows, 0, SA[k], b.off, b.rows, 1, b.cols, 1.0);
          }
        }
        sb.end();
      }
    }
    cur = O;
    cur_slot = o_slot;
  }
  P.derived = mids;
  for (auto& st : P.stages) P.flops_apply += st.flops;
  return IMPS_OK;
}

// Mixed transfer matrix of two unit cells on a general BlockMat X (one block per Qin, a
// fixed charge offset):
//   dir 0 (left, sites in order):   out(Qout(B_s) -> Qout(A_s)) += B_s^T X(Qin(B_s) -> Qin(A_s)) A_s
//   dir 1 (right, sites reversed):  out(Qin(A_s) -> Qin(B_s))   += A_s X(Qout(A_s) -> Qout(B_s)) B_s^T
// (TMBlockFunctions.hpp:336-344 / 474-482 as in*A resp. A*in followed by the mixed product
// with B, chained over the unit cell at :669-676 / :737-744).  A is the lower layer, B the
// upper one.  Two stages per site: W = X_x A_a (left) or A_a X_x (right) for every matched
// (block of X, physical index) pair, then the output blocks sum B^T W (left) or W B^T
// (right) over their pairs.  Products whose output sector is absent from `out` are counted
// in `dropped` (the reference prints "not present" and skips them, :380-384, 521-525).
// Slots: 0 in, 1 out, 2..n+1 A_k, n+2..2n+1 B_k, then internal scratch.
int build_tm_mixed(Plan& P, const std::vector<const Layout*>& A, const std::vector<const Layout*>& B,
                   int dir, const Layout& in, const Layout& out) {
  P = Plan();
  P.kind = dir == 0 ? PLAN_TMMIXED_L : PLAN_TMMIXED_R;
  const int n = (int)A.size();
  if (n < 1 || (int)B.size() != n) return IMPS_ERR_BAD_ARG;
  const int IN = add_slot(P, SLOT_EXTERNAL, in.nelem, "in");
  const int OUT = add_slot(P, SLOT_EXTERNAL, out.nelem, "out");
  std::vector<int> SA(n), SB(n);
  for (int k = 0; k < n; ++k) SA[k] = add_slot(P, SLOT_EXTERNAL, A[k]->nelem, "A");
  for (int k = 0; k < n; ++k) SB[k] = add_slot(P, SLOT_EXTERNAL, B[k]->nelem, "B");
  P.n_in = IN;
  P.n_out = OUT;
  struct Pair { int x, a, b; int64_t woff; Key oin, oout; int orows, ocols; };
  std::vector<Layout> mids;
  const Layout* cur = &in;
  int cur_slot = IN;
  for (int step = 0; step < n; ++step) {
    const int k = dir == 0 ? step : n - 1 - step;
    const Layout& LA = *A[k];
    const Layout& LB = *B[k];
    if (LA.ngroups != LB.ngroups) return IMPS_ERR_BAD_TABLE;
    // matched pairs and their scratch
    std::vector<Pair> pairs;
    int64_t woff = 0;
    for (int xi = 0; xi < (int)cur->blocks.size(); ++xi) {
      const Block& x = cur->blocks[xi];
      for (int g = 0; g < LA.ngroups; ++g) {
        const int a = dir == 0 ? LA.find_in(g, x.qout) : LA.find_out(g, x.qin);
        const int b = dir == 0 ? LB.find_in(g, x.qin) : LB.find_out(g, x.qout);
        if (a < 0 || b < 0) continue;
        const Block& ba = LA.blocks[a];
        const Block& bb = LB.blocks[b];
        Pair pr{xi, a, b, woff, {}, {}, 0, 0};
        if (dir == 0) {
          if (x.cols != ba.rows || x.rows != bb.rows) return IMPS_ERR_BAD_TABLE;
          pr.oin = bb.qout; pr.oout = ba.qout; pr.orows = bb.cols; pr.ocols = ba.cols;
          woff += (int64_t)x.rows * ba.cols;
        } else {
          if (ba.cols != x.rows || x.cols != bb.cols) return IMPS_ERR_BAD_TABLE;
          pr.oin = ba.qin; pr.oout = bb.qin; pr.orows = ba.rows; pr.ocols = bb.rows;
          woff += (int64_t)ba.rows * x.cols;
        }
        pairs.push_back(pr);
      }
    }
    const int SW = add_slot(P, SLOT_INTERNAL, std::max<int64_t>(woff, 1), "W");
    // output layout of this step: the given one, or derived from the pairs (std::map order)
    const bool last = step == n - 1;
    if (!last) {
      std::map<Key, std::pair<Key, std::pair<int, int>>> keys;
      for (const Pair& pr : pairs) {
        auto it = keys.find(pr.oin);
        if (it == keys.end()) keys.emplace(pr.oin, std::make_pair(pr.oout, std::make_pair(pr.orows, pr.ocols)));
        else if (it->second.first != pr.oout || it->second.second != std::make_pair(pr.orows, pr.ocols))
          return IMPS_ERR_BAD_TABLE;  // not a BlockMat: two outgoing charges for one incoming
      }
      Layout M;
      M.nsym = in.nsym;
      int64_t off = 0;
      for (auto& kv : keys) {
        Block bl;
        bl.qin = kv.first;
        bl.qout = kv.second.first;
        bl.rows = kv.second.second.first;
        bl.cols = kv.second.second.second;
        bl.off = off;
        off += (int64_t)bl.rows * bl.cols;
        M.blocks.push_back(bl);
      }
      M.nelem = off;
      layout_index(M);
      mids.push_back(M);
    }
    const Layout* O = last ? &out : &mids.back();
    const int o_slot = last ? OUT : add_slot(P, SLOT_INTERNAL, std::max<int64_t>(O->nelem, 1), "Y");
    // stage 1: W
    P.stages.emplace_back();
    {
      StageBuilder sb(P.stages.back());
      for (int pi = 0; pi < (int)pairs.size(); ++pi) {
        const Pair& pr = pairs[pi];
        const Block& x = cur->blocks[pr.x];
        const Block& ba = LA.blocks[pr.a];
        if (dir == 0) {
          sb.begin(SW, pr.woff, x.rows, x.rows, ba.cols, 0, pi);
          sb.term(cur_slot, x.off, x.rows, 0, SA[k], ba.off, ba.rows, 0, x.cols, 1.0);
        } else {
          sb.begin(SW, pr.woff, ba.rows, ba.rows, x.cols, 0, pi);
          sb.term(SA[k], ba.off, ba.rows, 0, cur_slot, x.off, x.rows, 0, x.rows, 1.0);
        }
        sb.end();
      }
    }
    // stage 2: output blocks
    P.stages.emplace_back();
    {
      StageBuilder sb(P.stages.back());
      std::vector<int> used(pairs.size(), 0);
      for (int oi = 0; oi < (int)O->blocks.size(); ++oi) {
        const Block& o = O->blocks[oi];
        sb.begin(o_slot, o.off, o.rows, o.rows, o.cols, 0, oi);
        for (int pi = 0; pi < (int)pairs.size(); ++pi) {
          const Pair& pr = pairs[pi];
          if (pr.oin != o.qin) continue;
          if (pr.oout != o.qout || pr.orows != o.rows || pr.ocols != o.cols) return IMPS_ERR_BAD_TABLE;
          used[pi] = 1;
          const Block& x = cur->blocks[pr.x];
          const Block& bb = LB.blocks[pr.b];
          if (dir == 0)  // out += B_b^T W
            sb.term(SB[k], bb.off, bb.rows, 1, SW, pr.woff, x.rows, 0, x.rows, 1.0);
          else  // out += W B_b^T
            sb.term(SW, pr.woff, o.rows, 0, SB[k], bb.off, bb.rows, 1, x.cols, 1.0);
        }
        sb.end();
      }
      for (int u : used) P.dropped += u ? 0 : 1;
    }
    cur = O;
    cur_slot = o_slot;
  }
  P.derived = mids;
  for (auto& st : P.stages) P.flops_apply += st.flops;
  return IMPS_OK;
}

// ReducedOp (MPSBlockUtilities.hpp:37-74).  dir 0 (l): HL[i1][j1] += h * A[i0]^T * A[j0];
// dir 1 (r): HR[i0][j0] += h * A[j1] * A[i1]^T.  The output RedOp layout (group i*d+j,
// BlockMat key order) is derived here.  Slots: 0 A, 1 out.
int build_redop(Plan& P, const Layout& A, int d, const std::vector<HNnz>& h, int dir) {
  P = Plan();
  P.kind = PLAN_REDOP;
  struct OB { Key qout; int rows, cols; std::vector<Term> terms; };
  std::map<std::pair<int, Key>, OB> outs;
  const int SAs = 0, SOUT = 1;
  for (const HNnz& z : h) {
    const int i0 = z.r / d, i1 = z.r % d, j0 = z.c / d, j1 = z.c % d;
    if (dir == 0) {
      const int g = i1 * d + j1;
      for (const Block& a : A.blocks) {
        if (a.group != i0) continue;
        int bj = A.find_in(j0, a.qin);
        if (bj < 0) continue;
        const Block& b = A.blocks[bj];
        auto key = std::make_pair(g, a.qout);
        auto it = outs.find(key);
        if (it == outs.end()) it = outs.emplace(key, OB{b.qout, a.cols, b.cols, {}}).first;
        else if (it->second.qout != b.qout) return IMPS_ERR_BAD_TABLE;
        Term t{};
        t.a_slot = SAs; t.a_off = a.off; t.a_ld = std::max(a.rows, 1); t.a_t = 1;
        t.b_slot = SAs; t.b_off = b.off; t.b_ld = std::max(b.rows, 1); t.b_t = 0;
        t.k = a.rows; t.alpha = z.v;
        it->second.terms.push_back(t);
      }
    } else {
      const int g = i0 * d + j0;
      for (const Block& b : A.blocks) {
        if (b.group != j1) continue;
        int ai = A.find_out(i1, b.qout);
        if (ai < 0) continue;
        const Block& a = A.blocks[ai];
        auto key = std::make_pair(g, b.qin);
        auto it = outs.find(key);
        if (it == outs.end()) it = outs.emplace(key, OB{a.qin, b.rows, a.rows, {}}).first;
        else if (it->second.qout != a.qin) return IMPS_ERR_BAD_TABLE;
        Term t{};
        t.a_slot = SAs; t.a_off = b.off; t.a_ld = std::max(b.rows, 1); t.a_t = 0;
        t.b_slot = SAs; t.b_off = a.off; t.b_ld = std::max(a.rows, 1); t.b_t = 1;
        t.k = b.cols; t.alpha = z.v;
        it->second.terms.push_back(t);
      }
    }
  }
  Layout R;
  R.nsym = A.nsym;
  int64_t off = 0;
  int maxg = 0;
  for (auto& kv : outs) {
    Block B;
    B.group = kv.first.first;
    B.qin = kv.first.second;
    B.qout = kv.second.qout;
    B.rows = kv.second.rows;
    B.cols = kv.second.cols;
    B.off = off;
    off += (int64_t)B.rows * B.cols;
    maxg = std::max(maxg, B.group);
    R.blocks.push_back(B);
  }
  R.nelem = off;
  R.ngroups = std::max(maxg + 1, d * d);
  layout_index(R);
  add_slot(P, SLOT_EXTERNAL, A.nelem, "A");
  add_slot(P, SLOT_EXTERNAL, R.nelem, "out");
  P.n_in = 0;
  P.n_out = SOUT;
  P.stages.emplace_back();
  Stage& S = P.stages.back();
  int bi = 0;
  for (auto& kv : outs) {
    const Block& B = R.blocks[bi];
    OutBlock o{};
    o.c_slot = SOUT;
    o.c_off = B.off;
    o.c_ld = std::max(B.rows, 1);
    o.M = B.rows;
    o.N = B.cols;
    o.t0 = (int32_t)S.terms.size();
    for (const Term& t : kv.second.terms) {
      S.terms.push_back(t);
      S.flops += 2LL * B.rows * B.cols * t.k;
    }
    o.t1 = (int32_t)S.terms.size();
    o.accumulate = 0;
    o.tag = bi++;
    S.outs.push_back(o);
  }
  P.derived.push_back(R);
  P.flops_apply = S.flops;
  return IMPS_OK;
}

// 2-site product AA = A0*A1 (MPSBlockMat.hpp:934-947) followed by the operator transfer
// matrix on it: dir 0: ApplyOpTMLeftDiag (TMBlockFunctions.hpp:797-802) = sum_{h_ij}
// h * AA_i^T AA_j; dir 1: ApplyOpTMRightDiag (:831-836) = sum_{h_ij} h * AA_j AA_i^T.
// Slots: 0 A0, 1 A1, 2 out (BlockDiag), 3 AA (internal, derived layout 0).
int build_optm(Plan& P, const Layout& A0, const Layout& A1, int d, const std::vector<HNnz>& h,
               int dir, const Layout& out) {
  P = Plan();
  P.kind = PLAN_OPTM;
  Layout AA;
  AA.nsym = A0.nsym;
  struct Pair { int a, b; };
  std::vector<Pair> prs;
  int64_t off = 0;
  for (int s0 = 0; s0 < d; ++s0)
    for (int s1 = 0; s1 < d; ++s1) {
      for (int ai = 0; ai < (int)A0.blocks.size(); ++ai) {
        const Block& a = A0.blocks[ai];
        if (a.group != s0) continue;
        int bi = A1.find_in(s1, a.qout);
        if (bi < 0) continue;
        const Block& b = A1.blocks[bi];
        if (b.rows != a.cols) return IMPS_ERR_BAD_TABLE;
        Block B;
        B.group = s0 * d + s1;
        B.qin = a.qin;
        B.qout = b.qout;
        B.rows = a.rows;
        B.cols = b.cols;
        B.off = off;
        off += (int64_t)B.rows * B.cols;
        AA.blocks.push_back(B);
        prs.push_back({ai, bi});
      }
    }
  AA.nelem = off;
  AA.ngroups = d * d;
  layout_index(AA);
  const int S0 = add_slot(P, SLOT_EXTERNAL, A0.nelem, "A0");
  const int S1 = add_slot(P, SLOT_EXTERNAL, A1.nelem, "A1");
  const int SOUT = add_slot(P, SLOT_EXTERNAL, out.nelem, "out");
  const int SAA = add_slot(P, SLOT_INTERNAL, AA.nelem, "AA");
  P.n_in = S0;
  P.n_out = SOUT;
  P.stages.emplace_back();
  {
    StageBuilder sb(P.stages.back());
    for (int i = 0; i < (int)AA.blocks.size(); ++i) {
      const Block& B = AA.blocks[i];
      const Block& a = A0.blocks[prs[i].a];
      const Block& b = A1.blocks[prs[i].b];
      sb.begin(SAA, B.off, B.rows, B.rows, B.cols, 0, i);
      sb.term(S0, a.off, a.rows, 0, S1, b.off, b.rows, 0, a.cols, 1.0);
      sb.end();
    }
  }
  P.stages.emplace_back();
  {
    StageBuilder sb(P.stages.back());
    for (int oi = 0; oi < (int)out.blocks.size(); ++oi) {
      const Block& o = out.blocks[oi];
      sb.begin(SOUT, o.off, o.rows, o.rows, o.cols, 0, oi);
      for (const HNnz& z : h) {
        const int i = z.r, j = z.c;
        if (dir == 0) {
          int ai = AA.find_out(i, o.qin);
          if (ai < 0) continue;
          const Block& a = AA.blocks[ai];
          int bj = AA.find_in(j, a.qin);
          if (bj < 0) continue;
          const Block& b = AA.blocks[bj];
          if (b.qout != a.qout) return IMPS_ERR_BAD_TABLE;
          sb.term(SAA, a.off, a.rows, 1, SAA, b.off, b.rows, 0, a.rows, z.v);
        } else {
          int ai = AA.find_in(i, o.qin);
          int bj = AA.find_in(j, o.qin);
          if (ai < 0 || bj < 0) continue;
          const Block& a = AA.blocks[ai];
          const Block& b = AA.blocks[bj];
          if (b.qout != a.qout) return IMPS_ERR_BAD_TABLE;
          sb.term(SAA, b.off, b.rows, 0, SAA, a.off, a.rows, 1, a.cols, z.v);
        }
      }
      sb.end();
    }
  }
  P.derived.push_back(AA);
  for (auto& st : P.stages) P.flops_apply += st.flops;
  return IMPS_OK;
}

// MPS x BlockDiagMat products (MPSBlockMat.hpp:1021-1043 via BlockObj.hpp:2570-2610).
// side 1: out_s = alpha * A_s * op(X); side 0: out_s = alpha * op(X) * A_s, where
// op(X) = X (xt=0) or X^T (xt=1, encoded in alpha's sign bit? no: separate flag below).
// Slots: 0 A, 1 X, 2 out (A's layout; blocks without an X sector are written as zero).
int build_mps_bd(Plan& P, const Layout& A, const Layout& X, int side, double alpha) {
  P = Plan();
  P.kind = side ? PLAN_MPS_BD : PLAN_BD_MPS;
  const int xt = (side >> 1) & 1;
  side &= 1;
  const int SA_ = add_slot(P, SLOT_EXTERNAL, A.nelem, "A");
  const int SX = add_slot(P, SLOT_EXTERNAL, X.nelem, "X");
  const int SOUT = add_slot(P, SLOT_EXTERNAL, A.nelem, "out");
  P.n_in = SA_;
  P.n_out = SOUT;
  P.stages.emplace_back();
  StageBuilder sb(P.stages.back());
  for (int bi = 0; bi < (int)A.blocks.size(); ++bi) {
    const Block& b = A.blocks[bi];
    sb.begin(SOUT, b.off, b.rows, b.rows, b.cols, 0, bi);
    if (side == 1) {
      int x = X.find_in(0, b.qout);
      if (x >= 0) {
        if (!square(X.blocks[x], b.cols)) return IMPS_ERR_BAD_TABLE;
        sb.term(SA_, b.off, b.rows, 0, SX, X.blocks[x].off, b.cols, xt, b.cols, alpha);
      } else {
        ++P.dropped;
      }
    } else {
      int x = X.find_in(0, b.qin);
      if (x >= 0) {
        if (!square(X.blocks[x], b.rows)) return IMPS_ERR_BAD_TABLE;
        sb.term(SX, X.blocks[x].off, b.rows, xt, SA_, b.off, b.rows, 0, b.rows, alpha);
      } else {
        ++P.dropped;
      }
    }
    sb.end();
  }
  P.flops_apply = P.stages[0].flops;
  return IMPS_OK;
}

// Tangent-space gradient of GradNormRight (VUMPS_helpers.hpp:145-153) without forming the
// null space: for N_R with N_R^T N_R = 1 - A_R^T A_R (per left sector, in the dense right
// representation of MPSBlockMat.hpp:636-719), |Y N_R^T|_F = |Y - (Y A_R^T) A_R|_F.
// Stage 0: dC(q) = sum_s Y_s(q) A_R,s(q)^T (ApplyTMmixedRight with B = A_R, :445-473);
// stage 1: G = Y - dC * A_R (G pre-initialised with a copy of Y).
// Slots: 0 Y, 1 AR, 2 G (AR layout, output), 3 dC (internal, derived layout 0).
int build_grad_right(Plan& P, const Layout& Y, const Layout& AR) {
  P = Plan();
  P.kind = PLAN_GRAD;
  Layout bond = layout_bond(AR, 0);
  const int SY = add_slot(P, SLOT_EXTERNAL, Y.nelem, "Y");
  const int SAR = add_slot(P, SLOT_EXTERNAL, AR.nelem, "AR");
  const int SG = add_slot(P, SLOT_EXTERNAL, AR.nelem, "G");
  const int SDC = add_slot(P, SLOT_INTERNAL, bond.nelem, "dC");
  P.n_in = SY;
  P.n_out = SG;
  if (Y.nelem != AR.nelem || Y.blocks.size() != AR.blocks.size()) return IMPS_ERR_BAD_TABLE;
  P.stages.emplace_back();
  {
    StageBuilder sb(P.stages.back());
    for (int oi = 0; oi < (int)bond.blocks.size(); ++oi) {
      const Block& o = bond.blocks[oi];
      sb.begin(SDC, o.off, o.rows, o.rows, o.cols, 0, oi);
      for (int g = 0; g < AR.ngroups; ++g) {
        int y = Y.find_in(g, o.qin), a = AR.find_in(g, o.qin);
        if (y < 0 || a < 0) continue;
        const Block& Yb = Y.blocks[y];
        const Block& Ab = AR.blocks[a];
        if (Yb.qout != Ab.qout || Yb.cols != Ab.cols) return IMPS_ERR_BAD_TABLE;
        sb.term(SY, Yb.off, Yb.rows, 0, SAR, Ab.off, Ab.rows, 1, Ab.cols, 1.0);
      }
      sb.end();
    }
  }
  P.stages.emplace_back();
  {
    StageBuilder sb(P.stages.back());
    for (int bi = 0; bi < (int)AR.blocks.size(); ++bi) {
      const Block& b = AR.blocks[bi];
      int x = bond.find_in(0, b.qin);
      sb.begin(SG, b.off, b.rows, b.rows, b.cols, 1, bi);
      sb.term(SDC, bond.blocks[x].off, b.rows, 0, SAR, b.off, b.rows, 0, b.rows, -1.0);
      sb.end();
    }
  }
  P.derived.push_back(bond);
  for (auto& st : P.stages) P.flops_apply += st.flops;
  return IMPS_OK;
}

// H_C apply, ApplyHC (VUMPS_helpers.hpp:91-111), restructured: for every nonzero h of the
// two-site operator the reference forms h * AL[i0]^T AL[j0] * C * AR[j1] AR[i1]^T.  Grouping
// the nonzeros by (i1, j1) gives
//   out = EHL*C + C*EHR + sum_{(i1,j1)} HLp[i1][j1] * C * Rr[j1][i1],
// HLp = ReducedOp(h, AL, l) and Rr[j1][i1] = AR[j1] AR[i1]^T (operator-dependent, computed
// by the prepare stages).  Slots: 0 in, 1 out, 2 EHL, 3 EHR, 4 AL, 5 AR, 6 HLp, 7 Rr, 8 W.
int build_hc(Plan& P, const Layout& C, const Layout& EHL, const Layout& EHR, const Layout& AL,
             const Layout& AR, int d, const std::vector<HNnz>& h) {
  Plan R;
  int rc = build_redop(R, AL, d, h, 0);
  if (rc) return rc;
  const Layout HLp = R.derived[0];
  // pairs (i1, j1) present, and Rr[j1][i1] = AR[j1] * AR[i1]^T layout (group j1*d+i1)
  std::vector<int> pair_present(d * d, 0);
  for (const HNnz& z : h) pair_present[(z.r % d) * d + (z.c % d)] = 1;
  struct OB { Key qout; int rows, cols; std::vector<std::pair<int, int>> ab; };
  std::map<std::pair<int, Key>, OB> rr;
  for (int i1 = 0; i1 < d; ++i1)
    for (int j1 = 0; j1 < d; ++j1) {
      if (!pair_present[i1 * d + j1]) continue;
      const int g = j1 * d + i1;
      for (int bi = 0; bi < (int)AR.blocks.size(); ++bi) {
        const Block& b = AR.blocks[bi];
        if (b.group != j1) continue;
        int ai = AR.find_out(i1, b.qout);
        if (ai < 0) continue;
        const Block& a = AR.blocks[ai];
        rr[{g, b.qin}] = OB{a.qin, b.rows, a.rows, {{bi, ai}}};
      }
    }
  Layout RR;
  RR.nsym = C.nsym;
  int64_t off = 0;
  for (auto& kv : rr) {
    Block B;
    B.group = kv.first.first;
    B.qin = kv.first.second;
    B.qout = kv.second.qout;
    B.rows = kv.second.rows;
    B.cols = kv.second.cols;
    B.off = off;
    off += (int64_t)B.rows * B.cols;
    RR.blocks.push_back(B);
  }
  RR.nelem = off;
  RR.ngroups = d * d;
  layout_index(RR);
  // W[(i1,j1)](q' -> q'') = C(q') * Rr[j1][i1](q' -> q'') ; layout keyed like Rr (group j1*d+i1)
  const Layout& W = RR;

  P = Plan();
  P.kind = PLAN_HC;
  const int IN = add_slot(P, SLOT_EXTERNAL, C.nelem, "in");
  const int OUT = add_slot(P, SLOT_EXTERNAL, C.nelem, "out");
  const int SEHL = add_slot(P, SLOT_EXTERNAL, EHL.nelem, "EHL");
  const int SEHR = add_slot(P, SLOT_EXTERNAL, EHR.nelem, "EHR");
  const int SAL = add_slot(P, SLOT_EXTERNAL, AL.nelem, "AL");
  const int SAR = add_slot(P, SLOT_EXTERNAL, AR.nelem, "AR");
  const int SHLP = add_slot(P, SLOT_INTERNAL, HLp.nelem, "HLp");
  const int SRR = add_slot(P, SLOT_INTERNAL, RR.nelem, "Rr");
  const int SW = add_slot(P, SLOT_INTERNAL, W.nelem, "W");
  P.n_in = IN;
  P.n_out = OUT;
  // prepare stage 0: HLp = ReducedOp(h, AL, l) (slot remap 0->AL, 1->HLp)
  {
    Stage S = R.stages[0];
    for (Term& t : S.terms) { t.a_slot = SAL; t.b_slot = SAL; }
    for (OutBlock& o : S.outs) o.c_slot = SHLP;
    P.prep.push_back(S);
  }
  // prepare stage 1: Rr
  P.prep.emplace_back();
  {
    StageBuilder sb(P.prep.back());
    int bi = 0;
    for (auto& kv : rr) {
      const Block& B = RR.blocks[bi];
      const Block& b = AR.blocks[kv.second.ab[0].first];
      const Block& a = AR.blocks[kv.second.ab[0].second];
      sb.begin(SRR, B.off, B.rows, B.rows, B.cols, 0, bi);
      sb.term(SAR, b.off, b.rows, 0, SAR, a.off, a.rows, 1, b.cols, 1.0);
      sb.end();
      ++bi;
    }
  }
  // apply stage 0: W = C * Rr
  P.stages.emplace_back();
  {
    StageBuilder sb(P.stages.back());
    for (int wi = 0; wi < (int)W.blocks.size(); ++wi) {
      const Block& w = W.blocks[wi];
      sb.begin(SW, w.off, w.rows, w.rows, w.cols, 0, wi);
      int c = C.find_in(0, w.qin);
      if (c >= 0) {
        if (!square(C.blocks[c], w.rows)) return IMPS_ERR_BAD_TABLE;
        sb.term(IN, C.blocks[c].off, w.rows, 0, SRR, RR.blocks[wi].off, w.rows, 0, w.rows, 1.0);
      }
      sb.end();
    }
  }
  // apply stage 1: out = EHL*C + C*EHR + sum_p HLp[p] * W[p]
  P.stages.emplace_back();
  {
    StageBuilder sb(P.stages.back());
    for (int ci = 0; ci < (int)C.blocks.size(); ++ci) {
      const Block& c = C.blocks[ci];
      const int m = c.rows;
      sb.begin(OUT, c.off, m, m, m, 0, ci);
      int e = EHL.find_in(0, c.qin);
      if (e >= 0) {
        if (!square(EHL.blocks[e], m)) return IMPS_ERR_BAD_TABLE;
        sb.term(SEHL, EHL.blocks[e].off, m, 0, IN, c.off, m, 0, m, 1.0);
      }
      e = EHR.find_in(0, c.qin);
      if (e >= 0) {
        if (!square(EHR.blocks[e], m)) return IMPS_ERR_BAD_TABLE;
        sb.term(IN, c.off, m, 0, SEHR, EHR.blocks[e].off, m, 0, m, 1.0);
      }
      for (int i1 = 0; i1 < d; ++i1)
        for (int j1 = 0; j1 < d; ++j1) {
          if (!pair_present[i1 * d + j1]) continue;
          int hl = HLp.find_in(i1 * d + j1, c.qin);
          if (hl < 0) continue;
          const Block& H = HLp.blocks[hl];
          int w = W.find_in(j1 * d + i1, H.qout);
          if (w < 0) continue;
          const Block& Wb = W.blocks[w];
          if (Wb.qout != c.qin) { ++P.dropped; continue; }
          if (H.rows != m || Wb.rows != H.cols || Wb.cols != m) return IMPS_ERR_BAD_TABLE;
          sb.term(SHLP, H.off, m, 0, SW, Wb.off, Wb.rows, 0, H.cols, 1.0);
        }
      sb.end();
    }
  }
  P.derived.push_back(HLp);
  P.derived.push_back(RR);
  for (auto& st : P.stages) P.flops_apply += st.flops;
  for (auto& st : P.prep) P.flops_prep += st.flops;
  return IMPS_OK;
}

}  // namespace imps
