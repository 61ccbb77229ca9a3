// Sector tables for the per-sector dense decompositions: the integer part of
// MPSBlockMat::GetSingleSecData / GetDenseMat (MPSBlockMat.hpp:468-526, 636-719).
//   dir l: one dense matrix per outgoing charge (right sector), blocks of A_s stacked by
//          rows in increasing s  -> (sum_s ml_s) x mr
//   dir r: one dense matrix per incoming charge (left sector), blocks stacked by columns
//          in increasing s -> ml x (sum_s mr_s); stored transposed so that M >= N.
// A BlockDiagMat is the d = 1 case.
#include <algorithm>
#include <map>

#include "imps_decomp.h"
#include "imps_status.h"

namespace imps {

int build_decomp(DecompPlan& D, const Layout& A, int dir) {
  D = DecompPlan();
  D.dir = dir;
  struct Sec { int n = -1; int m = 0; std::vector<int> blocks; };
  std::map<Key, Sec> secs;
  // blocks in (group, key) order = increasing s, as the reference's v_phys_ind
  for (int g = 0; g < A.ngroups; ++g)
    for (int b = 0; b < (int)A.blocks.size(); ++b) {
      const Block& B = A.blocks[b];
      if (B.group != g) continue;
      const Key& k = dir == 0 ? B.qout : B.qin;
      Sec& s = secs[k];
      const int n = dir == 0 ? B.cols : B.rows;
      if (s.n >= 0 && s.n != n) return IMPS_ERR_BAD_TABLE;
      s.n = n;
      s.m += dir == 0 ? B.rows : B.cols;
      s.blocks.push_back(b);
    }
  int64_t a = 0, r = 0, sv = 0, w = 0;
  D.rlayout = Layout();
  D.rlayout.nsym = A.nsym;
  for (auto& kv : secs) {
    Sec& s = kv.second;
    if (s.n > 512 || s.m > (1 << 20)) return IMPS_ERR_UNSUPPORTED;
    DenseMat mt{};
    mt.M = s.m;
    mt.N = s.n;
    if (mt.M < mt.N) D.tall = false;
    mt.a_off = a;
    mt.q_off = a;
    mt.r_off = r;
    mt.s_off = sv;
    mt.w_off = w;
    int pos = 0;
    for (int b : s.blocks) {
      const Block& B = A.blocks[b];
      GatherEntry e{};
      e.src_off = B.off;
      e.dst_off = a;
      e.rows = B.rows;
      e.cols = B.cols;
      e.dst_ld = std::max(mt.M, 1);
      if (dir == 0) { e.r0 = pos; e.c0 = 0; e.transpose = 0; pos += B.rows; }
      else { e.r0 = 0; e.c0 = pos; e.transpose = 1; pos += B.cols; }
      D.ent.push_back(e);
    }
    a += (int64_t)mt.M * mt.N;
    r += (int64_t)mt.N * mt.N;
    sv += mt.N;
    w += mt.N + (int64_t)mt.M * mt.N;
    D.mats.push_back(mt);
    Block rb;
    rb.qin = rb.qout = kv.first;
    rb.rows = rb.cols = mt.N;
    rb.off = (int64_t)mt.r_off;
    D.rlayout.blocks.push_back(rb);
  }
  D.rlayout.nelem = r;
  layout_index(D.rlayout);
  // null space of the stacked sector matrices (dir l): block rows follow the gather order
  if (dir == 0) {
    std::map<Key, int> sec_index;
    int si = 0;
    for (auto& kv : secs) sec_index[kv.first] = si++;
    int64_t ns = 0;
    for (DenseMat& mt : D.mats) {
      mt.ns_off = ns;
      ns += (int64_t)mt.M * std::max(mt.M - mt.N, 0);
    }
    D.ns_elems = ns;
    // row position of each block of A inside its stacked sector matrix
    std::map<int, int> row0;
    for (auto& kv : secs) {
      int pos = 0;
      for (int b : kv.second.blocks) { row0[b] = pos; pos += A.blocks[b].rows; }
    }
    D.nslayout = Layout();
    D.nslayout.nsym = A.nsym;
    int64_t off = 0;
    int maxg = 0;
    for (int b = 0; b < (int)A.blocks.size(); ++b) {  // A's (group, qin) order
      const Block& B = A.blocks[b];
      const DenseMat& mt = D.mats[sec_index[B.qout]];
      const int nul = mt.M - mt.N;
      if (nul <= 0) continue;
      Block nb;
      nb.qin = B.qin;
      nb.qout = B.qout;
      nb.rows = B.rows;
      nb.cols = nul;
      nb.group = B.group;
      nb.off = off;
      D.nslayout.blocks.push_back(nb);
      GatherEntry e{};
      e.src_off = off;
      e.dst_off = mt.ns_off;
      e.rows = B.rows;
      e.cols = nul;
      e.r0 = row0[b];
      e.c0 = 0;
      e.dst_ld = std::max(mt.M, 1);
      e.transpose = 0;
      D.nent.push_back(e);
      off += (int64_t)B.rows * nul;
      maxg = std::max(maxg, B.group);
    }
    D.nslayout.nelem = off;
    D.nslayout.ngroups = A.ngroups;
    layout_index(D.nslayout);
  }
  D.dense_elems = a;
  D.r_elems = r;
  D.s_elems = sv;
  D.w_elems = w;
  return IMPS_OK;
}

}  // namespace imps
