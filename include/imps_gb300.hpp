// C++ host interface over the C ABI of imps_gb300.h: RAII handles and the operator functors
// the reference hands to ARPACK and to its GMRES, with the reference's names and argument
// meaning, so that a call site of the reference changes only where its functor is built.
//
//   eigs_rs(Afun, Am_tot, EA, ACv, 1, "SA", tol, AC.Vectorize())   (VUMPS_main.cpp:184-186)
//     Afun = imps_cpp::ApplyHAvec(hac)                              (VUMPS_helpers.hpp:55-88)
//   TMDominantEig / TMMultDiag (EigsBlockFunctions.hpp:50-172)
//     imps_cpp::TMMultDiag(tm), imps_cpp::TMDominantEig(tm, ...)
//   InvertE_proj(MPSarr, x, L, R, dir, tol) (InvEBlockFunctions.hpp:201-266)
//     imps_cpp::InvertE_proj(tm, x, L, R, 'l' or 'r', y, tol)
//
// Vectors are the reference's Vectorize order (s-major, std::map key order, column-major
// blocks).  Errors: status < 0 throws imps_cpp::error (the reference aborts or throws there);
// status 1 (not converged) is returned, as the reference prints a warning and goes on.
#pragma once

#include <cstdint>
#include <functional>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "imps_gb300.h"

namespace imps_cpp {

struct error : std::runtime_error {
  int status;
  error(int st, const std::string& what) : std::runtime_error(what + ": " + imps_status_string(st)), status(st) {}
};

inline int check(int st, const char* what) {
  if (st < 0) throw error(st, what);
  return st;
}

class context {
 public:
  explicit context(int device = 0) { check(imps_ctx_create(device, &c_), "imps_ctx_create"); }
  ~context() { if (c_) imps_ctx_destroy(c_); }
  context(const context&) = delete;
  context& operator=(const context&) = delete;
  imps_ctx* get() const { return c_; }
  void synchronize() const { check(imps_ctx_synchronize(c_), "imps_ctx_synchronize"); }

 private:
  imps_ctx* c_ = nullptr;
};

// One block per row of the table: (group, qin[nsym], qout[nsym], rows, cols), in the
// reference's GetSizesVector order (MPSBlockMat.hpp:336-347).
struct block {
  int group;
  std::vector<int32_t> qin, qout;
  int rows, cols;
};

class layout {
 public:
  layout(int nsym, const std::vector<block>& blocks) {
    std::vector<int32_t> qin, qout, rows, cols, grp;
    for (const block& b : blocks) {
      qin.insert(qin.end(), b.qin.begin(), b.qin.end());
      qout.insert(qout.end(), b.qout.begin(), b.qout.end());
      rows.push_back(b.rows);
      cols.push_back(b.cols);
      grp.push_back(b.group);
    }
    check(imps_layout_create(nsym, (int)blocks.size(), qin.data(), qout.data(), rows.data(), cols.data(),
                             grp.data(), &L_),
          "imps_layout_create");
  }
  ~layout() { if (L_) imps_layout_destroy(L_); }
  layout(const layout&) = delete;
  layout& operator=(const layout&) = delete;
  layout(layout&& o) noexcept : L_(std::exchange(o.L_, nullptr)) {}
  const imps_layout* get() const { return L_; }
  imps_layout* get() { return L_; }
  int64_t nelem() const { return imps_layout_nelem(L_); }

 private:
  imps_layout* L_ = nullptr;
};

class plan {
 public:
  explicit plan(imps_plan* p = nullptr) : p_(p) {}
  ~plan() { if (p_) imps_plan_destroy(p_); }
  plan(const plan&) = delete;
  plan& operator=(const plan&) = delete;
  plan(plan&& o) noexcept : p_(std::exchange(o.p_, nullptr)) {}
  plan& operator=(plan&& o) noexcept {
    if (this != &o) {
      if (p_) imps_plan_destroy(p_);
      p_ = std::exchange(o.p_, nullptr);
    }
    return *this;
  }
  imps_plan* get() const { return p_; }
  void bind(int slot, double* device_ptr) { check(imps_plan_bind(p_, slot, device_ptr), "imps_plan_bind"); }
  void prepare() { check(imps_plan_prepare(p_), "imps_plan_prepare"); }

  // ApplyTMLeft (dir IMPS_DIR_LEFT) / ApplyTMRight on the unit cell A[0..n-1]; slots 2.. = A[k]
  static plan tm(const context& ctx, const std::vector<const layout*>& A, int dir, const layout& in,
                 const layout& out) {
    std::vector<const imps_layout*> a;
    for (const layout* l : A) a.push_back(l->get());
    imps_plan* p = nullptr;
    check(imps_plan_tm(ctx.get(), (int)a.size(), a.data(), dir, in.get(), out.get(), &p), "imps_plan_tm");
    return plan(p);
  }
  // per-sector decompositions of an MPS tensor, dir IMPS_DIR_LEFT (l) or IMPS_DIR_RIGHT (r)
  static plan decomp(const context& ctx, const layout& A, int dir) {
    imps_plan* p = nullptr;
    check(imps_plan_decomp(ctx.get(), A.get(), dir, &p), "imps_plan_decomp");
    return plan(p);
  }
  // a grouped-GEMM program (see struct program below); bind every slot, then run()
  static plan program(const context& ctx, const struct program& prog);
  void run() { check(imps_plan_run(p_), "imps_plan_run"); }
  // the plan applied to `copies` inputs at once (imps_plan_replicate), e.g. a mixed TM on the
  // 2P planes of P momenta
  static plan replicate(const plan& src, int copies) {
    imps_plan* p = nullptr;
    check(imps_plan_replicate(src.get(), copies, &p), "imps_plan_replicate");
    return plan(p);
  }
  // time every FP64 launch shape of the stages not tuned yet in this process, install the
  // fastest (imps_plan_autotune); returns the number of stages timed
  int autotune(int reps = 5) {
    int n = 0;
    check(imps_plan_autotune(p_, reps, &n), "imps_plan_autotune");
    return n;
  }

 private:
  imps_plan* p_ = nullptr;
};

// Tables of imps_plan_program: stages of output blocks C (+)= sum alpha op(A) op(B), the form
// into which the Python host code compiles the excitation ansatz, the energy gradient and the
// bond expansion.  Blocks are column-major regions (slot, offset, leading dimension, M, N).
struct program {
  struct term { int a_slot; int64_t a_off; int a_ld; bool a_trans; int b_slot; int64_t b_off; int b_ld;
                bool b_trans; int k; double alpha; };
  struct out { int slot; int64_t off; int ld, M, N; bool accumulate; std::vector<term> terms; };
  std::vector<int64_t> slot_nelem;
  std::vector<std::vector<out>> stages;
  std::vector<out>& stage() { stages.emplace_back(); return stages.back(); }
};

inline plan plan::program(const context& ctx, const struct program& prog) {
  std::vector<int32_t> nouts;
  std::vector<int64_t> outs, terms;
  std::vector<double> alphas;
  for (const auto& st : prog.stages) {
    nouts.push_back((int32_t)st.size());
    for (const auto& o : st) {
      outs.insert(outs.end(), {(int64_t)o.slot, o.off, (int64_t)o.ld, (int64_t)o.M, (int64_t)o.N,
                               (int64_t)o.accumulate, (int64_t)o.terms.size()});
      for (const auto& t : o.terms) {
        terms.insert(terms.end(), {(int64_t)t.a_slot, t.a_off, (int64_t)t.a_ld, (int64_t)t.a_trans, (int64_t)t.b_slot,
                                   t.b_off, (int64_t)t.b_ld, (int64_t)t.b_trans, (int64_t)t.k});
        alphas.push_back(t.alpha);
      }
    }
  }
  imps_plan* p = nullptr;
  check(imps_plan_program(ctx.get(), (int)prog.slot_nelem.size(), prog.slot_nelem.data(), (int)nouts.size(),
                          nouts.data(), outs.data(), terms.data(), alphas.data(), &p),
        "imps_plan_program");
  return plan(p);
}

// MultOPx of eigs_rs / eigs_n (eigs.h:43-58): out = Op(in), both of the operator's length
using multop = std::function<void(double*, double*)>;

// ApplyHAvec (VUMPS_helpers.hpp:55-88) on an H_AC plan
inline multop ApplyHAvec(plan& hac, int mem = IMPS_MEM_HOST) {
  return [&hac, mem](double* in, double* out) { check(imps_hac_apply(hac.get(), in, out, mem), "ApplyHAvec"); };
}
// ApplyHCvec (VUMPS_helpers.hpp:114-133) on an H_C plan
inline multop ApplyHCvec(plan& hc, int mem = IMPS_MEM_HOST) {
  return [&hc, mem](double* in, double* out) { check(imps_hc_apply(hc.get(), in, out, mem), "ApplyHCvec"); };
}
// TMMultDiag (EigsBlockFunctions.hpp:50-66) with ApplyTMLeft/Right on the unit cell
inline multop TMMultDiag(plan& tm, int mem = IMPS_MEM_HOST) {
  return [&tm, mem](double* in, double* out) { check(imps_tm_apply(tm.get(), in, out, mem), "TMMultDiag"); };
}
// InvEfun_proj (InvEBlockFunctions.hpp:12-47): out = in - T(in) + tr(in rho_in) rho_out
inline multop InvEfun_proj(plan& tm, const double* rho_in, const double* rho_out, int mem = IMPS_MEM_HOST) {
  return [&tm, rho_in, rho_out, mem](double* in, double* out) {
    check(imps_tm_proj_apply(tm.get(), in, rho_in, rho_out, out, mem), "InvEfun_proj");
  };
}

// eigs_rs(Afun, N, vals, vecs, 1, "SA", tol, x0) (eigs.cpp:369-494) on the device: x holds
// x0 on entry and the eigenvector on exit; returns the eigenvalue
inline double eigs_rs(plan& op, double* x, double tol, int ncv = 0, int* applies = nullptr,
                      int mem = IMPS_MEM_HOST) {
  double e = 0.0;
  int na = 0;
  check(imps_eigs_rs(op.get(), x, mem, tol, ncv, 0, &e, &na), "eigs_rs");
  if (applies) *applies = na;
  return e;
}

// eigs_n(fun, N, vals, vecs, nev, whch, tol) (eigs.cpp:193-342): the nev wanted eigenvalues
// (re, im) of a nonsymmetric plan; whch "LM", "LR" or "SR"
inline std::vector<std::pair<double, double>> eigs_n(plan& op, int nev, const std::string& whch, double tol,
                                                     int* applies = nullptr) {
  const int which = whch == "LR" ? IMPS_WHICH_LR : whch == "SR" ? IMPS_WHICH_SR : IMPS_WHICH_LM;
  std::vector<double> ev(2 * (size_t)nev);
  int na = 0;
  check(imps_eigs_n(op.get(), nullptr, IMPS_MEM_HOST, nev, which, tol, 0, 0, ev.data(), nullptr, nullptr, &na),
        "eigs_n");
  if (applies) *applies = na;
  std::vector<std::pair<double, double>> out;
  for (int i = 0; i < nev; ++i) out.emplace_back(ev[2 * i], ev[2 * i + 1]);
  return out;
}

// TMDominantEig (EigsBlockFunctions.hpp:91-172) of an isometric unit cell: V the fixed point,
// normalised to unit trace; returns the eigenvalue
inline double TMDominantEig(plan& tm, double* V, double tol, const double* x0 = nullptr, int mem = IMPS_MEM_HOST) {
  double lam = 0.0;
  int it = 0;
  check(imps_tm_dominant(tm.get(), x0, V, mem, tol, 0, &lam, &it), "TMDominantEig");
  return lam;
}

// InvertE_proj (InvEBlockFunctions.hpp:201-266): dir 'l' solves y (1 - T + |R)(L|) =
// x (1 - |R)(L|), dir 'r' (1 - T + |R)(L|) y = (1 - |R)(L|) x; y holds y0 on entry.  Returns
// the status (1: not converged, y returned, as the reference's cerr warning).
inline int InvertE_proj(plan& tm, const double* x, const double* L, const double* R, char dir, double* y,
                        double tol, int maxit = 0, int* iters = nullptr, int mem = IMPS_MEM_HOST) {
  int it = 0;
  double rr = 0.0;
  const int st = check(imps_invert_e_proj(tm.get(), x, L, R, dir == 'l' ? IMPS_DIR_LEFT : IMPS_DIR_RIGHT, y, mem,
                                          tol, maxit, 0, &it, &rr),
                       "InvertE_proj");
  if (iters) *iters = it;
  return st;
}

// InvertE_fac (InvEBlockFunctions.hpp:346-476) for P momenta at once on rep = plan::replicate(
// tmx, 2P): (1 - f_j T) y_j = x_j, device vectors; returns the status (1: some system not
// converged)
inline int InvertE_fac_batch(plan& rep, const std::vector<const double*>& x_re, const std::vector<const double*>& x_im,
                             const std::vector<double>& f_re, const std::vector<double>& f_im,
                             const std::vector<double*>& y_re, const std::vector<double*>& y_im, double tol,
                             int* iters = nullptr) {
  int it = 0;
  double rr = 0.0;
  const int st = check(imps_invert_e_fac_batch(rep.get(), (int)x_re.size(), x_re.data(), x_im.data(), f_re.data(),
                                               f_im.data(), y_re.data(), y_im.data(), tol, 0, 0, &it, &rr),
                       "InvertE_fac_batch");
  if (iters) *iters = it;
  return st;
}

// The nev lowest eigenvalues of P symmetric operators at once (imps_eigs_rs_batch_op): op
// applies all P operators to P consecutive device vectors of length n; X (device, P x n) holds
// the start vectors and receives each system's lowest Ritz vector.  Returns P x nev values.
using batch_op = std::function<void(const double* in, double* out)>;
inline std::vector<double> eigs_rs_batch(context& ctx, int P, int64_t n, const batch_op& op, double* X, int nev,
                                         double tol, int ncv = 0, int* applies = nullptr) {
  struct tramp {
    static int call(void* user, const double* in, double* out) {
      try {
        (*static_cast<const batch_op*>(user))(in, out);
        return IMPS_OK;
      } catch (...) {
        return IMPS_ERR_CUDA;  // a failing apply ends the solve with an error status
      }
    }
  };
  std::vector<double> ev((size_t)P * nev);
  int na = 0;
  check(imps_eigs_rs_batch_op(ctx.get(), P, n, &tramp::call, const_cast<batch_op*>(&op), X, nev, tol, ncv, 0,
                              ev.data(), &na, nullptr),
        "eigs_rs_batch");
  if (applies) *applies = na;
  return ev;
}

// qr(R, MPS, dir) (MPSBlockUtilities.hpp:181-244) on device buffers: Q in A's layout, R in
// the plan's DiagIso layout, diag(R) >= 0 (qr_pos)
inline void qr(plan& dec, const double* A, double* Q, double* R) {
  check(imps_sector_qr(dec.get(), A, Q, R, IMPS_MEM_DEVICE), "qr");
}

}  // namespace imps_cpp
