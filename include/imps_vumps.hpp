// The VUMPS sweep of VUMPS/VUMPS_main.cpp:97-354 as C++ host code over the C ABI of
// imps_gb300.h, for a two-site unit cell with abelian U(1)^k charges and bond expansion off: the
// same operations, in the same order, as the Python driver (imps_cpp_tools_gb300/vumps.py), so
// that a C++ program runs the hot path without Python.
//
//   imps_cpp::context ctx(0);
//   imps_cpp::vumps v(ctx, model, dimvec, init, opts);   // model: d, I2K, nonzeros of h
//   for (...) { auto E = v.sweep(); ... v.F ... v.prec ... }
//
// Indices.  Site n (n = 0, 1) maps bond n -> bond n+1 (mod 2); C[b] is the centre matrix on bond
// b; updating site n uses AC(n) = C[n] AR(n), HL from AL(n-1), HR from AR(n+1), CL = C[n],
// CR = C[n+1] (the reference rotates its unit-cell arrays after each site update instead,
// VUMPS_main.cpp:256-259).  Device memory: cudaMalloc'd buffers; the context runs on the legacy
// default stream, so the synchronous cudaMemcpy / cudaMemset here are ordered with its kernels.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <map>
#include <exception>
#include <memory>
#include <thread>
#include <vector>

#include "imps_gb300.hpp"

namespace imps_cpp {

using charge = std::vector<int32_t>;
using bond_dims = std::map<charge, int>;  // sector charge -> dimension (std::map order)

struct hnonzero {
  int row, col;
  double val;
};

// h as the list of its nonzeros (row, col over the d^2 two-site basis), with I2K: the charge
// shift of every physical index (Models.cpp:216-295, 642-733)
struct model {
  int d = 2;
  std::vector<charge> I2K;
  std::vector<hnonzero> h;
};

// the reference's defaults (VUMPS_main.cpp:31-40); fixed_tol > 0 replaces the tolerance
// schedule min(max(prec / 100, tolmin), tolmax) (VUMPS_main.cpp:177)
struct vumps_options {
  double fixed_tol = 0.0, tolmin = 5e-16, tolmax = 1e-6, InvETol = 5e-15, InvEfac = 2.0, svdthresh = 5e-7;
  double eig_margin = 0.1;  // the Lanczos tests every 4 steps, ARPACK once per cycle (vumps.py)
  int lanczos_ncv = 126, lanczos_maxit = 300, gmres_maxit = 4000;
  bool trueLR = true;
  bool autotune = false;  // time every plan's FP64 launch shapes once (imps_plan_autotune)
  // the two H_C eigensolves of a site update (VUMPS_main.cpp:199-200) on contexts of their own
  // (non-blocking streams, own Krylov workspaces) from threads of their own, beside the H_AC
  // eigensolve (:186); the results are those of the serial order
  bool concurrent = true;
};

// a device vector of doubles
class dvec {
 public:
  dvec() = default;
  explicit dvec(int64_t n) : n_(n) {
    if (cudaMalloc(&p_, std::max<int64_t>(n, 1) * sizeof(double)) != cudaSuccess) throw error(IMPS_ERR_OOM, "dvec");
    zero();
  }
  ~dvec() { if (p_) cudaFree(p_); }
  dvec(const dvec&) = delete;
  dvec& operator=(const dvec&) = delete;
  dvec(dvec&& o) noexcept : p_(std::exchange(o.p_, nullptr)), n_(std::exchange(o.n_, 0)) {}
  dvec& operator=(dvec&& o) noexcept {
    if (this != &o) { if (p_) cudaFree(p_); p_ = std::exchange(o.p_, nullptr); n_ = std::exchange(o.n_, 0); }
    return *this;
  }
  double* get() const { return p_; }
  int64_t size() const { return n_; }
  void zero() { cudaMemset(p_, 0, std::max<int64_t>(n_, 1) * sizeof(double)); }
  void upload(const std::vector<double>& h) {
    if ((int64_t)h.size() != n_) throw error(IMPS_ERR_BAD_ARG, "dvec upload size");
    if (cudaMemcpy(p_, h.data(), n_ * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
      throw error(IMPS_ERR_CUDA, "dvec upload");
  }
  std::vector<double> download() const {
    std::vector<double> h(n_);
    if (cudaMemcpy(h.data(), p_, n_ * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
      throw error(IMPS_ERR_CUDA, "dvec download");
    return h;
  }
  dvec clone() const {
    dvec o(n_);
    cudaMemcpy(o.p_, p_, n_ * sizeof(double), cudaMemcpyDeviceToDevice);
    return o;
  }

 private:
  double* p_ = nullptr;
  int64_t n_ = 0;
};

// MPSBlockMat(I2K, ml, mr) sector structure (MPSBlockMat.hpp:221-236), grouped by s
inline std::vector<block> mps_blocks(const std::vector<charge>& I2K, const bond_dims& dl, const bond_dims& dr) {
  std::vector<block> out;
  for (int s = 0; s < (int)I2K.size(); ++s)
    for (const auto& [ql, ml] : dl) {
      charge qr = ql;
      for (size_t i = 0; i < qr.size(); ++i) qr[i] += I2K[s][i];
      auto it = dr.find(qr);
      if (it != dr.end()) out.push_back(block{s, ql, qr, ml, it->second});
    }
  return out;
}

inline std::vector<block> bd_blocks(const bond_dims& d) {
  std::vector<block> out;
  for (const auto& [q, m] : d) out.push_back(block{0, q, q, m, m});
  return out;
}

class vumps {
 public:
  std::array<double, 2> F{1.0, 1.0}, prec{1.0, 1.0};
  int lanczos_applies = 0, gmres_iters = 0;

  // init: AL[n], AR[n] (MPS layout of site n) and C[b] (BlockDiagMat of bond b), flat in the
  // reference's Vectorize order
  vumps(context& ctx, const model& m, const std::array<bond_dims, 2>& dimvec,
        const std::array<std::vector<double>, 6>& init, const vumps_options& o = vumps_options())
      : ctx_(ctx), m_(m), dims_(dimvec), o_(o) {
    check(imps_ctx_set_stream(ctx_.get(), nullptr), "imps_ctx_set_stream");
    if (o_.concurrent) {
      int dev = 0;
      cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
      cuda_check(cudaEventCreateWithFlags(&ev_main_, cudaEventDisableTiming), "cudaEventCreate");
      for (side_ctx& s : side_) s.open(dev);
    }
    const int nsym = (int)m_.I2K.at(0).size();
    for (const auto& z : m_.h) { hr_.push_back(z.row); hc_.push_back(z.col); hv_.push_back(z.val); }
    for (int n = 0; n < 2; ++n) {
      LA_.emplace_back(nsym, mps_blocks(m_.I2K, dims_[n], dims_[1 - n]));
      LB_.emplace_back(nsym, bd_blocks(dims_[n]));
    }
    build_plans();
    // plan tables are uploaded by synchronous copies on the legacy default stream, whose last DMA
    // the non-blocking streams of the H_C contexts do not wait for
    if (o_.concurrent) cuda_check(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    for (int n = 0; n < 2; ++n) {
      AL_[n] = dvec(LA_[n].nelem()); AL_[n].upload(init[n]);
      AR_[n] = dvec(LA_[n].nelem()); AR_[n].upload(init[2 + n]);
      C_[n] = dvec(LB_[n].nelem()); C_[n].upload(init[4 + n]);
      eye_[n] = dvec(LB_[n].nelem());
      std::vector<double> e(LB_[n].nelem(), 0.0);
      int64_t off = 0;
      for (const auto& [q, mm] : dims_[n]) {
        for (int i = 0; i < mm; ++i) e[off + i + (int64_t)i * mm] = 1.0;
        off += (int64_t)mm * mm;
      }
      eye_[n].upload(e);
    }
    init_environments();
  }

  // one iteration of the outer loop (VUMPS_main.cpp:165-354); returns the two bond energies in
  // the reference's output order
  std::array<double, 2> sweep() {
    for (int n = 0; n < 2; ++n) site_update(n);
    return energy();
  }

  // MeasureObservables(H, AR, L) (MPSBlockUtilities.hpp:1017-1073) of the energy: per bond k,
  // tr(L_k OpTM_R(AR(k) AR(k+1))) with L_k = C[k]^T C[k]
  std::array<double, 2> energy() {
    std::array<double, 2> E{};
    int i = 0;
    for (int k : {1, 0}) {
      dvec X = z(LB_[k]);
      optm(false, k, AR_, X);
      dvec L = cct(k, false);
      check(imps_bd_trace_prod(ctx_.get(), LB_[k].get(), L.get(), X.get(), &E[i++]), "imps_bd_trace_prod");
    }
    return E;
  }

  ~vumps() {
    if (ev_main_) cudaEventDestroy(ev_main_);
  }
  vumps(const vumps&) = delete;
  vumps& operator=(const vumps&) = delete;

  const dvec& AL(int n) const { return AL_[n]; }
  const dvec& AR(int n) const { return AR_[n]; }
  const dvec& C(int b) const { return C_[b]; }

 private:
  static void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw error(IMPS_ERR_CUDA, what);
  }
  // a context of its own for one H_C eigensolve: a non-blocking stream, ordered with the legacy
  // default stream of the main context by events
  struct side_ctx {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    std::unique_ptr<context> ctx;
    int device = 0;
    side_ctx() = default;
    side_ctx(const side_ctx&) = delete;
    side_ctx& operator=(const side_ctx&) = delete;
    void open(int dev) {
      device = dev;
      ctx = std::make_unique<context>(dev);
      cuda_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
      cuda_check(cudaEventCreateWithFlags(&done, cudaEventDisableTiming), "cudaEventCreate");
      check(imps_ctx_set_stream(ctx->get(), stream), "imps_ctx_set_stream");
    }
    ~side_ctx() {
      ctx.reset();  // synchronises its stream
      if (stream) cudaStreamDestroy(stream);
      if (done) cudaEventDestroy(done);
    }
  };

  context& ctx_;
  // destroyed after the plans below (declared before them), which synchronise their context
  std::array<side_ctx, 2> side_;
  cudaEvent_t ev_main_ = nullptr;
  model m_;
  std::array<bond_dims, 2> dims_;
  vumps_options o_;
  std::vector<int32_t> hr_, hc_;
  std::vector<double> hv_;
  std::vector<layout> LA_, LB_;
  std::array<dvec, 2> AL_, AR_, C_, eye_, HLbuf_, HRbuf_, EHR0_;
  std::array<bool, 2> have_ehr0_{false, false};
  dvec EHL_, EHR_, EHL1_, EHR1_, EHLtmp_;
  bool dosvd_ = true;
  // plans (vumps.py _build_plans)
  std::vector<plan> redop_l_, redop_r_, p_ac_, p_hac_, p_grad_, p_hcl_, p_hcr_, p_mul_r_t_, p_mul_l_t_, p_mul_r_,
      p_mul_l_, dec_ac_l_, dec_ac_r_, dec_b_l_, dec_b_r_, optm_l_, optm_r_;
  std::map<std::pair<int, int>, plan> tm_;  // (kind, n): kind 0 L, 1 R, 2 L1, 3 R1
  std::vector<layout> lHL_, lHR_, rl_ac_l_, rl_ac_r_;
  std::array<plan, 4> cct_;  // (bond, right) -> C C^T (right) or C^T C
  // the right-environment chain's own plans on side_[1] (the left chain binds the same unit-cell
  // transfer matrices to AL at the same time), with o_.concurrent
  std::map<std::pair<int, int>, plan> env_tm_;
  std::vector<plan> env_optm_r_;
  std::array<plan, 4> env_cct_;

  dvec z(const layout& L) const { return dvec(L.nelem()); }

  static layout derived(const plan& p, int which) {
    imps_layout* h = nullptr;
    check(imps_plan_derived_layout(p.get(), which, &h), "imps_plan_derived_layout");
    // take ownership of a copy of the table (the plan keeps its own)
    const int nb = imps_layout_nblocks(h), ns = imps_layout_nsym(h);
    std::vector<int32_t> qin((size_t)nb * ns + 1), qout((size_t)nb * ns + 1), rows(nb + 1), cols(nb + 1),
        grp(nb + 1);
    check(imps_layout_get(h, qin.data(), qout.data(), rows.data(), cols.data(), grp.data(), nullptr),
          "imps_layout_get");
    imps_layout_destroy(h);
    std::vector<block> b;
    for (int i = 0; i < nb; ++i)
      b.push_back(block{grp[i], charge(qin.begin() + (size_t)i * ns, qin.begin() + (size_t)(i + 1) * ns),
                        charge(qout.begin() + (size_t)i * ns, qout.begin() + (size_t)(i + 1) * ns), rows[i], cols[i]});
    return layout(ns, b);
  }

  plan mk(int rc, imps_plan* p, const char* what) {
    check(rc, what);
    return plan(p);
  }

  void build_plans() {
    imps_ctx* c = ctx_.get();
    imps_ctx* hc_ctx[2] = {o_.concurrent ? side_[0].ctx->get() : c, o_.concurrent ? side_[1].ctx->get() : c};
    const int d = m_.d, nnz = (int)hv_.size();
    imps_plan* p = nullptr;
    for (int mm = 0; mm < 2; ++mm) {
      redop_l_.push_back(mk(imps_plan_redop(c, LA_[mm].get(), d, nnz, hr_.data(), hc_.data(), hv_.data(), 0, &p), p,
                            "imps_plan_redop"));
      redop_r_.push_back(mk(imps_plan_redop(c, LA_[mm].get(), d, nnz, hr_.data(), hc_.data(), hv_.data(), 1, &p), p,
                            "imps_plan_redop"));
      lHL_.push_back(derived(redop_l_.back(), 0));
      lHR_.push_back(derived(redop_r_.back(), 0));
      HLbuf_[mm] = z(lHL_.back());
      HRbuf_[mm] = z(lHR_.back());
    }
    for (int n = 0; n < 2; ++n) {
      const int l = n, r = 1 - n, mm = 1 - n;
      p_ac_.push_back(mk(imps_plan_mps_bd(c, LA_[n].get(), LB_[l].get(), 0, 1.0, &p), p, "mps_bd"));
      p_hac_.push_back(mk(imps_plan_hac(c, LA_[n].get(), LB_[l].get(), LB_[r].get(), lHL_[mm].get(), lHR_[mm].get(),
                                        d, &p), p, "imps_plan_hac"));
      p_grad_.push_back(mk(imps_plan_grad_right(c, LA_[n].get(), LA_[n].get(), &p), p, "imps_plan_grad_right"));
      p_hcl_.push_back(mk(imps_plan_hc(hc_ctx[0], LB_[l].get(), LB_[l].get(), LB_[l].get(), LA_[mm].get(),
                                       LA_[n].get(), d, nnz, hr_.data(), hc_.data(), hv_.data(), &p), p,
                          "imps_plan_hc"));
      p_hcr_.push_back(mk(imps_plan_hc(hc_ctx[1], LB_[r].get(), LB_[r].get(), LB_[r].get(), LA_[n].get(),
                                       LA_[mm].get(), d, nnz, hr_.data(), hc_.data(), hv_.data(), &p), p,
                          "imps_plan_hc"));
      p_mul_r_t_.push_back(mk(imps_plan_mps_bd(c, LA_[n].get(), LB_[r].get(), 1 | 2, 1.0, &p), p, "mps_bd"));
      p_mul_l_t_.push_back(mk(imps_plan_mps_bd(c, LA_[n].get(), LB_[l].get(), 0 | 2, 1.0, &p), p, "mps_bd"));
      p_mul_r_.push_back(mk(imps_plan_mps_bd(c, LA_[n].get(), LB_[r].get(), 1, 1.0, &p), p, "mps_bd"));
      p_mul_l_.push_back(mk(imps_plan_mps_bd(c, LA_[n].get(), LB_[l].get(), 0, 1.0, &p), p, "mps_bd"));
      dec_ac_l_.push_back(mk(imps_plan_decomp(c, LA_[n].get(), 0, &p), p, "imps_plan_decomp"));
      dec_ac_r_.push_back(mk(imps_plan_decomp(c, LA_[n].get(), 1, &p), p, "imps_plan_decomp"));
      rl_ac_l_.push_back(derived(dec_ac_l_.back(), 1));
      rl_ac_r_.push_back(derived(dec_ac_r_.back(), 1));
      const imps_layout* uc[2] = {LA_[n].get(), LA_[mm].get()};
      tm_.emplace(std::make_pair(0, n), mk(imps_plan_tm(c, 2, uc, 0, LB_[l].get(), LB_[l].get(), &p), p, "tm"));
      tm_.emplace(std::make_pair(1, n), mk(imps_plan_tm(c, 2, uc, 1, LB_[l].get(), LB_[l].get(), &p), p, "tm"));
      const imps_layout* one[1] = {LA_[n].get()};
      tm_.emplace(std::make_pair(2, n), mk(imps_plan_tm(c, 1, one, 0, LB_[l].get(), LB_[r].get(), &p), p, "tm"));
      tm_.emplace(std::make_pair(3, n), mk(imps_plan_tm(c, 1, one, 1, LB_[r].get(), LB_[l].get(), &p), p, "tm"));
    }
    for (int b = 0; b < 2; ++b) {
      dec_b_l_.push_back(mk(imps_plan_decomp(c, LB_[b].get(), 0, &p), p, "imps_plan_decomp"));
      dec_b_r_.push_back(mk(imps_plan_decomp(c, LB_[b].get(), 1, &p), p, "imps_plan_decomp"));
      cct_[2 * b + 1] = mk(imps_plan_mps_bd(c, LB_[b].get(), LB_[b].get(), 1 | 2, 1.0, &p), p, "mps_bd");
      cct_[2 * b] = mk(imps_plan_mps_bd(c, LB_[b].get(), LB_[b].get(), 0 | 2, 1.0, &p), p, "mps_bd");
    }
    for (int a = 0; a < 2; ++a) {
      optm_l_.push_back(mk(imps_plan_optm(c, LA_[a].get(), LA_[1 - a].get(), d, nnz, hr_.data(), hc_.data(),
                                          hv_.data(), 0, LB_[a].get(), &p), p, "imps_plan_optm"));
      optm_r_.push_back(mk(imps_plan_optm(c, LA_[a].get(), LA_[1 - a].get(), d, nnz, hr_.data(), hc_.data(),
                                          hv_.data(), 1, LB_[a].get(), &p), p, "imps_plan_optm"));
    }
    if (o_.concurrent) {
      imps_ctx* e = side_[1].ctx->get();
      for (int n = 0; n < 2; ++n) {
        const int l = n, r = 1 - n, mm = 1 - n;
        const imps_layout* uc[2] = {LA_[n].get(), LA_[mm].get()};
        env_tm_.emplace(std::make_pair(0, n), mk(imps_plan_tm(e, 2, uc, 0, LB_[l].get(), LB_[l].get(), &p), p, "tm"));
        env_tm_.emplace(std::make_pair(1, n), mk(imps_plan_tm(e, 2, uc, 1, LB_[l].get(), LB_[l].get(), &p), p, "tm"));
        const imps_layout* one[1] = {LA_[n].get()};
        env_tm_.emplace(std::make_pair(3, n), mk(imps_plan_tm(e, 1, one, 1, LB_[r].get(), LB_[l].get(), &p), p, "tm"));
        env_cct_[2 * n] = mk(imps_plan_mps_bd(e, LB_[n].get(), LB_[n].get(), 0 | 2, 1.0, &p), p, "mps_bd");
        env_optm_r_.push_back(mk(imps_plan_optm(e, LA_[n].get(), LA_[1 - n].get(), d, nnz, hr_.data(), hc_.data(),
                                                hv_.data(), 1, LB_[n].get(), &p), p, "imps_plan_optm"));
      }
    }
    if (o_.autotune) {
      for (auto* v : {&redop_l_, &redop_r_, &p_ac_, &p_hac_, &p_grad_, &p_hcl_, &p_hcr_, &p_mul_r_t_, &p_mul_l_t_,
                      &p_mul_r_, &p_mul_l_, &optm_l_, &optm_r_, &env_optm_r_})
        for (plan& q : *v) q.autotune();
      for (auto* t : {&tm_, &env_tm_})
        for (auto& kv : *t) kv.second.autotune();
      for (plan& q : cct_) q.autotune();
      for (plan& q : env_cct_)
        if (q.get()) q.autotune();
    }
  }

  // ---- small helpers (vumps.py) ----
  void tm(int kind, int n, std::array<dvec, 2>& A, const dvec& vin, dvec& vout) {
    plan& p = tm_.at({kind, n});
    if (kind < 2) { p.bind(2, A[n].get()); p.bind(3, A[1 - n].get()); }
    else p.bind(2, A[n].get());
    p.bind(0, vin.get());
    p.bind(1, vout.get());
    p.run();
  }
  void optm(bool left, int a, std::array<dvec, 2>& A, dvec& out) {
    plan& p = (left ? optm_l_ : optm_r_)[a];
    p.bind(0, A[a].get());
    p.bind(1, A[1 - a].get());
    p.bind(2, out.get());
    p.run();
  }
  static void mul(plan& p, const dvec& A, const dvec& X, dvec& out) {
    p.bind(0, A.get());
    p.bind(1, X.get());
    p.bind(2, out.get());
    p.run();
  }
  void axpby(double a, const dvec& x, double b, dvec& y) {
    check(imps_axpby(ctx_.get(), a, x.get(), b, y.get(), y.size()), "imps_axpby");
  }
  dvec cct(int b, bool right) {  // C C^T (right) or C^T C on bond b
    dvec out = z(LB_[b]);
    mul(cct_[2 * b + (right ? 1 : 0)], C_[b], C_[b], out);
    return out;
  }
  void redops(int mm) {  // ReducedOp (MPSBlockUtilities.hpp:37-74): HL from AL(m), HR from AR(m)
    redop_l_[mm].bind(0, AL_[mm].get()); redop_l_[mm].bind(1, HLbuf_[mm].get()); redop_l_[mm].run();
    redop_r_[mm].bind(0, AR_[mm].get()); redop_r_[mm].bind(1, HRbuf_[mm].get()); redop_r_[mm].run();
  }
  dvec get_hl(int n) {  // GetHL (VUMPS_helpers.hpp:3-18) of [AL(n), AL(n+1)] -> bond n
    const int mm = 1 - n;
    dvec t = z(LB_[mm]);
    optm(true, mm, AL_, t);
    dvec out = z(LB_[n]);
    tm(2, mm, AL_, t, out);
    dvec t2 = z(LB_[n]);
    optm(true, n, AL_, t2);
    axpby(1.0, t2, 1.0, out);
    return out;
  }
  dvec get_hr(int n) {  // GetHR (VUMPS_helpers.hpp:20-36) of [AR(n), AR(n+1)] -> bond n
    const int mm = 1 - n;
    dvec t = z(LB_[mm]);
    optm(false, mm, AR_, t);
    dvec out = z(LB_[n]);
    tm(3, n, AR_, t, out);
    dvec t2 = z(LB_[n]);
    optm(false, n, AR_, t2);
    axpby(1.0, t2, 1.0, out);
    return out;
  }
  dvec invert_e(int kind, int n, std::array<dvec, 2>& A, const dvec& x, const dvec& L, const dvec& R, char dir,
                const dvec* y0, double tol) {
    plan& p = tm_.at({kind, n});
    p.bind(2, A[n].get());
    p.bind(3, A[1 - n].get());
    dvec y = y0 ? y0->clone() : dvec(x.size());
    int it = 0;
    double rr = 0.0;
    check(imps_invert_e_proj(p.get(), x.get(), L.get(), R.get(), dir == 'l' ? IMPS_DIR_LEFT : IMPS_DIR_RIGHT,
                             y.get(), IMPS_MEM_DEVICE, tol, o_.gmres_maxit, 0, &it, &rr),
          "InvertE_proj");
    gmres_iters += it;
    return y;
  }
  dvec tm_dominant(int kind, int n, std::array<dvec, 2>& A, const dvec& x0, double tol) {
    plan& p = tm_.at({kind, n});
    p.bind(2, A[n].get());
    p.bind(3, A[1 - n].get());
    dvec V(x0.size());
    double lam = 0.0;
    int it = 0;
    check(imps_tm_dominant(p.get(), x0.get(), V.get(), IMPS_MEM_DEVICE, tol, o_.gmres_maxit, &lam, &it),
          "TMDominantEig");
    gmres_iters += it;
    return V;
  }
  // the plans of the right-environment chain and the context they run on
  struct chain_plans {
    imps_ctx* ctx;
    std::map<std::pair<int, int>, plan>* tm;  // (0, n) L, (1, n) R, (3, n) R1
    std::vector<plan>* optm_r;
    std::array<plan, 4>* cct;  // [2b]: C^T C on bond b
  };
  // its buffers, allocated (and y filled with the previous EHR of the site) on the legacy default
  // stream before the chain starts
  struct env_bufs {
    dvec L, V, t, out, t2, y;
  };
  env_bufs env_buffers(int n) {
    const int l = n, mm = 1 - n;
    return env_bufs{z(LB_[l]), z(LB_[l]), z(LB_[mm]), z(LB_[l]), z(LB_[l]),
                    have_ehr0_[mm] ? EHR0_[mm].clone() : z(LB_[l])};
  }
  // Right environment for site n+1 (VUMPS_main.cpp:241-247): L = C^T C on bond n (= bond n+2), its
  // fixed point of [AR(n), AR(n+1)], GetHR, then EHR by InvertE_proj into b.y; returns the
  // iterations of the two solves
  int right_env(int n, double gtol, chain_plans P, env_bufs& b) {
    const int l = n, mm = 1 - n;
    int iters = 0, it = 0;
    mul((*P.cct)[2 * l], C_[l], C_[l], b.L);
    const dvec* L = &b.L;
    auto bind_uc = [&](plan& q) { q.bind(2, AR_[n].get()); q.bind(3, AR_[mm].get()); return q.get(); };
    if (o_.trueLR) {
      double lam = 0.0;
      check(imps_tm_dominant(bind_uc(P.tm->at({0, n})), b.L.get(), b.V.get(), IMPS_MEM_DEVICE, 1e-15, o_.gmres_maxit,
                             &lam, &it),
            "TMDominantEig");
      iters += it;
      L = &b.V;
    }
    // GetHR (VUMPS_helpers.hpp:20-36) of [AR(n), AR(n+1)] -> bond n, into b.out
    auto optm_r = [&](int a, dvec& out) {
      plan& q = (*P.optm_r)[a];
      q.bind(0, AR_[a].get()); q.bind(1, AR_[1 - a].get()); q.bind(2, out.get());
      q.run();
    };
    optm_r(mm, b.t);
    plan& r1 = P.tm->at({3, n});
    r1.bind(2, AR_[n].get()); r1.bind(0, b.t.get()); r1.bind(1, b.out.get());
    r1.run();
    optm_r(n, b.t2);
    check(imps_axpby(P.ctx, 1.0, b.t2.get(), 1.0, b.out.get(), b.out.size()), "imps_axpby");
    double rr = 0.0;
    check(imps_invert_e_proj(bind_uc(P.tm->at({1, n})), b.out.get(), L->get(), eye_[l].get(), IMPS_DIR_RIGHT,
                             b.y.get(), IMPS_MEM_DEVICE, gtol, o_.gmres_maxit, 0, &it, &rr),
          "InvertE_proj");
    return iters + it;
  }
  // eigs_rs "SA" with x0 = x; returns the number of applies
  int eigs(plan& p, dvec& x, double tol) const {
    double e = 0.0;
    int na = 0;
    check(imps_eigs_rs(p.get(), x.get(), IMPS_MEM_DEVICE, tol, o_.lanczos_ncv, o_.lanczos_maxit, &e, &na),
          "eigs_rs");
    return na;
  }
  double absmax(const dvec& x) {
    double r = 0.0;
    check(imps_absmax(ctx_.get(), x.get(), x.size(), &r), "imps_absmax");
    return r;
  }

  // VUMPS_main.cpp:103-136: reduced operators, EHL / EHR, EHL1 / EHR1
  void init_environments() {
    redops(0);
    redops(1);
    dvec R = cct(0, true);
    EHL_ = invert_e(0, 0, AL_, get_hl(0), eye_[0], R, 'l', nullptr, o_.InvETol);
    EHR_ = invert_e(1, 1, AR_, get_hr(1), cct(1, false), eye_[1], 'r', nullptr, o_.InvETol);
    EHL1_ = z(LB_[1]);
    optm(true, 1, AL_, EHL1_);
    dvec t = z(LB_[1]);
    tm(2, 0, AL_, EHL_, t);
    axpby(1.0, EHL1_, 1.0, t);
    EHL1_ = std::move(t);
    EHR1_ = z(LB_[0]);
    optm(false, 0, AR_, EHR1_);
    dvec t2 = z(LB_[0]);
    tm(3, 0, AR_, EHR_, t2);
    axpby(1.0, EHR1_, 1.0, t2);
    EHR1_ = std::move(t2);
  }

  // one iteration of the site loop, VUMPS_main.cpp:171-313, for site n
  void site_update(int n) {
    imps_ctx* c = ctx_.get();
    const int l = n, r = 1 - n, mm = 1 - n;
    EHR0_[n] = EHR_.clone();
    have_ehr0_[n] = true;
    plan& hac = p_hac_[n];
    hac.bind(2, EHL_.get()); hac.bind(3, EHR_.get()); hac.bind(4, HLbuf_[mm].get()); hac.bind(5, HRbuf_[mm].get());
    hac.prepare();
    // gradient norm (GradNormRight, VUMPS_helpers.hpp:145-153) at AC = C[n] AR(n)
    dvec AC = z(LA_[n]);
    mul(p_ac_[n], AR_[n], C_[l], AC);
    dvec Y = z(LA_[n]);
    check(imps_hac_apply(hac.get(), AC.get(), Y.get(), IMPS_MEM_DEVICE), "ApplyHAvec");
    dvec gscr = z(LA_[n]);
    plan& g = p_grad_[n];
    g.bind(0, Y.get()); g.bind(1, AR_[n].get()); g.bind(2, gscr.get());
    check(imps_grad_norm_right(g.get(), &F[n]), "GradNormRight");
    const double tol = o_.fixed_tol > 0 ? o_.fixed_tol : std::min(std::max(prec[n] / 100.0, o_.tolmin), o_.tolmax);
    const double tol_eig = tol * o_.eig_margin;
    // H_C eigensolves for CL = C[n] (EHL, EHR1) and CR = C[n+1] (EHL1, EHR)
    dvec CL = C_[l].clone(), CR = C_[r].clone();
    if (o_.concurrent) {
      // the operands and start vectors were written on the legacy default stream
      cuda_check(cudaEventRecord(ev_main_, nullptr), "cudaEventRecord");
      for (side_ctx& s : side_) cuda_check(cudaStreamWaitEvent(s.stream, ev_main_, 0), "cudaStreamWaitEvent");
    }
    plan& pl = p_hcl_[n];
    pl.bind(2, EHL_.get()); pl.bind(3, EHR1_.get()); pl.bind(4, AL_[mm].get()); pl.bind(5, AR_[n].get());
    pl.prepare();
    plan& pr = p_hcr_[n];
    pr.bind(2, EHL1_.get()); pr.bind(3, EHR_.get()); pr.bind(4, AL_[n].get()); pr.bind(5, AR_[mm].get());
    pr.prepare();
    int na_c[2] = {0, 0};
    std::exception_ptr err[2];
    std::thread jobs[2];
    if (o_.concurrent) {
      plan* ps[2] = {&pl, &pr};
      dvec* xs[2] = {&CL, &CR};
      for (int k = 0; k < 2; ++k)
        jobs[k] = std::thread([this, k, ps, xs, tol_eig, &na_c, &err] {
          try {
            cuda_check(cudaSetDevice(side_[k].device), "cudaSetDevice");
            na_c[k] = eigs(*ps[k], *xs[k], tol_eig);
          } catch (...) {
            err[k] = std::current_exception();
          }
        });
    }
    // H_AC eigensolve (eigs_rs "SA", x0 = AC)
    std::exception_ptr err_ac;
    try {
      lanczos_applies += eigs(hac, AC, tol_eig);
    } catch (...) {
      err_ac = std::current_exception();
    }
    if (o_.concurrent) {
      for (std::thread& t : jobs) t.join();
    }
    if (err_ac) std::rethrow_exception(err_ac);
    if (o_.concurrent) {
      for (const std::exception_ptr& e : err)
        if (e) std::rethrow_exception(e);
      for (side_ctx& s : side_) {
        cuda_check(cudaEventRecord(s.done, s.stream), "cudaEventRecord");
        cuda_check(cudaStreamWaitEvent(nullptr, s.done, 0), "cudaStreamWaitEvent");
      }
    } else {
      na_c[0] = eigs(pl, CL, tol_eig);
      na_c[1] = eigs(pr, CR, tol_eig);
    }
    lanczos_applies += na_c[0] + na_c[1];
    check(imps_sign_normalize(c, CL.get(), CL.size()), "sign");
    check(imps_sign_normalize(c, CR.get(), CR.size()), "sign");
    if (dosvd_ && prec[n] < o_.svdthresh) dosvd_ = false;
    dvec ALnew = z(LA_[n]), ARnew = z(LA_[n]);
    if (dosvd_) {
      // polar: AL = U V^T of AC CR^T, AR = U V^T of CL^T AC (VUMPS_main.cpp:213-220), one launch
      dvec X = z(LA_[n]), X2 = z(LA_[n]);
      mul(p_mul_r_t_[n], AC, CR, X);
      mul(p_mul_l_t_[n], AC, CL, X2);
      dvec U = z(LA_[n]), V = z(rl_ac_l_[n]), U2 = z(LA_[n]), V2 = z(rl_ac_r_[n]);
      imps_plan* plans[2] = {dec_ac_l_[n].get(), dec_ac_r_[n].get()};
      const double* As[2] = {X.get(), X2.get()};
      double* Us[2] = {U.get(), U2.get()};
      double* Ss[2] = {nullptr, nullptr};
      double* Vs[2] = {V.get(), V2.get()};
      check(imps_sector_svd_batch(2, plans, As, Us, Ss, Vs, IMPS_MEM_DEVICE), "svd");
      mul(p_mul_r_[n], U, V, ALnew);
      mul(p_mul_l_[n], U2, V2, ARnew);
    } else {
      // QR scheme (VUMPS_main.cpp:221-234)
      dvec QL = z(LA_[n]), Rt = z(rl_ac_l_[n]);
      check(imps_sector_qr(dec_ac_l_[n].get(), AC.get(), QL.get(), Rt.get(), IMPS_MEM_DEVICE), "qr");
      dvec PL = z(LB_[r]), RL = z(LB_[r]);
      check(imps_sector_qr(dec_b_l_[r].get(), CR.get(), PL.get(), RL.get(), IMPS_MEM_DEVICE), "qr");
      mul(p_mul_r_t_[n], QL, PL, ALnew);
      dvec QR = z(LA_[n]), Rt2 = z(rl_ac_r_[n]);
      check(imps_sector_qr(dec_ac_r_[n].get(), AC.get(), QR.get(), Rt2.get(), IMPS_MEM_DEVICE), "qr");
      dvec PR = z(LB_[l]), RR = z(LB_[l]);
      check(imps_sector_qr(dec_b_r_[l].get(), CL.get(), PR.get(), RR.get(), IMPS_MEM_DEVICE), "qr");
      mul(p_mul_l_t_[n], QR, PR, ARnew);
    }
    // err_l = |AC - AL CR|_inf, err_r = |AC - CL AR|_inf
    dvec t = z(LA_[n]);
    mul(p_mul_r_[n], ALnew, CR, t);
    axpby(1.0, AC, -1.0, t);
    const double err_l = absmax(t);
    dvec t3 = z(LA_[n]);
    mul(p_mul_l_[n], ARnew, CL, t3);
    axpby(1.0, AC, -1.0, t3);
    const double err_r = absmax(t3);
    prec[n] = std::max(err_l, err_r);
    AL_[n] = std::move(ALnew);
    AR_[n] = std::move(ARnew);
    C_[r] = std::move(CR);
    C_[l] = std::move(CL);
    // left environment: R = CL CL^T, fixed point of [AL(n), AL(n+1)], EHL on bond n
    const double gtol = std::max(tol / o_.InvEfac, o_.InvETol);
    // the right environment: with o_.concurrent on side_[1] (its own plans and a thread) beside
    // the left chain
    env_bufs eb = env_buffers(n);
    int env_iters = 0;
    std::exception_ptr env_err;
    std::thread env_job;
    if (o_.concurrent) {
      cuda_check(cudaEventRecord(ev_main_, nullptr), "cudaEventRecord");
      cuda_check(cudaStreamWaitEvent(side_[1].stream, ev_main_, 0), "cudaStreamWaitEvent");
      env_job = std::thread([this, n, gtol, &eb, &env_iters, &env_err] {
        try {
          cuda_check(cudaSetDevice(side_[1].device), "cudaSetDevice");
          env_iters = right_env(n, gtol, chain_plans{side_[1].ctx->get(), &env_tm_, &env_optm_r_, &env_cct_}, eb);
        } catch (...) {
          env_err = std::current_exception();
        }
      });
    }
    try {
      left_env(n, gtol);
    } catch (...) {
      if (env_job.joinable()) env_job.join();
      throw;
    }
    if (o_.concurrent) {
      env_job.join();
      if (env_err) std::rethrow_exception(env_err);
      cuda_check(cudaEventRecord(side_[1].done, side_[1].stream), "cudaEventRecord");
      cuda_check(cudaStreamWaitEvent(nullptr, side_[1].done, 0), "cudaStreamWaitEvent");
    } else {
      env_iters = right_env(n, gtol, chain_plans{c, &tm_, &optm_r_, &cct_}, eb);
    }
    gmres_iters += env_iters;
    EHR_ = std::move(eb.y);
    EHL_ = std::move(EHLtmp_);
    dvec er = z(LB_[r]);
    tm(3, mm, AR_, EHR_, er);
    dvec er2 = z(LB_[r]);
    optm(false, mm, AR_, er2);
    axpby(1.0, er, 1.0, er2);
    EHR1_ = std::move(er2);
    redops(n);
  }

  // the left-environment chain of site n (VUMPS_main.cpp:236-240): EHL on bond n, EHL1, and EHL
  // shifted to bond n+1 (kept in EHLtmp_ until the right chain has finished)
  void left_env(int n, double gtol) {
    const int l = n, r = 1 - n, mm = 1 - n;
    dvec R = cct(l, true);
    if (o_.trueLR) R = tm_dominant(1, n, AL_, R, 1e-15);
    dvec HAL = get_hl(n);
    EHL_ = invert_e(0, n, AL_, HAL, eye_[l], R, 'l', &EHL_, gtol);
    // shift to site n+1: EHLtmp = OpTM(AL(n-1) AL(n)) + T_L(AL(n), EHL) on bond n+1
    dvec EHLtmp = z(LB_[r]);
    optm(true, mm, AL_, EHLtmp);
    dvec tt = z(LB_[r]);
    tm(2, n, AL_, EHL_, tt);
    axpby(1.0, EHLtmp, 1.0, tt);
    EHLtmp = std::move(tt);
    dvec e1 = z(LB_[l]);
    optm(true, n, AL_, e1);
    dvec tt2 = z(LB_[l]);
    tm(2, mm, AL_, EHLtmp, tt2);
    axpby(1.0, e1, 1.0, tt2);
    EHL1_ = std::move(tt2);
    EHLtmp_ = std::move(EHLtmp);
  }
};

}  // namespace imps_cpp
