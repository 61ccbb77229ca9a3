// C++ host code over the C ABI (include/imps_gb300.hpp), as a reference call site would use it:
// a two-site U(1) unit cell made left-canonical by the device QR (qr(R, MPS, l)), then
//   * the left-isometry identity T_L(1) = 1 through the TMMultDiag functor,
//   * the right fixed point by TMDominantEig and T_R(R) = R,
//   * the dominant eigenvalue 1 of T_R by eigs_n ("LM"),
//   * InvertE_proj (dir l) checked through the InvEfun_proj functor.
// Exit status 0 when every check passes.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <map>
#include <random>
#include <vector>

#include "../../include/imps_gb300.hpp"

using imps_cpp::block;
using imps_cpp::layout;
using imps_cpp::plan;

static std::vector<block> mps_blocks(const std::map<int, int>& dl, const std::map<int, int>& dr) {
  // physical index s = 0, 1 adds the charge label +1, -1 (XXZ's I2K in 2 Sz units)
  std::vector<block> out;
  for (int s = 0; s < 2; ++s)
    for (const auto& [q, m] : dl) {
      const int qo = q + (s == 0 ? 1 : -1);
      auto it = dr.find(qo);
      if (it != dr.end()) out.push_back(block{s, {q}, {qo}, m, it->second});
    }
  return out;
}

static std::vector<block> bd_blocks(const std::map<int, int>& d) {
  std::vector<block> out;
  for (const auto& [q, m] : d) out.push_back(block{0, {q}, {q}, m, m});
  return out;
}

static std::vector<double> identity(const std::map<int, int>& d) {
  std::vector<double> v;
  for (const auto& [q, m] : d)
    for (int j = 0; j < m; ++j)
      for (int i = 0; i < m; ++i) v.push_back(i == j ? 1.0 : 0.0);
  return v;
}

static double maxdiff(const std::vector<double>& a, const std::vector<double>& b) {
  double e = 0.0;
  for (size_t i = 0; i < a.size(); ++i) e = std::fmax(e, std::fabs(a[i] - b[i]));
  return e;
}

static double trace_prod(const std::map<int, int>& d, const std::vector<double>& X, const std::vector<double>& Y) {
  double t = 0.0;
  size_t o = 0;
  for (const auto& [q, m] : d) {
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) t += X[o + i + (size_t)j * m] * Y[o + j + (size_t)i * m];
    o += (size_t)m * m;
  }
  return t;
}

int main() {
  bool ok = true;
  try {
    imps_cpp::context ctx(0);
    const std::map<int, int> b0 = {{-2, 3}, {0, 5}, {2, 3}}, b1 = {{-3, 1}, {-1, 4}, {1, 4}, {3, 1}};
    layout LA0(1, mps_blocks(b0, b1)), LA1(1, mps_blocks(b1, b0)), LB0(1, bd_blocks(b0));
    const int64_t n0 = LA0.nelem(), n1 = LA1.nelem(), nb = LB0.nelem();
    // random tensors, made left-canonical on the device
    std::mt19937_64 rng(7);
    std::normal_distribution<double> g;
    std::vector<double> a0(n0), a1(n1);
    for (double& x : a0) x = g(rng);
    for (double& x : a1) x = g(rng);
    double *dA0, *dA1, *dQ0, *dQ1, *dR0, *dR1;
    cudaMalloc(&dA0, n0 * 8);
    cudaMalloc(&dA1, n1 * 8);
    cudaMalloc(&dQ0, n0 * 8);
    cudaMalloc(&dQ1, n1 * 8);
    cudaMemcpy(dA0, a0.data(), n0 * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(dA1, a1.data(), n1 * 8, cudaMemcpyHostToDevice);
    plan dec0 = plan::decomp(ctx, LA0, IMPS_DIR_LEFT), dec1 = plan::decomp(ctx, LA1, IMPS_DIR_LEFT);
    imps_layout *R0l, *R1l;
    imps_cpp::check(imps_plan_derived_layout(dec0.get(), 1, &R0l), "derived layout");
    imps_cpp::check(imps_plan_derived_layout(dec1.get(), 1, &R1l), "derived layout");
    cudaMalloc(&dR0, imps_layout_nelem(R0l) * 8);
    cudaMalloc(&dR1, imps_layout_nelem(R1l) * 8);
    imps_cpp::qr(dec0, dA0, dQ0, dR0);
    imps_cpp::qr(dec1, dA1, dQ1, dR1);
    // transfer matrices of the unit cell [AL0, AL1]
    plan tmL = plan::tm(ctx, {&LA0, &LA1}, IMPS_DIR_LEFT, LB0, LB0);
    plan tmR = plan::tm(ctx, {&LA0, &LA1}, IMPS_DIR_RIGHT, LB0, LB0);
    for (plan* p : {&tmL, &tmR}) {
      p->bind(2, dQ0);
      p->bind(3, dQ1);
    }
    // 1. left isometry
    imps_cpp::multop TL = imps_cpp::TMMultDiag(tmL), TR = imps_cpp::TMMultDiag(tmR);
    std::vector<double> I = identity(b0), TI(nb);
    TL(I.data(), TI.data());
    const double e1 = maxdiff(TI, I);
    // 2. right fixed point
    std::vector<double> R(nb), TRR(nb);
    const double lam = imps_cpp::TMDominantEig(tmR, R.data(), 1e-14);
    TR(R.data(), TRR.data());
    const double e2 = maxdiff(TRR, R);
    // 3. dominant eigenvalue by the device Arnoldi
    int na = 0;
    const auto ev = imps_cpp::eigs_n(tmR, 2, "LM", 1e-12, &na);
    const double e3 = std::hypot(ev[0].first - 1.0, ev[0].second);
    // 4. InvertE_proj, dir l: y (1 - T + |R)(1|) = x (1 - |R)(1|); check with InvEfun_proj
    //    (out = y - T(y) + tr(y rho_in) rho_out, rho_in = R, rho_out = 1 for dir l)
    std::vector<double> x(nb), y(nb, 0.0), Ay(nb);
    for (double& v : x) v = g(rng);
    int it = 0;
    const int st = imps_cpp::InvertE_proj(tmL, x.data(), I.data(), R.data(), 'l', y.data(), 1e-12, 0, &it);
    imps_cpp::multop A = imps_cpp::InvEfun_proj(tmL, R.data(), I.data());
    A(y.data(), Ay.data());
    const double tx = trace_prod(b0, x, R);
    std::vector<double> b(nb);
    for (int64_t i = 0; i < nb; ++i) b[i] = x[i] - tx * I[i];
    double rn = 0.0, bn = 0.0;
    for (int64_t i = 0; i < nb; ++i) {
      rn += (Ay[i] - b[i]) * (Ay[i] - b[i]);
      bn += b[i] * b[i];
    }
    const double e4 = std::sqrt(rn / bn);
    std::printf("left isometry |T_L(1) - 1| = %.2e\n", e1);
    std::printf("TMDominantEig lambda = %.15f, |T_R(R) - R| = %.2e\n", lam, e2);
    std::printf("eigs_n LM: %.15f %+.2ei, %.6f %+.6fi (%d applies)\n", ev[0].first, ev[0].second, ev[1].first,
                ev[1].second, na);
    std::printf("InvertE_proj status %d, %d iterations, relative residual through InvEfun_proj %.2e\n", st, it, e4);
    ok = e1 < 1e-12 && e2 < 1e-12 && std::fabs(lam - 1.0) < 1e-12 && e3 < 1e-10 && st == 0 && e4 < 1e-10;
    imps_layout_destroy(R0l);
    imps_layout_destroy(R1l);
    for (double* p : {dA0, dA1, dQ0, dQ1, dR0, dR1}) cudaFree(p);
  } catch (const imps_cpp::error& e) {
    std::printf("error: %s\n", e.what());
    ok = false;
  }
  std::printf(ok ? "cpp host check ok\n" : "cpp host check FAILED\n");
  return ok ? 0 : 1;
}
