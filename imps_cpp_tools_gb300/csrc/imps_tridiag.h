// Host-side symmetric tridiagonal eigen-routines for the projected matrix of the device
// Lanczos (abi.cu, imps_eigs_rs).  Header-only and free of CUDA so that the CPU tests compile
// them directly.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <limits>
#include <vector>

namespace imps {

// ---- projected Lanczos matrix: symmetric tridiagonal T = tridiag(a[0..k-1]; b[0..k-2]) with
// b[i] coupling rows i and i+1, k <= kMaxCols.  Eigenvalues by Sturm-sequence bisection,
// eigenvectors by inverse iteration (both O(k) per solve), so a convergence check costs
// microseconds whatever the Krylov dimension. ----
constexpr double kEps = 2.220446049250313e-16;

inline double tri_norm(int k, const double* a, const double* b) {
  double t = 0.0;
  for (int i = 0; i < k; ++i)
    t = std::max(t, std::fabs(a[i]) + (i ? std::fabs(b[i - 1]) : 0.0) + (i < k - 1 ? std::fabs(b[i]) : 0.0));
  return t;
}

// number of eigenvalues of T below x: negative pivots of the LDL^T factorisation of T - x
inline int sturm_below(int k, const double* a, const double* b, double x, double pivmin) {
  int cnt = 0;
  double d = 1.0;
  for (int i = 0; i < k; ++i) {
    d = (a[i] - x) - (i ? b[i - 1] * b[i - 1] / d : 0.0);
    if (std::fabs(d) < pivmin) d = -pivmin;
    if (d < 0.0) ++cnt;
  }
  return cnt;
}

// Gershgorin interval of T (widened by rounding) and the pivot floor of its Sturm sequences
inline void tri_bounds(int k, const double* a, const double* b, double* lo, double* hi, double* pivmin) {
  double l = a[0], h = a[0], bmax2 = 0.0;
  for (int r = 0; r < k; ++r) {
    const double rad = (r ? std::fabs(b[r - 1]) : 0.0) + (r < k - 1 ? std::fabs(b[r]) : 0.0);
    l = std::min(l, a[r] - rad);
    h = std::max(h, a[r] + rad);
    if (r < k - 1) bmax2 = std::max(bmax2, b[r] * b[r]);
  }
  *pivmin = std::numeric_limits<double>::min() * std::max(1.0, bmax2);
  const double widen = 2.0 * kEps * std::max(std::fabs(l), std::fabs(h)) + *pivmin;
  *lo = l - widen;
  *hi = h + widen;
}

// Sturm counts at kMulti shifts in lockstep: the kMulti division chains are independent, so
// their latencies overlap (one pass over T costs about one chain).
constexpr int kMulti = 8;
inline void sturm_multi(int k, const double* a, const double* b, const double* x, double pivmin, int* cnt) {
  double d[kMulti];
  int c[kMulti];
  for (int s = 0; s < kMulti; ++s) { d[s] = 1.0; c[s] = 0; }
  for (int i = 0; i < k; ++i) {
    const double bb = i ? b[i - 1] * b[i - 1] : 0.0;
    for (int s = 0; s < kMulti; ++s) {
      double di = (a[i] - x[s]) - (i ? bb / d[s] : 0.0);
      if (std::fabs(di) < pivmin) di = -pivmin;
      d[s] = di;
      c[s] += di < 0.0;
    }
  }
  for (int s = 0; s < kMulti; ++s) cnt[s] = c[s];
}

// The nlow smallest eigenvalues (ascending) by multisection: each round probes kMulti points
// (midpoints of the unconverged brackets, or an even split of the few that remain) and every
// Sturm count tightens the brackets of all wanted eigenvalues at once.
inline void tri_eigvals_lowest(int k, const double* a, const double* b, int nlow, double* w,
                               double xtol = 0.0) {
  double glo, ghi, pivmin;
  tri_bounds(k, a, b, &glo, &ghi, &pivmin);
  std::vector<double> lo(nlow, glo), hi(nlow, ghi);
  double x[kMulti];
  int cnt[kMulti];
  std::vector<int> open;
  open.reserve(nlow);
  for (int round = 0; round < 8192; ++round) {
    open.clear();
    for (int j = 0; j < nlow; ++j) {
      const bool same = !open.empty() && lo[open.back()] == lo[j] && hi[open.back()] == hi[j];
      const double tolx = std::max(2.0 * kEps * std::max(std::fabs(lo[j]), std::fabs(hi[j])) + pivmin, xtol);
      if (hi[j] - lo[j] > tolx && !same) open.push_back(j);
    }
    if (open.empty()) break;
    const int no = (int)open.size();
    if (no >= kMulti) {
      for (int s = 0; s < kMulti; ++s) x[s] = 0.5 * (lo[open[s]] + hi[open[s]]);
    } else {
      int s = 0;
      for (int q = 0; q < no; ++q) {
        const int np = kMulti / no + (q < kMulti % no ? 1 : 0);
        const double l = lo[open[q]], h = hi[open[q]];
        for (int p = 1; p <= np; ++p) x[s++] = l + (h - l) * p / (np + 1);
      }
    }
    sturm_multi(k, a, b, x, pivmin, cnt);
    for (int s = 0; s < kMulti; ++s)
      for (int j = 0; j < nlow; ++j) {
        if (cnt[s] > j) hi[j] = std::min(hi[j], x[s]);
        else lo[j] = std::max(lo[j], x[s]);
      }
  }
  for (int j = 0; j < nlow; ++j) w[j] = 0.5 * (lo[j] + hi[j]);
}

// i-th smallest eigenvalue (0-based)
inline double tri_eigval(int k, const double* a, const double* b, int i) {
  std::vector<double> w(i + 1);
  tri_eigvals_lowest(k, a, b, i + 1, w.data());
  return w[i];
}

// Unit eigenvector z of T for the eigenvalue lam: inverse iteration with a tridiagonal LU
// (partial pivoting; a zero pivot is perturbed to eps*|T|), orthogonalised after each solve
// against the earlier eigenvectors prev[:, c] (column-major, k rows) whose eigenvalues lie
// within 1e-3*|T| of lam, so that a cluster comes out orthonormal.
inline void tri_eigvec(int k, const double* a, const double* b, double lam, double tnorm, double* z,
                const double* prev, const double* prev_lam, int nprev) {
  if (k == 1) { z[0] = 1.0; return; }
  std::vector<double> d(k), du(k, 0.0), du2(k, 0.0), dl(k, 0.0), y(k);
  std::vector<char> sw(k, 0);
  const double tiny = kEps * std::max(tnorm, 1e-280);
  for (int i = 0; i < k; ++i) {
    d[i] = a[i] - lam;
    if (i < k - 1) du[i] = dl[i] = b[i];
  }
  for (int i = 0; i < k - 1; ++i) {
    if (std::fabs(d[i]) >= std::fabs(dl[i])) {
      if (std::fabs(d[i]) < tiny) d[i] = tiny;
      dl[i] /= d[i];
      d[i + 1] -= dl[i] * du[i];
    } else {  // pivot on row i+1: it moves up, row i is eliminated below it
      const double l = d[i] / dl[i];
      const double di1 = d[i + 1], dui = du[i], dui1 = i + 1 < k - 1 ? du[i + 1] : 0.0;
      d[i] = dl[i];
      du[i] = di1;
      du2[i] = dui1;
      dl[i] = l;
      sw[i] = 1;
      d[i + 1] = dui - l * di1;
      if (i + 1 < k - 1) du[i + 1] = -l * dui1;
    }
  }
  if (std::fabs(d[k - 1]) < tiny) d[k - 1] = tiny;
  for (int i = 0; i < k; ++i) z[i] = 1.0 + 0.125 * (double)((i * 7 + nprev * 3) % 11);
  std::vector<int> cl;
  for (int c = 0; c < nprev; ++c)
    if (std::fabs(prev_lam[c] - lam) <= 1e-3 * tnorm) cl.push_back(c);
  for (int it = 0; it < 4; ++it) {
    for (int i = 0; i < k; ++i) y[i] = z[i];
    for (int i = 0; i < k - 1; ++i) {
      if (sw[i]) std::swap(y[i], y[i + 1]);
      y[i + 1] -= dl[i] * y[i];
    }
    z[k - 1] = y[k - 1] / d[k - 1];
    z[k - 2] = (y[k - 2] - du[k - 2] * z[k - 1]) / d[k - 2];
    for (int i = k - 3; i >= 0; --i) z[i] = (y[i] - du[i] * z[i + 1] - du2[i] * z[i + 2]) / d[i];
    for (int pass = 0; pass < 2; ++pass)
      for (int c : cl) {
        const double* q = prev + (size_t)c * k;
        double dt = 0.0;
        for (int i = 0; i < k; ++i) dt += q[i] * z[i];
        for (int i = 0; i < k; ++i) z[i] -= dt * q[i];
      }
    double nz = 0.0;
    for (int i = 0; i < k; ++i) nz += z[i] * z[i];
    nz = std::sqrt(nz);
    if (!(nz > 0.0) || !std::isfinite(nz)) {  // start over from a unit vector
      for (int i = 0; i < k; ++i) z[i] = i == it % k ? 1.0 : 0.0;
      continue;
    }
    for (int i = 0; i < k; ++i) z[i] /= nz;
  }
}

// Thick-restart bookkeeping: the kept Ritz pairs (th[i], coupling s[i] to the residual
// direction) form an arrowhead.  A Lanczos run on diag(th) from s/|s| (full
// re-orthogonalisation) returns Q (kk x kk, column-major) with Q^T diag(th) Q =
// tridiag(qa, qb) and Q[:, 0] = s/|s|, the only column coupled to the residual direction.
// Where the Krylov space of s is exhausted (qb = 0) a fresh orthogonal direction starts the
// next block, which is then exactly decoupled.
inline void arrow_tridiag(int kk, const double* th, const double* s, double* Q, double* qa, double* qb) {
  double sn = 0.0, thn = 1e-300;
  for (int i = 0; i < kk; ++i) {
    sn += s[i] * s[i];
    thn = std::max(thn, std::fabs(th[i]));
  }
  sn = std::sqrt(sn);
  std::vector<double> r(kk);
  auto orth = [&](int t) {
    for (int pass = 0; pass < 2; ++pass)
      for (int c = 0; c < t; ++c) {
        const double* q = Q + (size_t)c * kk;
        double dt = 0.0;
        for (int i = 0; i < kk; ++i) dt += q[i] * r[i];
        for (int i = 0; i < kk; ++i) r[i] -= dt * q[i];
      }
  };
  auto normalise = [&]() {
    double nr = 0.0;
    for (int i = 0; i < kk; ++i) nr += r[i] * r[i];
    nr = std::sqrt(nr);
    for (int i = 0; i < kk; ++i) r[i] /= nr;
  };
  auto fresh = [&](int t) {  // the unit vector least represented in span(Q[:, :t])
    int best = 0;
    double bw = -1.0;
    for (int j = 0; j < kk; ++j) {
      double w = 1.0;
      for (int c = 0; c < t; ++c) w -= Q[j + (size_t)c * kk] * Q[j + (size_t)c * kk];
      if (w > bw) { bw = w; best = j; }
    }
    std::fill(r.begin(), r.end(), 0.0);
    r[best] = 1.0;
    orth(t);
    normalise();
  };
  for (int t = 0; t < kk; ++t) {
    if (t == 0) {
      if (sn > 0.0) for (int i = 0; i < kk; ++i) r[i] = s[i] / sn;
      else fresh(0);
    } else {
      const double* q1 = Q + (size_t)(t - 1) * kk;
      const double* q2 = t >= 2 ? Q + (size_t)(t - 2) * kk : nullptr;
      for (int i = 0; i < kk; ++i) r[i] = (th[i] - qa[t - 1]) * q1[i] - (q2 ? qb[t - 2] * q2[i] : 0.0);
      orth(t);
      double nr = 0.0;
      for (int i = 0; i < kk; ++i) nr += r[i] * r[i];
      nr = std::sqrt(nr);
      if (nr <= 1e-12 * thn) {
        qb[t - 1] = 0.0;
        fresh(t);
      } else {
        qb[t - 1] = nr;
        for (int i = 0; i < kk; ++i) r[i] /= nr;
      }
    }
    double at = 0.0;
    for (int i = 0; i < kk; ++i) {
      Q[i + (size_t)t * kk] = r[i];
      at += th[i] * r[i] * r[i];
    }
    qa[t] = at;
  }
}

// The nlow lowest eigenpairs (w ascending, Z column-major k x nlow): eigenvalues bracketed to
// full precision by multisection (a bracket merely as wide as 1e-9 |T| cannot separate a
// nearly degenerate lowest pair, and inverse iteration from it returns a mixture of the two),
// then inverse iteration from those shifts with the members of each cluster orthogonalised.
inline void tri_lowest_pairs(int k, const double* a, const double* b, int nlow, double* w, double* Z) {
  const double tn = std::max(tri_norm(k, a, b), 1e-300);
  tri_eigvals_lowest(k, a, b, nlow, w);
  for (int i = 0; i < nlow; ++i) tri_eigvec(k, a, b, w[i], tn, Z + (size_t)i * k, Z, w, i);
}

}  // namespace imps
