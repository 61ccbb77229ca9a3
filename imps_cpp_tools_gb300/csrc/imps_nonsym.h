// Small dense nonsymmetric eigenproblems on the host: the projected matrices of the device
// Arnoldi solver (k <= 64).  Eigenvalues by Householder reduction to upper Hessenberg form and
// the Francis implicit double-shift QR iteration (Golub & Van Loan, Matrix Computations, 4th
// ed., Algorithms 7.4.2 and 7.5.2, with the deflation test of section 7.5.1 and ad hoc shifts
// after 10 and 20 steps without deflation); eigenvectors by inverse iteration on the original
// matrix in complex arithmetic (ibid. section 7.6.1).  Header-only, so that the test shim
// compiles it with g++ alone.
#pragma once
#include <algorithm>
#include <cmath>
#include <complex>
#include <limits>
#include <vector>

namespace imps {

using cplx = std::complex<double>;

// Householder reduction of the k x k column-major matrix A to upper Hessenberg form, in place
// (the reflectors are not kept: the result serves the eigenvalue iteration only).
inline void hess_reduce(int k, double* A) {
  std::vector<double> v(k);
  auto a = [&](int i, int j) -> double& { return A[i + (size_t)j * k]; };
  for (int j = 0; j + 2 < k; ++j) {
    double s = 0.0;
    for (int i = j + 1; i < k; ++i) s += a(i, j) * a(i, j);
    const double nr = std::sqrt(s);
    if (nr == 0.0) continue;
    const double x0 = a(j + 1, j);
    const double beta = x0 >= 0.0 ? -nr : nr;  // the new subdiagonal entry
    v[j + 1] = x0 - beta;
    double vv = v[j + 1] * v[j + 1];
    for (int i = j + 2; i < k; ++i) {
      v[i] = a(i, j);
      vv += v[i] * v[i];
    }
    if (vv == 0.0) continue;
    const double sc = 2.0 / vv;
    for (int c = j + 1; c < k; ++c) {  // A <- P A (column j is set explicitly below)
      double t = 0.0;
      for (int i = j + 1; i < k; ++i) t += v[i] * a(i, c);
      t *= sc;
      for (int i = j + 1; i < k; ++i) a(i, c) -= t * v[i];
    }
    for (int r = 0; r < k; ++r) {  // A <- A P
      double t = 0.0;
      for (int i = j + 1; i < k; ++i) t += a(r, i) * v[i];
      t *= sc;
      for (int i = j + 1; i < k; ++i) a(r, i) -= t * v[i];
    }
    a(j + 1, j) = beta;
    for (int i = j + 2; i < k; ++i) a(i, j) = 0.0;
  }
}

// Eigenvalues (wr + i wi) of the k x k upper Hessenberg matrix H (column-major, overwritten).
// Complex eigenvalues come in adjacent conjugate pairs, positive imaginary part first.  Only
// the active diagonal window is updated (the eigenvalues of a block triangular matrix are
// those of its diagonal blocks).  Returns false if the iteration did not converge within
// 30 k double-shift steps.
inline bool hess_eigvals(int k, double* H, double* wr, double* wi) {
  auto h = [&](int i, int j) -> double& { return H[i + (size_t)j * k]; };
  const double eps = std::numeric_limits<double>::epsilon();
  double hn = 0.0;
  for (int j = 0; j < k; ++j)
    for (int i = 0; i <= std::min(j + 1, k - 1); ++i) hn += h(i, j) * h(i, j);
  hn = std::sqrt(hn);
  int u = k - 1, its = 0, total = 0;
  while (u >= 0) {
    int l = u;
    for (; l > 0; --l) {  // deflation: a negligible subdiagonal entry splits the problem
      double s = std::fabs(h(l - 1, l - 1)) + std::fabs(h(l, l));
      if (s == 0.0) s = hn;
      if (std::fabs(h(l, l - 1)) <= eps * s) {
        h(l, l - 1) = 0.0;
        break;
      }
    }
    if (l == u) {
      wr[u] = h(u, u);
      wi[u] = 0.0;
      --u;
      its = 0;
      continue;
    }
    if (l == u - 1) {  // 2 x 2 block: lambda = d + mu with mu^2 - 2 p mu - b c = 0
      const double a = h(u - 1, u - 1), b = h(u - 1, u), c = h(u, u - 1), d = h(u, u);
      const double p = 0.5 * (a - d), q = p * p + b * c;
      if (q >= 0.0) {
        const double mu = p + std::copysign(std::sqrt(q), p);
        wr[u - 1] = d + mu;
        wr[u] = mu != 0.0 ? d - b * c / mu : d + mu;
        wi[u - 1] = wi[u] = 0.0;
      } else {
        wr[u - 1] = wr[u] = d + p;
        wi[u - 1] = std::sqrt(-q);
        wi[u] = -wi[u - 1];
      }
      u -= 2;
      its = 0;
      continue;
    }
    if (total >= 30 * k) return false;
    ++its;
    ++total;
    double s, t;  // sum and product of the two shifts
    if (its == 10 || its == 20) {
      const double ex = std::fabs(h(u, u - 1)) + std::fabs(h(u - 1, u - 2));
      s = 1.5 * ex;
      t = ex * ex;
    } else {
      s = h(u - 1, u - 1) + h(u, u);
      t = h(u - 1, u - 1) * h(u, u) - h(u - 1, u) * h(u, u - 1);
    }
    // first column of (H - s1)(H - s2), then chase the bulge down the window
    double x = h(l, l) * h(l, l) + h(l, l + 1) * h(l + 1, l) - s * h(l, l) + t;
    double y = h(l + 1, l) * (h(l, l) + h(l + 1, l + 1) - s);
    double z = h(l + 1, l) * h(l + 2, l + 1);
    for (int q = l; q <= u - 2; ++q) {
      const double nr = std::sqrt(x * x + y * y + z * z);
      if (nr != 0.0) {
        const double al = x >= 0.0 ? -nr : nr;
        const double v0 = x - al, v1 = y, v2 = z;
        const double sc = 2.0 / (v0 * v0 + v1 * v1 + v2 * v2);
        for (int c = std::max(l, q - 1); c <= u; ++c) {
          const double r = sc * (v0 * h(q, c) + v1 * h(q + 1, c) + v2 * h(q + 2, c));
          h(q, c) -= r * v0;
          h(q + 1, c) -= r * v1;
          h(q + 2, c) -= r * v2;
        }
        for (int r = l; r <= std::min(q + 3, u); ++r) {
          const double w = sc * (h(r, q) * v0 + h(r, q + 1) * v1 + h(r, q + 2) * v2);
          h(r, q) -= w * v0;
          h(r, q + 1) -= w * v1;
          h(r, q + 2) -= w * v2;
        }
        if (q > l) h(q + 1, q - 1) = h(q + 2, q - 1) = 0.0;
      }
      x = h(q + 1, q);
      y = h(q + 2, q);
      if (q < u - 2) z = h(q + 3, q);
    }
    const double nr = std::sqrt(x * x + y * y);  // last 2-row reflector
    if (nr != 0.0) {
      const double al = x >= 0.0 ? -nr : nr;
      const double v0 = x - al, v1 = y;
      const double sc = 2.0 / (v0 * v0 + v1 * v1);
      for (int c = std::max(l, u - 2); c <= u; ++c) {
        const double r = sc * (v0 * h(u - 1, c) + v1 * h(u, c));
        h(u - 1, c) -= r * v0;
        h(u, c) -= r * v1;
      }
      for (int r = l; r <= u; ++r) {
        const double w = sc * (h(r, u - 1) * v0 + h(r, u) * v1);
        h(r, u - 1) -= w * v0;
        h(r, u) -= w * v1;
      }
      if (u - 2 >= l) h(u, u - 2) = 0.0;
    }
  }
  return true;
}

// Eigenvalues of a general k x k matrix G (column-major, not modified).
inline bool dense_eigvals(int k, const double* G, double* wr, double* wi) {
  std::vector<double> H(G, G + (size_t)k * k);
  hess_reduce(k, H.data());
  return hess_eigvals(k, H.data(), wr, wi);
}

// Eigenvector y (unit 2-norm, largest component real and positive) of the real k x k matrix G
// for its eigenvalue lam: three steps of inverse iteration with the LU factors of G - lam I
// (partial pivoting; a zero pivot is replaced by eps |G|).
inline void dense_eigvec(int k, const double* G, double gnorm, cplx lam, cplx* y) {
  std::vector<cplx> M((size_t)k * k);
  std::vector<int> piv(k);
  auto m = [&](int i, int j) -> cplx& { return M[i + (size_t)j * k]; };
  for (int j = 0; j < k; ++j)
    for (int i = 0; i < k; ++i) m(i, j) = cplx(G[i + (size_t)j * k], 0.0) - (i == j ? lam : cplx(0.0));
  const double tiny = std::numeric_limits<double>::epsilon() * std::max(gnorm, 1e-300);
  for (int j = 0; j < k; ++j) {
    int pr = j;
    for (int i = j + 1; i < k; ++i)
      if (std::abs(m(i, j)) > std::abs(m(pr, j))) pr = i;
    piv[j] = pr;
    if (pr != j)
      for (int c = 0; c < k; ++c) std::swap(m(j, c), m(pr, c));
    if (std::abs(m(j, j)) < tiny) m(j, j) = tiny;
    for (int i = j + 1; i < k; ++i) {
      const cplx f = m(i, j) / m(j, j);
      m(i, j) = f;
      for (int c = j + 1; c < k; ++c) m(i, c) -= f * m(j, c);
    }
  }
  // start vector: not orthogonal to any eigenvector in practice
  for (int i = 0; i < k; ++i) y[i] = cplx(1.0 + 0.37 * std::sin(1.0 + 3.1 * i), 0.0);
  for (int it = 0; it < 3; ++it) {
    for (int j = 0; j < k; ++j)
      if (piv[j] != j) std::swap(y[j], y[piv[j]]);
    for (int i = 1; i < k; ++i)
      for (int j = 0; j < i; ++j) y[i] -= m(i, j) * y[j];
    for (int i = k - 1; i >= 0; --i) {
      for (int j = i + 1; j < k; ++j) y[i] -= m(i, j) * y[j];
      y[i] /= m(i, i);
    }
    double nr = 0.0;
    for (int i = 0; i < k; ++i) nr += std::norm(y[i]);
    nr = std::sqrt(nr);
    if (!(nr > 0.0) || !std::isfinite(nr)) break;
    for (int i = 0; i < k; ++i) y[i] /= nr;
  }
  int imax = 0;
  for (int i = 1; i < k; ++i)
    if (std::abs(y[i]) > std::abs(y[imax]) * (1.0 + 1e-12)) imax = i;
  const cplx ph = std::abs(y[imax]) > 0.0 ? std::conj(y[imax]) / std::abs(y[imax]) : cplx(1.0);
  for (int i = 0; i < k; ++i) y[i] *= ph;
}

// Order of the eigenvalues for the Arnoldi "which" codes: 0 largest modulus (LM), 1 largest
// real part (LR), 2 smallest real part (SR).  Conjugate pairs stay adjacent, +im first.
inline std::vector<int> order_ritz(int k, const double* wr, const double* wi, int which) {
  std::vector<int> idx(k);
  for (int i = 0; i < k; ++i) idx[i] = i;
  auto key = [&](int i) {
    if (which == 0) return -std::hypot(wr[i], wi[i]);
    if (which == 1) return -wr[i];
    return wr[i];
  };
  // (the two members of a conjugate pair come from one 2 x 2 block with identical real parts,
  // so their keys compare equal exactly)
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) {
    const double ka = key(a), kb = key(b);
    if (ka != kb) return ka < kb;
    if (wr[a] != wr[b]) return wr[a] > wr[b];
    return wi[a] > wi[b];
  });
  return idx;
}

}  // namespace imps
