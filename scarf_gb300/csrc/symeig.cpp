// Host symmetric eigensolver for the small FP64 Rayleigh-Ritz problems of the
// PCA basis (tens to a few hundred rows), where a GPU solver is bound by
// launch latency: Householder reduction to tridiagonal form with the
// orthogonal transform accumulated, then the implicit QL iteration with a
// Wilkinson-type shift, rotations accumulated into the transform (Golub and
// Van Loan, Matrix Computations, 4th ed., sections 8.3.1-8.3.5).
#include "symeig.h"

#include <algorithm>
#include <limits>
#include <cmath>
#include <vector>

namespace sg {

int symeig_host(int n, const double* A, double* w, double* V) {
  if (n <= 0) return 0;
  // a: full symmetric working copy, row-major; q: the accumulated transform,
  // column-major (column j at q[j * n]), so rotations touch contiguous columns
  const size_t N = static_cast<size_t>(n);
  std::vector<double> a(N * N), q(N * N, 0.0), v(N), p(N), t(N);
  for (int j = 0; j < n; ++j)
    for (int i = j; i < n; ++i) a[size_t(i) * n + j] = a[size_t(j) * n + i] = A[size_t(j) * n + i];
  for (int i = 0; i < n; ++i) q[size_t(i) * n + i] = 1.0;
  // Householder: zero column k below its subdiagonal, k = 0 .. n-3
  for (int k = 0; k + 2 < n; ++k) {
    const int r = n - k - 1;  // size of the trailing block
    double norm2 = 0.0;
    for (int i = 0; i < r; ++i) {
      v[size_t(i)] = a[size_t(k + 1 + i) * n + k];
      norm2 += v[size_t(i)] * v[size_t(i)];
    }
    if (norm2 == 0.0) continue;
    const double norm = std::sqrt(norm2);
    const double alpha = v[0] > 0.0 ? -norm : norm;
    v[0] -= alpha;
    double vv = 0.0;
    for (int i = 0; i < r; ++i) vv += v[size_t(i)] * v[size_t(i)];
    if (vv == 0.0) continue;
    const double beta = 2.0 / vv;
    // p = beta T v, K = beta/2 p.v, w = p - K v; T -= v w^T + w v^T
    double pv = 0.0;
    for (int i = 0; i < r; ++i) {
      const double* row = &a[size_t(k + 1 + i) * n + (k + 1)];
      double s = 0.0;
      for (int j = 0; j < r; ++j) s += row[j] * v[size_t(j)];
      p[size_t(i)] = beta * s;
      pv += p[size_t(i)] * v[size_t(i)];
    }
    const double K = 0.5 * beta * pv;
    for (int i = 0; i < r; ++i) p[size_t(i)] -= K * v[size_t(i)];
    for (int i = 0; i < r; ++i) {
      double* row = &a[size_t(k + 1 + i) * n + (k + 1)];
      for (int j = 0; j < r; ++j) row[j] -= v[size_t(i)] * p[size_t(j)] + p[size_t(i)] * v[size_t(j)];
    }
    a[size_t(k + 1) * n + k] = a[size_t(k) * n + (k + 1)] = alpha;
    for (int i = 1; i < r; ++i) a[size_t(k + 1 + i) * n + k] = a[size_t(k) * n + (k + 1 + i)] = 0.0;
    // q <- q H on columns k+1 ..: t = q[:, k+1:] v, then q[:, k+1+j] -= beta v_j t
    std::fill(t.begin(), t.end(), 0.0);
    for (int j = 0; j < r; ++j) {
      const double* col = &q[size_t(k + 1 + j) * n];
      const double vj = v[size_t(j)];
      for (int i = 0; i < n; ++i) t[size_t(i)] += col[i] * vj;
    }
    for (int j = 0; j < r; ++j) {
      double* col = &q[size_t(k + 1 + j) * n];
      const double bv = beta * v[size_t(j)];
      for (int i = 0; i < n; ++i) col[i] -= bv * t[size_t(i)];
    }
  }
  std::vector<double> d(N), e(N, 0.0);
  for (int i = 0; i < n; ++i) d[size_t(i)] = a[size_t(i) * n + i];
  for (int i = 0; i + 1 < n; ++i) e[size_t(i)] = a[size_t(i + 1) * n + i];
  // implicit QL: e[i] couples d[i] and d[i+1]
  const double eps = std::numeric_limits<double>::epsilon();
  for (int l = 0; l < n; ++l) {
    for (int iter = 0;; ++iter) {
      int m = l;
      for (; m + 1 < n; ++m) {
        const double dd = std::fabs(d[size_t(m)]) + std::fabs(d[size_t(m + 1)]);
        if (std::fabs(e[size_t(m)]) <= eps * dd) break;
      }
      if (m == l) break;
      if (iter >= 60) return 1;
      // shift from the leading 2 x 2 of the unreduced block
      double g = (d[size_t(l + 1)] - d[size_t(l)]) / (2.0 * e[size_t(l)]);
      double r = std::hypot(g, 1.0);
      g = d[size_t(m)] - d[size_t(l)] + e[size_t(l)] / (g + (g >= 0.0 ? r : -r));
      double s = 1.0, c = 1.0, pp = 0.0;
      bool early = false;
      for (int i = m - 1; i >= l; --i) {
        const double f = s * e[size_t(i)], b = c * e[size_t(i)];
        r = std::hypot(f, g);
        e[size_t(i + 1)] = r;
        if (r == 0.0) {  // the block splits: restart with the same l
          d[size_t(i + 1)] -= pp;
          e[size_t(m)] = 0.0;
          early = true;
          break;
        }
        s = f / r;
        c = g / r;
        g = d[size_t(i + 1)] - pp;
        r = (d[size_t(i)] - g) * s + 2.0 * c * b;
        pp = s * r;
        d[size_t(i + 1)] = g + pp;
        g = c * r - b;
        double* c0 = &q[size_t(i) * n];
        double* c1 = &q[size_t(i + 1) * n];
        for (int k = 0; k < n; ++k) {
          const double x = c0[k], y = c1[k];
          c1[k] = s * x + c * y;
          c0[k] = c * x - s * y;
        }
      }
      if (early) continue;
      d[size_t(l)] -= pp;
      e[size_t(l)] = g;
      e[size_t(m)] = 0.0;
    }
  }
  // ascending order
  std::vector<int> ord(N);
  for (int i = 0; i < n; ++i) ord[size_t(i)] = i;
  std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return d[size_t(x)] < d[size_t(y)]; });
  for (int j = 0; j < n; ++j) {
    const int src = ord[size_t(j)];
    w[j] = d[size_t(src)];
    for (int i = 0; i < n; ++i) V[size_t(j) * n + i] = q[size_t(src) * n + i];
  }
  return 0;
}

}  // namespace sg
