// Small dense symmetric eigensolver (cyclic Jacobi, FP64) for the Davidson
// Rayleigh-Ritz step.  The subspace is at most 10x10, so the solve is done on
// the host between two device syncs; the reference calls LAPACK dsyev here
// (src/diagonalize.hpp:368-371).
#pragma once

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

namespace mpsxx {

// a: n*n row-major symmetric.  w: ascending eigenvalues.  v[i*n + j]: component i
// of eigenvector j (the column layout LAPACKE_dsyev returns in row-major mode).
inline void jacobi_eigh(int n, const std::vector<double>& a_in, std::vector<double>& w, std::vector<double>& v) {
  std::vector<double> a(a_in);
  std::vector<double> q(size_t(n) * n, 0.0);
  for (int i = 0; i < n; ++i) q[size_t(i) * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        const double x = a[size_t(i) * n + j] * a[size_t(i) * n + j];
        tot += x;
        if (i != j) off += x;
      }
    if (off <= 1e-30 * tot || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int r = p + 1; r < n; ++r) {
        const double apr = a[size_t(p) * n + r];
        if (apr == 0.0) continue;
        const double app = a[size_t(p) * n + p], arr = a[size_t(r) * n + r];
        const double theta = (arr - app) / (2.0 * apr);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {
          const double akp = a[size_t(k) * n + p], akr = a[size_t(k) * n + r];
          a[size_t(k) * n + p] = c * akp - s * akr;
          a[size_t(k) * n + r] = s * akp + c * akr;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = a[size_t(p) * n + k], ark = a[size_t(r) * n + k];
          a[size_t(p) * n + k] = c * apk - s * ark;
          a[size_t(r) * n + k] = s * apk + c * ark;
        }
        for (int k = 0; k < n; ++k) {
          const double qkp = q[size_t(k) * n + p], qkr = q[size_t(k) * n + r];
          q[size_t(k) * n + p] = c * qkp - s * qkr;
          q[size_t(k) * n + r] = s * qkp + c * qkr;
        }
      }
  }
  std::vector<int> ord(n);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(),
                   [&](int x, int y) { return a[size_t(x) * n + x] < a[size_t(y) * n + y]; });
  w.assign(n, 0.0);
  v.assign(size_t(n) * n, 0.0);
  for (int j = 0; j < n; ++j) {
    w[j] = a[size_t(ord[j]) * n + ord[j]];
    // deterministic sign: largest-magnitude component positive
    int big = 0;
    for (int i = 1; i < n; ++i)
      if (std::fabs(q[size_t(i) * n + ord[j]]) > std::fabs(q[size_t(big) * n + ord[j]])) big = i;
    const double sg = q[size_t(big) * n + ord[j]] < 0 ? -1.0 : 1.0;
    for (int i = 0; i < n; ++i) v[size_t(i) * n + j] = sg * q[size_t(i) * n + ord[j]];
  }
}

}  // namespace mpsxx
