// ORACLE -- test infrastructure only.
// Symmetric Moore-Penrose pseudoinverse with Armadillo's default tolerance
// (max(rows, cols) * largest singular value * machine epsilon), by cyclic Jacobi
// eigen-decomposition. The correlation submatrices of the reference's level tests
// (src/executor/testing/cpuRowTests.cpp:93-113) are symmetric, so their singular
// values are the absolute eigenvalues and pinv(A) = V diag(1/lambda) V^T over the
// eigenvalues above the tolerance. Shared by the oracle and by the shim that lets
// the reference's CPU sources compile without Armadillo.
#pragma once
#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

namespace orc {
inline void pinv_sym(const double *A, int k, double *P) {
  std::vector<double> a(A, A + k * k), v(k * k, 0.0);
  for (int i = 0; i < k; ++i) v[i * k + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int i = 0; i < k; ++i) {
      diag += a[i * k + i] * a[i * k + i];
      for (int j = i + 1; j < k; ++j) off += a[i * k + j] * a[i * k + j];
    }
    if (off == 0.0 || off <= 1e-34 * diag) break;
    for (int pi = 0; pi < k; ++pi) {
      for (int qi = pi + 1; qi < k; ++qi) {
        double apq = a[pi * k + qi];
        if (apq == 0.0) continue;
        double app = a[pi * k + pi], aqq = a[qi * k + qi];
        double theta = (aqq - app) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int r = 0; r < k; ++r) {
          double arp = a[r * k + pi], arq = a[r * k + qi];
          a[r * k + pi] = c * arp - s * arq;
          a[r * k + qi] = s * arp + c * arq;
        }
        for (int r = 0; r < k; ++r) {
          double apr = a[pi * k + r], aqr = a[qi * k + r];
          a[pi * k + r] = c * apr - s * aqr;
          a[qi * k + r] = s * apr + c * aqr;
        }
        for (int r = 0; r < k; ++r) {
          double vrp = v[r * k + pi], vrq = v[r * k + qi];
          v[r * k + pi] = c * vrp - s * vrq;
          v[r * k + qi] = s * vrp + c * vrq;
        }
      }
    }
  }
  double smax = 0.0;
  for (int i = 0; i < k; ++i) smax = std::max(smax, std::fabs(a[i * k + i]));
  const double tol = (double)k * smax * std::numeric_limits<double>::epsilon();
  std::fill(P, P + k * k, 0.0);
  for (int e = 0; e < k; ++e) {
    double lam = a[e * k + e];
    if (!(std::fabs(lam) > tol)) continue;
    double inv = 1.0 / lam;
    for (int i = 0; i < k; ++i)
      for (int j = 0; j < k; ++j) P[i * k + j] += v[i * k + e] * inv * v[j * k + e];
  }
}
}  // namespace orc
