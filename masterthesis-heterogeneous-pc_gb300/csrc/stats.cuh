// Fisher-z independence statistics and subset combinatorics, compiled for the
// host and the device from the same source.
//
// FP64 formulas follow the reference's CPU path exactly
// (src/executor/independence/cpuInd.cpp:8-38), because accept/reject decisions
// must match it: p = 2 * upper-tail(|z|) with |z| = sqrt(n-3) * 0.5 *
// log1p(2r/(1-r)), |r| clamped to 0.9999999, NaN r -> 0; an edge is removed iff
// p >= alpha. The upper tail of the standard normal is erfc(z / sqrt 2) / 2.
#pragma once
#include <math.h>
#include <stdint.h>

#include "../../include/heterogpc.h"

#define HPC_HD __host__ __device__ __forceinline__

namespace hpc {

HPC_HD double calc_pvalue64(double r_in, int n) {
  double r = isnan(r_in) ? 0.0 : fmin(0.9999999, fabs(r_in));
  double absz = sqrt(n - 3.0) * 0.5 * log1p(2.0 * r / (1.0 - r));
  return 2.0 * (erfc(absz / 1.41421356237309504880) / 2.0);
}

// The same formula in FP32, for the record p-value of a removal decided in FP32 from
// its FP32 |r| (which carries FP32 rounding anyway; a removal's p-value is at least
// alpha, far from FP32's underflow): log1pf / erfcf instead of their FP64 versions on
// this GPU's 1/64-rate FP64 pipe.
HPC_HD float calc_pvalue32(float r_in, int n) {
  const float r = isnan(r_in) ? 0.f : fminf(0.9999999f, fabsf(r_in));
  const float absz = sqrtf((float)n - 3.0f) * 0.5f * log1pf(2.0f * r / (1.0f - r));
  return erfcf(absz * 0.707106781186547524f);
}

// closed-form level-1 partial correlation (cpuInd.cpp:16-27)
HPC_HD double pval_l1_64(double x1, double x2, double x3, int n) {
  double r = (x1 - x2 * x3) / sqrt((1.0 - x3 * x3) * (1.0 - x2 * x2));
  if (isnan(x1) || isnan(x2) || isnan(x3)) return nan("");
  return calc_pvalue64(r, n);
}

// Corner entries P00, P01, P11 of the Moore-Penrose inverse of a symmetric k x k
// matrix (row-major) with tolerance k * max|eigenvalue| * eps, by cyclic Jacobi
// rotations. This is the definition of arma::pinv (the singular values of a
// symmetric matrix are its absolute eigenvalues), and those three entries are all
// the partial correlation -P01 / sqrt(P00 * P11) needs (cpuInd.cpp:35-36). Used only
// for submatrices too ill-conditioned for a Cholesky factorisation. `a` (k*k) is
// overwritten; `v` is k*k scratch.
HPC_HD void pinv_sym64_corner(double *a, int k, double *v, double *p00, double *p01, double *p11) {
  for (int i = 0; i < k * k; ++i) v[i] = 0.0;
  for (int i = 0; i < k; ++i) v[i * k + i] = 1.0;
  for (int sweep = 0; sweep < 60; ++sweep) {
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
        double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
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
  for (int i = 0; i < k; ++i) smax = fmax(smax, fabs(a[i * k + i]));
  const double tol = (double)k * smax * 2.220446049250313e-16;
  double s00 = 0.0, s01 = 0.0, s11 = 0.0;
  for (int e = 0; e < k; ++e) {
    double lam = a[e * k + e];
    if (!(fabs(lam) > tol)) continue;
    double inv = 1.0 / lam;
    s00 += v[e] * inv * v[e];
    s01 += v[e] * inv * v[k + e];
    s11 += v[k + e] * inv * v[k + e];
  }
  *p00 = s00;
  *p01 = s01;
  *p11 = s11;
}

// Binomial coefficient, saturating at UINT64_MAX (src/util/cuda_util.cu:20-32
// computes the same product without the saturation).
HPC_HD unsigned long long binom_sat(int n, int k) {
  if (k < 0 || n < k) return 0ull;
  if (k > n - k) k = n - k;
  unsigned long long res = 1ull;
  for (int i = 0; i < k; ++i) {
    unsigned long long num = (unsigned long long)(n - i);
    // res * num / (i+1) is exact at every step; guard the multiplication
    if (res > 0xFFFFFFFFFFFFFFFFull / num) return 0xFFFFFFFFFFFFFFFFull;
    res = res * num / (unsigned long long)(i + 1);
  }
  return res;
}

#ifdef __CUDACC__
// C(n, k) for n < 64 and k <= HPC_MAX_LEVEL (Pascal's triangle at compile time; the
// largest entry, C(63, 32) = 9.2e17, fits 64 bits). Lookups replace binom_sat's
// 64-bit divisions on the CI-test path.
struct BinomTable {
  unsigned long long v[64][HPC_MAX_LEVEL + 1];
  constexpr BinomTable() : v() {
    v[0][0] = 1ull;
    for (int n = 1; n < 64; ++n) {
      v[n][0] = 1ull;
      for (int k = 1; k <= HPC_MAX_LEVEL; ++k) v[n][k] = v[n - 1][k - 1] + v[n - 1][k];
    }
  }
};
static __device__ const BinomTable kBinomTab = BinomTable();
static constexpr BinomTable kBinomHostTab = BinomTable();

HPC_HD unsigned long long binom_table(int n, int k) {
#ifdef __CUDA_ARCH__
  return __ldg(&kBinomTab.v[n][k]);
#else
  return kBinomHostTab.v[n][k];
#endif
}

HPC_HD unsigned long long umul64hi(unsigned long long a, unsigned long long b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (unsigned long long)(((unsigned __int128)a * b) >> 64);
#endif
}

// C(n, k) for k <= HPC_MAX_LEVEL: the table below n = 64, else the product
// C(n, q + 1) = C(n, q) (n - q) / (q + 1) with the loop unrolled, so that every
// division is by a constant (a multiply-high, not a 64-bit division routine).
// Saturates at UINT64_MAX when a partial product overflows (the work of such a row
// does not fit 64 bits either and is rejected by the test-count scan).
HPC_HD unsigned long long binom_fast(int n, int k) {
  if (k < 0 || n < k) return 0ull;
  if (n < 64) return binom_table(n, k);
  unsigned long long res = 1ull;
#pragma unroll
  for (int q = 0; q < HPC_MAX_LEVEL; ++q) {
    if (q < k) {
      const unsigned long long num = (unsigned long long)(n - q);
      if (umul64hi(res, num) != 0ull) return 0xFFFFFFFFFFFFFFFFull;
      res = res * num / (unsigned long long)(q + 1);
    }
  }
  return res;
}

// unrank_lex (below) in O(l log m) binomials: the subsets whose member i lies in
// [a, x] number C(m - a, k + 1) - C(m - x - 1, k + 1) (k = l - i - 1, the hockey-stick
// identity), so member i is the smallest x with C(m - x - 1, k + 1) < C(m - a, k + 1) -
// rank, found by bisection (C(m - x - 1, k + 1) falls as x grows). Below m = 64 the
// members are found by a forward scan of table lookups.
HPC_HD void unrank_lex_fast(unsigned long long rank, int l, int m, int *pos) {
  int x = 0;
  if (m < 64) {
    for (int i = 0; i < l; ++i) {
      for (;;) {
        const unsigned long long cnt = binom_fast(m - x - 1, l - i - 1);
        if (rank < cnt) {
          pos[i] = x;
          ++x;
          break;
        }
        rank -= cnt;
        ++x;
      }
    }
    return;
  }
  for (int i = 0; i < l; ++i) {
    const int k1 = l - i;  // k + 1
    const unsigned long long all = binom_fast(m - x, k1);
    const unsigned long long R = all - rank;  // > 0: rank < C(m - x, l - i)
    int lo = x, hi = m - k1;                  // C(m - hi - 1, k1) = C(k1 - 1, k1) = 0 < R
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (binom_fast(m - mid - 1, k1) < R) hi = mid; else lo = mid + 1;
    }
    pos[i] = lo;
    rank -= all - binom_fast(m - lo, k1);  // subsets with member i in [x, lo)
    x = lo + 1;
  }
}
#endif

// Lexicographic unranking of an l-subset of {0, .., m-1}: rank -> ascending
// positions. The same order as ithCombination (src/util/cuda_util.cu:34-50),
// which returns the positions 1-based.
HPC_HD void unrank_lex(unsigned long long rank, int l, int m, int *pos) {
  int x = 0;
  for (int i = 0; i < l; ++i) {
    for (;;) {
      unsigned long long cnt = binom_sat(m - x - 1, l - i - 1);
      if (rank < cnt) { pos[i] = x; ++x; break; }
      rank -= cnt;
      ++x;
    }
  }
}

// Next subset in lexicographic order; returns the lowest changed index, or -1
// when pos was the last subset.
HPC_HD int next_lex(int l, int m, int *pos) {
  int i = l - 1;
  while (i >= 0 && pos[i] == m - l + i) --i;
  if (i < 0) return -1;
  ++pos[i];
  for (int j = i + 1; j < l; ++j) pos[j] = pos[j - 1] + 1;
  return i;
}

}  // namespace hpc
