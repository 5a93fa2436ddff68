// ORACLE -- test infrastructure only. CPU restatement (FP64, OpenMP) of the
// reference's skeleton path. Only the tests, the smoke check and the CPU-baseline
// legs of the benchmark load this library; the product never does.
//
// What it restates (paths relative to the milanpro/Masterthesis-Heterogeneous-PC tree):
//   correlation    src/correlation/corHelper.cu:8-116 (means, SD, PMCC; NaN skipping)
//   statistics     src/executor/independence/cpuInd.cpp:8-38 (Fisher z, closed-form
//                  level-1 partial correlation, pinv-based level >= 2)
//   level tests    src/executor/testing/cpuRowTests.cpp:5-155, generalised to any
//                  level as src/executor/testing/cpuWorkstealingTests.cpp:39-112 does
//   deletion       src/executor/testing/cpuUtil.cpp:3-48
//   row order      src/executor/cpuExecutor.cpp:80-119 (rows with length >= level,
//                  sorted by length descending, (row, col) loop, dynamic schedule 10)
//   compaction     src/independence/compact.cu:4-89 (ascending neighbour ids + count)
//   level loop     src/independence/skeleton.cpp:104-190
//   state init     src/util/state.cu:31-43
// Third-party arithmetic the reference calls, restated from its published
// definition:
//   Armadillo 10.5.1 arma::pinv (docker/Dockerfile.base:32): Moore-Penrose inverse
//     with tolerance max(rows, cols) * max singular value * machine epsilon; here by a
//     cyclic Jacobi eigen-decomposition (the submatrix is symmetric, so its singular
//     values are the absolute eigenvalues).
//   Boost.Math cdf(complement(normal(0,1), z)) = erfc(z / sqrt(2)) / 2.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <mutex>
#include <tuple>
#include <unordered_map>
#include <vector>
#include <omp.h>

#include "pinv_sym.hpp"

namespace {

constexpr double kCutThr = 0.9999999;  // cpuInd.cpp:6
constexpr int kMaxLevel = 64;

// cpuInd.cpp:8-14
double calc_pvalue(double r_in, int n) {
  double r = std::isnan(r_in) ? 0.0 : std::min(kCutThr, std::fabs(r_in));
  double absz = std::sqrt(n - 3.0) * 0.5 * std::log1p(2 * r / (1 - r));
  // 2 * cdf(complement(normal, absz)) with cdf(complement) = erfc(absz / sqrt 2) / 2
  return 2.0 * (std::erfc(absz / 1.41421356237309504880) / 2.0);
}

// cpuInd.cpp:16-27
double pval_l1(double x1, double x2, double x3, int n) {
  double r = (x1 - x2 * x3) / std::sqrt((1.0 - x3 * x3) * (1.0 - x2 * x2));
  if (std::isnan(x1) || std::isnan(x2) || std::isnan(x3)) return std::numeric_limits<double>::quiet_NaN();
  return calc_pvalue(r, n);
}

using orc::pinv_sym;

// cpuInd.cpp:29-38
double pval_ln(const double *M, int k, int n) {
  for (int i = 0; i < k * k; ++i)
    if (std::isnan(M[i])) return std::numeric_limits<double>::quiet_NaN();
  double P[(kMaxLevel + 2) * (kMaxLevel + 2)];
  pinv_sym(M, k, P);
  double r = -P[1] / std::sqrt(P[0] * P[k + 1]);
  return calc_pvalue(r, n);
}

// cuda_util.cu:20-32 (host part)
uint64_t binom(int n, int k) {
  if (n < k || k < 0) return 0;
  uint64_t res = 1;
  if (k > n - k) k = n - k;
  for (int i = 0; i < k; ++i) {
    res *= (uint64_t)(n - i);
    res /= (uint64_t)(i + 1);
  }
  return res;
}

// cuda_util.cu:34-50: 0-based rank -> 1-based ascending positions
void ith_combination(int *out, uint64_t comb_number, int level, int neighbours) {
  uint64_t sum = 0, tmp = 0;
  for (int i = 0; i < level; i++) {
    out[i] = (i > 0) ? out[i - 1] : 0;
    while (sum <= comb_number) {
      out[i]++;
      tmp = binom(neighbours - out[i], level - (i + 1));
      sum += tmp;
    }
    sum -= tmp;
  }
}

struct SepRec {
  int level;
  double pmax;
  std::vector<int> ids;
};

struct State {
  int64_t p = 0;
  int n = 0;
  double alpha = 0.05;
  double r_crit = 2.0;              // |r| with calc_pvalue == alpha
  std::vector<double> cor;          // p x p row-major
  std::vector<uint8_t> adj;         // p x p, live
  std::vector<std::vector<int>> compact;  // snapshot neighbour lists (ascending)
  std::mutex seps_lock;  // guards the map; removals at level >= 1 are rare
  std::unordered_map<int64_t, SepRec> seps;  // key i*p+j (i<j), level >= 1
  std::vector<uint8_t> l0_deleted;  // pair deleted at level 0 (i*p+j, i<j)
  std::vector<double> pmax0;        // p-value of level-0 deletions (i*p+j)
  std::atomic<int64_t> tests{0};
};

// cpuUtil.cpp:3-21
void delete_edge_l0(State &s, int col, int row, double pmax) {
  s.adj[s.p * row + col] = 0;
  s.adj[s.p * col + row] = 0;
  int64_t key = row < col ? row * s.p + col : col * s.p + row;
  s.l0_deleted[key] = 1;
  s.pmax0[key] = pmax;
}

// cpuUtil.cpp:23-48 (the last deleting test overwrites, as in the reference)
void delete_edge(State &s, int level, int col, int row, double pmax, const int *sep) {
  s.adj[s.p * row + col] = 0;
  s.adj[s.p * col + row] = 0;
  int64_t key = row < col ? row * s.p + col : col * s.p + row;
  std::lock_guard<std::mutex> g(s.seps_lock);
  SepRec &r = s.seps[key];
  r.level = level;
  r.pmax = pmax;
  r.ids.assign(sep, sep + level);
}

// cpuRowTests.cpp:5-21
void test_l0(State &s, int row, int col) {
  int64_t idx = s.p * row + col;
  if (col < row && s.adj[idx]) {
    s.tests.fetch_add(1, std::memory_order_relaxed);
    double pv = calc_pvalue(s.cor[idx], s.n);
    if (pv >= s.alpha) delete_edge_l0(s, col, row, pv);
  }
}

// cpuRowTests.cpp:23-56. The sepset stored is the conditioning variable itself;
// the reference stores adj_compact[col*p + subIndex] there (cpuRowTests.cpp:47),
// an entry of an unrelated row, which changes no edge.
void test_l1(State &s, int row, int col_slot) {
  const std::vector<int> &nb = s.compact[row];
  int row_count = (int)nb.size();
  if (!(row_count > col_slot && row_count >= 1)) return;
  int col = nb[col_slot];
  int64_t tests = 0;
  for (int next = 0; next < row_count; next++) {
    if (next == col_slot) continue;
    int k = nb[next];
    ++tests;
    double pv = pval_l1(s.cor[(int64_t)row * s.p + col], s.cor[(int64_t)row * s.p + k],
                        s.cor[(int64_t)col * s.p + k], s.n);
    if (pv >= s.alpha) {
      delete_edge(s, 1, col, row, pv, &k);
      break;
    }
    if (s.adj[(int64_t)row * s.p + col] == 0) break;
  }
  s.tests.fetch_add(tests, std::memory_order_relaxed);
}

// |r| at which calc_pvalue == alpha (p is decreasing in |r|); 2 when every r is removed
double r_crit_for(double alpha, int n) {
  double lo = 0.0, hi = kCutThr;
  if (calc_pvalue(hi, n) >= alpha) return 2.0;
  for (int it = 0; it < 200; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (calc_pvalue(mid, n) >= alpha) lo = mid; else hi = mid;
  }
  return 0.5 * (lo + hi);
}

// The test's decision p >= alpha from the k x k submatrix M (ordered i, j, S), with the
// reference's pinv formula (cpuInd.cpp:29-38) wherever it can matter: the partial
// correlation is formed by Cholesky of the S block in FP64 and decides only when the
// block is well conditioned (every pivot above 1e-8) and |r| lies outside 1e-8 relative
// of r_crit (p is monotone in |r|); otherwise, and for the p-value of every removal
// (*pv), pval_ln decides. A Cholesky |r| of a well-conditioned block differs from the
// pinv one by orders of magnitude less than that band, so the decisions are pval_ln's.
bool test_removes(const double *M, int k, int n, double alpha, double rc, double *pv) {
  const int l = k - 2;
  double Lm[kMaxLevel * kMaxLevel], wx[kMaxLevel], wy[kMaxLevel];
  bool ok = true;
  for (int i = 0; i < k * k && ok; ++i) ok = !std::isnan(M[i]);
  for (int r = 0; r < l && ok; ++r) {
    double vx = M[(r + 2) * k + 0], vy = M[(r + 2) * k + 1], d = 1.0;
    for (int c = 0; c < r; ++c) {
      double v = M[(c + 2) * k + (r + 2)];
      for (int q = 0; q < c; ++q) v -= Lm[r * kMaxLevel + q] * Lm[c * kMaxLevel + q];
      v /= Lm[c * kMaxLevel + c];
      Lm[r * kMaxLevel + c] = v;
      d -= v * v;
      vx -= v * wx[c];
      vy -= v * wy[c];
    }
    if (!(d > 1e-8)) {
      ok = false;
      break;
    }
    Lm[r * kMaxLevel + r] = std::sqrt(d);
    wx[r] = vx / Lm[r * kMaxLevel + r];
    wy[r] = vy / Lm[r * kMaxLevel + r];
  }
  if (ok) {
    double ax = 1.0, ay = 1.0, b = M[1];
    for (int q = 0; q < l; ++q) {
      ax -= wx[q] * wx[q];
      ay -= wy[q] * wy[q];
      b -= wx[q] * wy[q];
    }
    if (ax > 1e-8 && ay > 1e-8) {
      const double r = std::fabs(b / std::sqrt(ax * ay));
      if (r > rc * (1.0 + 1e-8)) return false;  // p < alpha: kept, no p-value needed
      if (r < rc * (1.0 - 1e-8)) {
        *pv = pval_ln(M, k, n);
        return true;
      }
    }
  }
  *pv = pval_ln(M, k, n);
  return *pv >= alpha;
}

// cpuRowTests.cpp:58-136 for any level (as cpuWorkstealingTests.cpp:39-112), subsets in
// ascending rank order as the row variant: the first subset by ith_combination
// (cuda_util.cu:34-50), each further one as the lexicographic successor (the next rank).
void test_ln(State &s, int level, int row, int col_slot) {
  const std::vector<int> &nb = s.compact[row];
  int row_count = (int)nb.size();
  if (!(row_count > col_slot && row_count >= level)) return;
  int col = nb[col_slot];
  int row_neighbours = row_count - 1;
  uint64_t count = binom(row_neighbours, level);
  int pos[kMaxLevel], sep[kMaxLevel];
  const int k = level + 2;
  double M[(kMaxLevel + 2) * (kMaxLevel + 2)];
  int64_t tests = 0;
  const int64_t p = s.p;
  if (count > 0) ith_combination(pos, 0, level, row_neighbours);  // 1-based positions 1..level
  for (uint64_t t = 0; t < count; ++t) {
    if (t > 0) {  // lexicographic successor of pos over 1..row_neighbours
      int q = level - 1;
      while (q >= 0 && pos[q] == row_neighbours - level + q + 1) --q;
      ++pos[q];
      for (int r = q + 1; r < level; ++r) pos[r] = pos[r - 1] + 1;
    }
    for (int ind = 0; ind < level; ++ind)
      sep[ind] = (pos[ind] - 1 >= col_slot) ? nb[pos[ind]] : nb[pos[ind] - 1];
    for (int i = 0; i < k * k; ++i) M[i] = 0.0;
    for (int i = 0; i < k; ++i) M[i * k + i] = 1.0;
    M[1] = M[k] = s.cor[row * p + col];
    for (int j = 2; j < k; ++j) {
      M[j] = M[j * k] = s.cor[row * p + sep[j - 2]];
      M[k + j] = M[j * k + 1] = s.cor[(int64_t)col * p + sep[j - 2]];
    }
    for (int i = 2; i < k; ++i)
      for (int j = i + 1; j < k; ++j)
        M[i * k + j] = M[j * k + i] = s.cor[(int64_t)sep[i - 2] * p + sep[j - 2]];
    ++tests;
    double pv = 0.0;
    if (test_removes(M, k, s.n, s.alpha, s.r_crit, &pv)) {
      delete_edge(s, level, col, row, pv, sep);
      break;
    }
    if (s.adj[(int64_t)row * p + col] == 0) break;
  }
  s.tests.fetch_add(tests, std::memory_order_relaxed);
}

// compact.cu:4-89: ascending neighbour ids of every row, snapshot of adj.
int64_t compact(State &s) {
  int64_t total = 0;
#pragma omp parallel for schedule(static) reduction(+ : total)
  for (int64_t i = 0; i < s.p; ++i) {
    std::vector<int> &nb = s.compact[i];
    nb.clear();
    for (int64_t j = 0; j < s.p; ++j)
      if (s.adj[i * s.p + j]) nb.push_back((int)j);
    total += (int64_t)nb.size();
  }
  return total;
}

bool comp_tuple(const std::tuple<int, int> &a, const std::tuple<int, int> &b) {
  return std::get<1>(a) > std::get<1>(b);
}

// cpuExecutor.cpp:80-119
void execute_level(State &s, int level, int threads) {
  std::vector<std::tuple<int, int>> rows;
  for (int64_t i = 0; i < s.p; ++i) {
    // at level 0 the reference reads the initial adj_compact slot p-1 (1, or 0 on the
    // last row's diagonal), so every row passes the `>= 0` filter
    int len = level == 0 ? 1 : (int)s.compact[i].size();
    if (len >= level) rows.push_back({(int)i, len});
  }
  std::sort(rows.begin(), rows.end(), comp_tuple);
  const int64_t nrows = (int64_t)rows.size();
  const int p = (int)s.p;
#pragma omp parallel for num_threads(threads) collapse(2) schedule(dynamic, 10)
  for (int64_t i = 0; i < nrows; i++) {
    for (int col = 0; col < p; col++) {
      int row = std::get<0>(rows[i]);
      if (level == 0)
        test_l0(s, row, col);
      else if (level == 1)
        test_l1(s, row, col);
      else
        test_ln(s, level, row, col);
    }
  }
}

// potential tests T_l at the current snapshot
int64_t potential_tests(const State &s, int level) {
  int64_t t = 0;
  for (int64_t i = 0; i < s.p; ++i) {
    int d = (int)s.compact[i].size();
    if (d >= level && d - 1 >= level) t += (int64_t)d * (int64_t)binom(d - 1, level);
  }
  return t;
}

}  // namespace

extern "C" {

struct orc_result {
  State st;
  int levels_run = 0;
  int64_t tests_per_level[kMaxLevel + 1] = {0};
  int64_t potential_per_level[kMaxLevel + 1] = {0};
  int64_t edges_after_level[kMaxLevel + 1] = {0};
  double ms_per_level[kMaxLevel + 1] = {0};
};

double orc_calc_pvalue(double r, int n) { return calc_pvalue(r, n); }
double orc_pval_l1(double x1, double x2, double x3, int n) { return pval_l1(x1, x2, x3, n); }
double orc_pval_ln(const double *M, int k, int n) {
  if (k < 2 || k > kMaxLevel + 2) return std::numeric_limits<double>::quiet_NaN();
  return pval_ln(M, k, n);
}
void orc_pinv(const double *M, int k, double *P) { pinv_sym(M, k, P); }
uint64_t orc_binom(int n, int k) { return binom(n, k); }
void orc_ith_combination(int *out, uint64_t rank, int level, int neighbours) {
  ith_combination(out, rank, level, neighbours);
}

// corHelper.cu:8-116. X column-major n x p. ref_compat = 1 rounds the SD through
// float as corHelper.cu:75 does (sqrtf of a double argument, denominator dim-1.f).
int orc_correlation(const double *X, int64_t n, int64_t p, int ref_compat, double *C) {
  if (!X || !C || n < 2 || p < 1) return 1;
  std::vector<double> mean(p), sd(p);
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < p; ++v) {
    const double *x = X + v * n;
    double s = 0.0;
    int64_t cnt = 0;
    for (int64_t k = 0; k < n; ++k)
      if (!std::isnan(x[k])) { s += x[k]; ++cnt; }
    mean[v] = s / (double)cnt;
    double ss = 0.0;
    for (int64_t k = 0; k < n; ++k)
      if (!std::isnan(x[k])) { double d = x[k] - mean[v]; ss += d * d; }
    if (ref_compat)
      sd[v] = (double)sqrtf((float)(ss / (double)((float)n - 1.f)));
    else
      sd[v] = std::sqrt(ss / (double)(n - 1));
  }
  const double denom = ref_compat ? (double)((float)n - 1.f) : (double)(n - 1);
  // corHelper.cu:98-106 evaluates ((x_a - mean_a) / sd_a) * ((x_b - mean_b) / sd_b) per
  // sample, skipping samples where either value is NaN. Each factor is formed here once
  // per variable (the same operations, so the same doubles) and the NaN skip kept as a
  // mask; the per-pair sum runs over k in order, as there.
  std::vector<double> z((size_t)(n * p));
  std::vector<uint8_t> miss((size_t)(n * p));
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < p; ++v)
    for (int64_t k = 0; k < n; ++k) {
      const double x = X[v * n + k];
      miss[v * n + k] = std::isnan(x) ? 1 : 0;
      z[v * n + k] = (x - mean[v]) / sd[v];
    }
  constexpr int64_t kTile = 16;
  const int64_t nt = (p + kTile - 1) / kTile;
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t t = 0; t < nt * nt; ++t) {
    const int64_t ta = t / nt, tb = t % nt;
    if (tb < ta) continue;
    for (int64_t a = ta * kTile; a < std::min(p, (ta + 1) * kTile); ++a) {
      const double *za = z.data() + a * n;
      const uint8_t *ma = miss.data() + a * n;
      for (int64_t b = std::max(a, tb * kTile); b < std::min(p, (tb + 1) * kTile); ++b) {
        const double *zb = z.data() + b * n;
        const uint8_t *mb = miss.data() + b * n;
        double s = 0.0;
        for (int64_t k = 0; k < n; ++k)
          if (!(ma[k] | mb[k])) s += za[k] * zb[k];
        C[a * p + b] = C[b * p + a] = s / denom;
      }
    }
  }
  return 0;
}

// Re-test of stored separation sets in FP64 with the reference's formulas
// (cpuInd.cpp:8-38): ok[t] = 1 iff p >= alpha for edge (i, j) given ids. ijl holds
// (i, j, level) per record, ids max_ids slots per record.
void orc_verify_sepsets(const double *C, int64_t p, int n, double alpha, int64_t k, const int32_t *ijl,
                        const int32_t *ids, int max_ids, uint8_t *ok) {
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t t = 0; t < k; ++t) {
    const int64_t i = ijl[3 * t], j = ijl[3 * t + 1];
    const int l = ijl[3 * t + 2];
    const int32_t *S = ids + t * max_ids;
    double pv;
    if (l == 0) {
      pv = calc_pvalue(C[std::max(i, j) * p + std::min(i, j)], n);
    } else if (l == 1) {
      pv = pval_l1(C[i * p + j], C[i * p + S[0]], C[j * p + S[0]], n);
    } else {
      const int kk = l + 2;
      std::vector<int64_t> V((size_t)kk);
      V[0] = i;
      V[1] = j;
      for (int q = 0; q < l; ++q) V[2 + q] = S[q];
      std::sort(V.begin() + 2, V.end());
      std::vector<double> M((size_t)(kk * kk));
      for (int a = 0; a < kk; ++a)
        for (int b = 0; b < kk; ++b) M[a * kk + b] = a == b ? 1.0 : C[V[a] * p + V[b]];
      pv = pval_ln(M.data(), kk, n);
    }
    ok[t] = pv >= alpha ? 1 : 0;
  }
}

namespace {
// Does the subset S (|S| = l >= 2) separate i and j? The partial correlation by
// Cholesky of the S block in FP64; where the block is ill-conditioned or |r| lies within
// 1e-8 relative of r_crit, the reference's pinv formula (pval_ln) decides.
bool separates(const double *C, int64_t p, int n, double alpha, double rc, int64_t i, int64_t j, const int *S,
               int l) {
  double Lm[kMaxLevel * kMaxLevel], wx[kMaxLevel], wy[kMaxLevel];
  bool ok = true;
  for (int r = 0; r < l && ok; ++r) {
    double vx = C[i * p + S[r]], vy = C[j * p + S[r]], d = 1.0;
    for (int c = 0; c < r; ++c) {
      double v = C[(int64_t)S[c] * p + S[r]];
      for (int q = 0; q < c; ++q) v -= Lm[r * kMaxLevel + q] * Lm[c * kMaxLevel + q];
      v /= Lm[c * kMaxLevel + c];
      Lm[r * kMaxLevel + c] = v;
      d -= v * v;
      vx -= v * wx[c];
      vy -= v * wy[c];
    }
    if (!(d > 1e-8)) ok = false;
    else {
      Lm[r * kMaxLevel + r] = std::sqrt(d);
      wx[r] = vx / Lm[r * kMaxLevel + r];
      wy[r] = vy / Lm[r * kMaxLevel + r];
    }
  }
  if (ok) {
    double ax = 1.0, ay = 1.0, b = C[i * p + j];
    for (int q = 0; q < l; ++q) {
      ax -= wx[q] * wx[q];
      ay -= wy[q] * wy[q];
      b -= wx[q] * wy[q];
    }
    if (ax > 1e-8 && ay > 1e-8 && std::isfinite(b)) {
      const double r = std::fabs(b / std::sqrt(ax * ay));
      if (r < rc * (1.0 - 1e-8)) return true;
      if (r > rc * (1.0 + 1e-8)) return false;
    }
  }
  const int kk = l + 2;
  std::vector<int64_t> V((size_t)kk);
  V[0] = i;
  V[1] = j;
  for (int q = 0; q < l; ++q) V[2 + q] = S[q];
  std::vector<double> M((size_t)(kk * kk));
  for (int a = 0; a < kk; ++a)
    for (int b = 0; b < kk; ++b) M[a * kk + b] = a == b ? 1.0 : C[V[a] * p + V[b]];
  return pval_ln(M.data(), kk, n) >= alpha;
}
}  // namespace

// Exhaustive check of edges kept at `level`: for edge (i, j) every level-subset of
// i's snapshot neighbours other than j, and of j's other than i (adj_before: the p x p
// adjacency at the level start), is tested in FP64; status[t] = 0 no subset separates,
// 1 a subset separates (the edge should have been removed), 2 not checked (more than
// max_subsets subsets in a direction).
void orc_check_retained(const double *C, int64_t p, int n, double alpha, int level, const uint8_t *adj_before,
                        int64_t k, const int32_t *edges, int64_t max_subsets, int8_t *status) {
  const double rc = r_crit_for(alpha, n);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t t = 0; t < k; ++t) {
    const int64_t ends[2] = {edges[2 * t], edges[2 * t + 1]};
    std::vector<int> nb[2];
    for (int e = 0; e < 2; ++e)
      for (int64_t v = 0; v < p; ++v)
        if (adj_before[ends[e] * p + v] && v != ends[1 - e]) nb[e].push_back((int)v);
    int8_t st = 0;
    for (int e = 0; e < 2 && st == 0; ++e)
      if ((int)nb[e].size() >= level && binom((int)nb[e].size(), level) > (uint64_t)max_subsets) st = 2;
    for (int e = 0; e < 2 && st == 0; ++e) {
      const int m = (int)nb[e].size();
      if (m < level) continue;
      const int64_t i = ends[e], j = ends[1 - e];
      if (level == 1) {
        for (int q = 0; q < m && st == 0; ++q)
          if (pval_l1(C[i * p + j], C[i * p + nb[e][q]], C[j * p + nb[e][q]], n) >= alpha) st = 1;
        continue;
      }
      int pos[kMaxLevel], S[kMaxLevel];
      for (int q = 0; q < level; ++q) pos[q] = q;
      for (;;) {
        for (int q = 0; q < level; ++q) S[q] = nb[e][pos[q]];
        if (separates(C, p, n, alpha, rc, i, j, S, level)) {
          st = 1;
          break;
        }
        int q = level - 1;
        while (q >= 0 && pos[q] == m - level + q) --q;
        if (q < 0) break;
        ++pos[q];
        for (int r = q + 1; r < level; ++r) pos[r] = pos[r - 1] + 1;
      }
    }
    status[t] = st;
  }
}

// skeleton.cpp:152-190 level loop; max_level < 0 runs until a level has no test.
orc_result *orc_run(const double *C, int64_t p, int n_obs, double alpha, int max_level, int threads) {
  if (!C || p < 2 || n_obs < 4) return nullptr;
  if (threads <= 0) threads = omp_get_max_threads();
  orc_result *res = new orc_result();
  State &s = res->st;
  s.p = p;
  s.n = n_obs;
  s.alpha = alpha;
  s.r_crit = r_crit_for(alpha, n_obs);
  s.cor.assign(C, C + p * p);
  s.adj.assign((size_t)(p * p), 1);  // state.cu:31-36
  for (int64_t i = 0; i < p; ++i) s.adj[i * p + i] = 0;
  s.compact.resize(p);
  s.l0_deleted.assign((size_t)(p * p), 0);
  s.pmax0.assign((size_t)(p * p), 0.0);
  const int top = max_level < 0 ? kMaxLevel : std::min(max_level, kMaxLevel);
  for (int lvl = 0; lvl <= top; ++lvl) {
    double t0 = omp_get_wtime();
    int64_t before = s.tests.load();
    if (lvl >= 1) compact(s);
    int64_t pot = lvl == 0 ? p * (p - 1) / 2 : potential_tests(s, lvl);
    if (lvl >= 1 && pot == 0) break;
    execute_level(s, lvl, threads);
    res->tests_per_level[lvl] = s.tests.load() - before;
    res->potential_per_level[lvl] = pot;
    int64_t e = 0;
    for (int64_t i = 0; i < p; ++i)
      for (int64_t j = i + 1; j < p; ++j) e += s.adj[i * p + j];
    res->edges_after_level[lvl] = e;
    res->ms_per_level[lvl] = (omp_get_wtime() - t0) * 1e3;
    res->levels_run = lvl + 1;
  }
  return res;
}

void orc_free(orc_result *r) { delete r; }
int orc_levels_run(const orc_result *r) { return r->levels_run; }
int64_t orc_tests(const orc_result *r, int level) { return r->tests_per_level[level]; }
int64_t orc_potential(const orc_result *r, int level) { return r->potential_per_level[level]; }
int64_t orc_edges_after(const orc_result *r, int level) { return r->edges_after_level[level]; }
double orc_ms(const orc_result *r, int level) { return r->ms_per_level[level]; }
void orc_adjacency(const orc_result *r, uint8_t *out) {
  std::memcpy(out, r->st.adj.data(), r->st.adj.size());
}
int64_t orc_num_records(const orc_result *r) { return (int64_t)r->st.seps.size(); }
// records of level >= 1 removals, sorted by (i, j): i, j, level, ids[max_ids], pmax
int64_t orc_records(const orc_result *r, int32_t *ij_level, int32_t *ids, int max_ids, double *pmax,
                    int64_t cap) {
  std::vector<int64_t> keys;
  keys.reserve(r->st.seps.size());
  for (auto &kv : r->st.seps) keys.push_back(kv.first);
  std::sort(keys.begin(), keys.end());
  int64_t n = std::min<int64_t>(cap, (int64_t)keys.size());
  for (int64_t t = 0; t < n; ++t) {
    const SepRec &rec = r->st.seps.at(keys[t]);
    ij_level[3 * t] = (int32_t)(keys[t] / r->st.p);
    ij_level[3 * t + 1] = (int32_t)(keys[t] % r->st.p);
    ij_level[3 * t + 2] = rec.level;
    for (int k = 0; k < max_ids; ++k) ids[t * max_ids + k] = k < (int)rec.ids.size() ? rec.ids[k] : -1;
    pmax[t] = rec.pmax;
  }
  return n;
}
// level-0 removal flag and its p-value for pair (i < j)
int orc_l0_deleted(const orc_result *r, int64_t i, int64_t j) { return r->st.l0_deleted[i * r->st.p + j]; }
double orc_l0_pmax(const orc_result *r, int64_t i, int64_t j) { return r->st.pmax0[i * r->st.p + j]; }

}  // extern "C"
