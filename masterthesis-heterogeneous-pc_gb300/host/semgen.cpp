// Seeded linear-Gaussian SEM generator for synthetic skeleton-discovery inputs.
//
// The reference ships no data generator (its benchmarks read TCGA correlation
// matrices that are not distributed, benchmark.py:21-41). This generator builds the
// synthetic workloads the benchmarks here use: an Erdos-Renyi or
// preferential-attachment DAG over a random topological order, edge weights
// sign * U[w_lo, w_hi], and X_j = sum_{i in pa(j)} w_ij X_i + N(0,1).
//
// Bit reproducibility: the output must be identical on x86-64 and aarch64, so
// that committed golden fixtures stay valid on any host. Only IEEE +,-,*,/ and
// sqrt (all correctly rounded) are used; the natural log needed by the Marsaglia
// polar method is evaluated with a fixed series (below) instead of libm, and the
// file is compiled with -ffp-contract=off so that no FMA contraction changes the
// rounding on hosts that have FMA.
#include "../../include/heterogpc.h"

#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <cmath>
#include <thread>

namespace {

// splitmix64: seeds and per-stream state.
inline uint64_t splitmix64(uint64_t &x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// xoshiro256** generator (Blackman & Vigna).
struct Rng {
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    uint64_t x = seed;
    for (int i = 0; i < 4; ++i) s[i] = splitmix64(x);
  }
  static inline uint64_t rotl(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }
  uint64_t next() {
    const uint64_t result = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return result;
  }
  // uniform in [0,1) with 53 random bits
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  // uniform integer in [0, m)
  uint64_t below(uint64_t m) {
    // Lemire-free simple rejection for exactness
    const uint64_t lim = UINT64_MAX - UINT64_MAX % m;
    uint64_t v;
    do { v = next(); } while (v >= lim);
    return v % m;
  }
};

// ln(x) for x > 0 using only +,-,*,/ : x = m * 2^e with m in [1/sqrt2, sqrt2),
// ln m = 2 * atanh(s), s = (m-1)/(m+1), |s| < 0.1716, series to s^41.
double det_log(double x) {
  int e = 0;
  double m = x;
  // scale into [0.5, 1) by exact multiplications by 2
  while (m >= 1.0) { m *= 0.5; ++e; }
  while (m < 0.5) { m *= 2.0; --e; }
  if (m < 0.70710678118654752440) { m *= 2.0; --e; }
  const double s = (m - 1.0) / (m + 1.0);
  const double s2 = s * s;
  double term = s, sum = 0.0;
  for (int k = 1; k <= 41; k += 2) {
    sum = sum + term / (double)k;
    term = term * s2;
  }
  const double ln2 = 0.69314718055994530942;
  return 2.0 * sum + (double)e * ln2;
}

// Standard normal pair by the Marsaglia polar method.
struct Normal {
  Rng rng;
  bool have = false;
  double spare = 0.0;
  explicit Normal(uint64_t seed) : rng(seed) {}
  double operator()() {
    if (have) { have = false; return spare; }
    double u, v, s;
    do {
      u = 2.0 * rng.uniform() - 1.0;
      v = 2.0 * rng.uniform() - 1.0;
      s = u * u + v * v;
    } while (s >= 1.0 || s == 0.0);
    const double f = std::sqrt(-2.0 * det_log(s) / s);
    spare = v * f;
    have = true;
    return u * f;
  }
};

uint64_t stream_seed(uint64_t seed, uint64_t stream) {
  uint64_t x = seed ^ (0xD1B54A32D192ED03ull * (stream + 1));
  return splitmix64(x);
}

}  // namespace

extern "C" hpc_status hpc_sem_generate(const hpc_sem_params *prm, double *X, float *X32,
                                       uint8_t *dag, double *weights) {
  if (!prm || prm->p < 2 || prm->n < 4) return HPC_ERR_INVALID_ARG;
  if (prm->graph != HPC_GRAPH_ER && prm->graph != HPC_GRAPH_PA) return HPC_ERR_INVALID_ARG;
  if (!(prm->w_lo > 0.0) || prm->w_hi < prm->w_lo) return HPC_ERR_INVALID_ARG;
  const int64_t p = prm->p, n = prm->n;

  // 1. random topological order: order[t] = variable at topological position t
  Rng grng(stream_seed(prm->seed, 0));
  std::vector<int64_t> order(p);
  for (int64_t i = 0; i < p; ++i) order[i] = i;
  for (int64_t i = p - 1; i > 0; --i) {
    int64_t j = (int64_t)grng.below((uint64_t)(i + 1));
    std::swap(order[i], order[j]);
  }

  // 2. parent lists in topological positions
  std::vector<std::vector<int64_t>> parents(p);  // indexed by topological position
  if (prm->graph == HPC_GRAPH_ER) {
    const double q = prm->degree / (double)(p - 1);
    for (int64_t t = 1; t < p; ++t)
      for (int64_t s = 0; s < t; ++s)
        if (grng.uniform() < q) parents[t].push_back(s);
  } else {
    // preferential attachment: node t picks min(m, t) distinct parents among
    // positions [0, t) with probability proportional to (degree + 1)
    const int m = prm->pa_parents > 0 ? prm->pa_parents : 2;
    std::vector<int64_t> urn;  // each endpoint of every edge, plus each node once
    urn.reserve((size_t)p * (m + 1) * 2);
    urn.push_back(0);
    for (int64_t t = 1; t < p; ++t) {
      const int want = (int)std::min<int64_t>(m, t);
      std::vector<int64_t> &pa = parents[t];
      while ((int)pa.size() < want) {
        int64_t c = urn[grng.below(urn.size())];
        if (std::find(pa.begin(), pa.end(), c) == pa.end()) pa.push_back(c);
      }
      std::sort(pa.begin(), pa.end());
      for (int64_t c : pa) { urn.push_back(c); urn.push_back(t); }
      urn.push_back(t);
    }
  }

  // 3. weights
  std::vector<std::vector<double>> w(p);
  for (int64_t t = 0; t < p; ++t) {
    w[t].resize(parents[t].size());
    for (size_t k = 0; k < parents[t].size(); ++k) {
      double mag = prm->w_lo + (prm->w_hi - prm->w_lo) * grng.uniform();
      w[t][k] = (grng.next() >> 63) ? -mag : mag;
    }
  }
  if (dag) {
    std::memset(dag, 0, (size_t)(p * p));
    for (int64_t t = 0; t < p; ++t)
      for (int64_t s : parents[t]) dag[order[s] * p + order[t]] = 1;  // parent -> child
  }
  if (weights) {
    std::memset(weights, 0, sizeof(double) * (size_t)(p * p));
    for (int64_t t = 0; t < p; ++t)
      for (size_t k = 0; k < parents[t].size(); ++k)
        weights[order[parents[t][k]] * p + order[t]] = w[t][k];
  }
  if (!X && !X32) return HPC_OK;

  // 4. data: noise per variable from its own stream (parallel), then the linear
  //    combination in topological order. Column-major n x p: X[v*n + k].
  std::vector<double> buf;
  double *D = X;
  if (!D) {
    buf.resize((size_t)(n * p));
    D = buf.data();
  }
  unsigned nth = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  std::vector<std::thread> pool;
  for (unsigned th = 0; th < nth; ++th) {
    pool.emplace_back([&, th]() {
      for (int64_t v = th; v < p; v += nth) {
        Normal g(stream_seed(prm->seed, (uint64_t)v + 1));
        double *col = D + v * n;
        for (int64_t k = 0; k < n; ++k) col[k] = g();
      }
    });
  }
  for (auto &t : pool) t.join();
  for (int64_t t = 0; t < p; ++t) {
    double *col = D + order[t] * n;
    for (size_t k = 0; k < parents[t].size(); ++k) {
      const double *pc = D + order[parents[t][k]] * n;
      const double wk = w[t][k];
      for (int64_t r = 0; r < n; ++r) col[r] = col[r] + wk * pc[r];
    }
  }
  if (X32)
    for (int64_t i = 0; i < n * p; ++i) X32[i] = (float)D[i];
  return HPC_OK;
}
