// Host check of the CI-test kernels' combinatorics (csrc/stats.cuh), compiled by
// nvcc as a host program: binom_fast against binom_sat, and unrank_lex_fast (table
// scan below m = 64, bisection above) against the plain lexicographic unranking
// unrank_lex (the order of ithCombination, src/util/cuda_util.cu:34-50) and against
// next_lex walks. Prints "ok <cases>" or the first mismatch and exits non-zero.
#include <cstdio>
#include <random>

#include "../masterthesis-heterogeneous-pc_gb300/csrc/stats.cuh"

using namespace hpc;

static int check(unsigned long long rank, int l, int m) {
  int a[HPC_MAX_LEVEL], b[HPC_MAX_LEVEL];
  unrank_lex(rank, l, m, a);
  unrank_lex_fast(rank, l, m, b);
  for (int q = 0; q < l; ++q)
    if (a[q] != b[q]) {
      std::printf("mismatch rank=%llu l=%d m=%d member %d: %d vs %d\n", rank, l, m, q, a[q], b[q]);
      return 1;
    }
  return 0;
}

int main() {
  long cases = 0;
  for (int n = 0; n < 3000; n += (n < 200 ? 1 : 37))
    for (int k = 0; k <= HPC_MAX_LEVEL; ++k) {
      const unsigned long long s = binom_sat(n, k), f = binom_fast(n, k);
      if (s != 0xFFFFFFFFFFFFFFFFull && s < (1ull << 60) && s != f) {
        std::printf("binom mismatch C(%d,%d): %llu vs %llu\n", n, k, s, f);
        return 1;
      }
      ++cases;
    }
  // every rank of small spaces, on both sides of the m = 64 switch
  const int ms[] = {1, 2, 5, 17, 40, 63, 64, 65, 70, 90};
  for (int m : ms)
    for (int l = 1; l <= 4 && l <= m; ++l) {
      const unsigned long long c = binom_sat(m, l);
      const unsigned long long stride = c > 200000 ? c / 200000 : 1;
      for (unsigned long long r = 0; r < c; r += stride, ++cases)
        if (check(r, l, m)) return 1;
      if (check(c - 1, l, m)) return 1;
    }
  // random ranks of large spaces (hub degrees), every level
  std::mt19937_64 g(12345);
  for (int it = 0; it < 200000; ++it, ++cases) {
    const int m = 64 + (int)(g() % 20000);
    const int l = 1 + (int)(g() % HPC_MAX_LEVEL);
    const unsigned long long c = binom_sat(m, l);
    if (c >= (1ull << 60)) continue;  // rows beyond the test-count limit never run
    const unsigned long long r = g() % c;
    if (check(r, l, m)) return 1;
    if (check(c - 1, l, m) || check(0, l, m)) return 1;
  }
  // successors: unranking r + 1 equals one next_lex step from r
  for (int it = 0; it < 20000; ++it, ++cases) {
    const int m = 64 + (int)(g() % 3000), l = 1 + (int)(g() % 6);
    const unsigned long long c = binom_sat(m, l);
    if (c >= (1ull << 60) || c < 2) continue;
    const unsigned long long r = g() % (c - 1);
    int a[HPC_MAX_LEVEL], b[HPC_MAX_LEVEL];
    unrank_lex_fast(r, l, m, a);
    next_lex(l, m, a);
    unrank_lex_fast(r + 1, l, m, b);
    for (int q = 0; q < l; ++q)
      if (a[q] != b[q]) {
        std::printf("successor mismatch r=%llu l=%d m=%d\n", r, l, m);
        return 1;
      }
  }
  std::printf("ok %ld\n", cases);
  return 0;
}
