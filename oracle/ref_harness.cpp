// ORACLE -- test infrastructure only.
// Drives the reference's own CPU test code (compiled from its sources by
// oracle/build_ref.sh, against the stand-in headers in oracle/ref_shim/) to pin the
// oracle. The MMState buffers are allocated with malloc here instead of
// cudaMallocManaged (src/util/state.cu:3-44 needs a GPU) and initialised as
// src/util/state.cu:31-43 does. Levels 0-3 run through CPUExecutor::executeLevel
// with every row queued on the CPU, which is the --cpu-only balancing of
// src/loadbalance/balancer.cpp:46-54; levels >= 4 (no row-variant code exists in
// the reference) run through its level-generic testEdgeWorkstealing
// (src/executor/testing/cpuWorkstealingTests.cpp:114-124). The compaction between
// levels restates src/independence/compact.cu:4-89 (ascending neighbour ids, count
// in slot p-1), which is a GPU kernel in the reference.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <tuple>
#include <vector>

#include "executor/cpuExecutor.hpp"
#include "executor/testing/cpuWorkstealingTests.hpp"
#include "util/state.cuh"

static void compact_rows(MMState &s) {
  const int64_t p = (int64_t)s.p;
  int maxlen = 0;
  for (int64_t i = 0; i < p; ++i) {
    int len = 0;
    for (int64_t j = 0; j < p; ++j)
      if (s.adj[i * p + j]) s.adj_compact[i * p + len++] = (int)j;
    for (int64_t j = len; j < p - 1; ++j) s.adj_compact[i * p + j] = 0;
    s.adj_compact[i * p + p - 1] = len;
    maxlen = std::max(maxlen, len);
  }
  s.max_adj[0] = maxlen;
}

extern "C" int ref_run(const double *C, int64_t p, int n_obs, double alpha, int max_level, int threads,
                       uint8_t *adj_out, int32_t *sep_out, double *pmax_out) {
  MMState s;
  s.p = (uint64_t)p;
  s.observations = n_obs;
  s.alpha = alpha;
  s.maxLevel = max_level;
  s.ats = true;
  s.maxCondSize = std::max(max_level, 1);
  s.gpu_done = false;
  s.cor = (double *)malloc(sizeof(double) * p * p);
  s.adj = (int *)malloc(sizeof(int) * p * p);
  s.adj_compact = (int *)malloc(sizeof(int) * p * p);
  s.pMax = (double *)malloc(sizeof(double) * p * p);
  s.sepSets = (int *)malloc(sizeof(int) * p * p * s.maxCondSize);
  s.lock = (int *)malloc(sizeof(int) * p * p);
  s.node_status = (statusbool *)malloc(sizeof(statusbool) * p * p);
  s.max_adj = (int *)malloc(sizeof(int));
  std::memcpy(s.cor, C, sizeof(double) * p * p);
  std::fill_n(s.adj, p * p, 1);
  std::fill_n(s.adj_compact, p * p, 1);
  std::fill_n(s.node_status, p * p, false);
  for (int64_t i = 0; i < p; ++i) {
    s.adj[i * p + i] = 0;
    s.adj_compact[i * p + i] = 0;
  }
  std::fill_n(s.pMax, p * p, 0.0);
  std::fill_n(s.sepSets, p * p * s.maxCondSize, -1);
  std::memset(s.lock, 0, sizeof(int) * p * p);
  s.max_adj[0] = (int)p;

  CPUExecutor cpu(&s);
  for (int lvl = 0; lvl <= max_level; ++lvl) {
    if (lvl >= 1) compact_rows(s);
    cpu.cleanupSplitTasks();
    for (int64_t row = 0; row < p; ++row) cpu.enqueueSplitTask(SplitTask{(int)row, 1});
    if (lvl <= 3) {
      cpu.executeLevel(lvl, threads, false);
    } else {
      cpu.calculateRowLengthMap(lvl);
      std::atomic<int> done{0};
      for (auto &rl : cpu.rowLengthMap) {
        int row = std::get<0>(rl), len = std::get<1>(rl);
        for (int col = 0; col < len; ++col)
          testEdgeWorkstealing(&s, row, col, s.adj_compact[row * p + col], cpu.deletedEdges, len, done, lvl);
      }
    }
  }
  for (int64_t i = 0; i < p * p; ++i) adj_out[i] = (uint8_t)(s.adj[i] != 0);
  if (sep_out) std::memcpy(sep_out, s.sepSets, sizeof(int) * p * p * s.maxCondSize);
  if (pmax_out) std::memcpy(pmax_out, s.pMax, sizeof(double) * p * p);
  free(s.cor); free(s.adj); free(s.adj_compact); free(s.pMax); free(s.sepSets);
  free(s.lock); free(s.node_status); free(s.max_adj);
  return 0;
}
