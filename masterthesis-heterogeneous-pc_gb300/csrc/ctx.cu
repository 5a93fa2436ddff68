// C ABI of libheterogpc: contexts (one or many skeleton instances), correlation entry
// points, the level loop and result retrieval. The reference equivalents are named
// beside each function in include/heterogpc.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "internal.cuh"
#include "stats.cuh"

namespace hpc {

static thread_local std::string g_last_error;

void set_error(const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

hpc_status cuda_fail(cudaError_t e, const char *what, const char *file, int line) {
  set_error("CUDA error %s (%s) in %s at %s:%d", cudaGetErrorName(e), cudaGetErrorString(e), what, file, line);
  if (e == cudaErrorMemoryAllocation) return HPC_ERR_OOM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return HPC_ERR_NO_DEVICE;
  return HPC_ERR_CUDA;
}

namespace {

constexpr int kLevels = HPC_MAX_LEVEL + 1;

// z with erfc(z / sqrt 2) == alpha, by bisection in FP64 (host set-up only)
double z_crit_of(double alpha) {
  double lo = 0.0, hi = 40.0;
  for (int it = 0; it < 200; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (std::erfc(mid / 1.41421356237309504880) >= alpha) lo = mid; else hi = mid;
  }
  return 0.5 * (lo + hi);
}

// |r| with calc_pvalue64(r) == alpha (p is decreasing in |r|); 2 if every r is removed
double r_crit_of(double alpha, int n) {
  double lo = 0.0, hi = kCutThr;
  if (calc_pvalue64(hi, n) >= alpha) return 2.0;
  for (int it = 0; it < 200; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (calc_pvalue64(mid, n) >= alpha) lo = mid; else hi = mid;
  }
  return 0.5 * (lo + hi);
}

// Absolute error bound of the tensor-core (split-BF16, FP32-accumulated) correlation
// entries used by the FP32 decision bands: the rounding of the low halves (2^-17
// relative per value) averages over the n samples, plus the FP32 accumulation; four
// times the model, which bounds the measured errors of tests/test_gpu_tensorcore.py.
double tc_entry_err(int64_t n) { return 4.0 * (1.6e-5 / std::sqrt((double)n) + 1e-7); }

// Device memory comes from the stream-ordered allocator on one non-blocking stream
// per device: unlike cudaFree, returning memory does not synchronise the device, so
// contexts created and destroyed while others run (the serving loop) do not stall
// them. Freed memory stays in the device's default pool for the next context.
cudaStream_t alloc_stream() {
  static std::mutex mu;
  static cudaStream_t streams[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> g(mu);
  if (!streams[dev]) {
    cudaStreamCreateWithFlags(&streams[dev], cudaStreamNonBlocking);
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t keep = ~0ull;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
  }
  return streams[dev];
}

// Test hooks: the k-th device allocation from now fails (0 = none), and the number of
// the library's device allocations currently live.
std::atomic<long long> g_fail_alloc_in{0};
std::atomic<int> g_set_from{kSetOrderFrom};
std::atomic<long long> g_live_allocs{0};

template <typename T>
hpc_status dev_alloc(T **ptr, int64_t count, const char *what) {
  if (count <= 0) count = 1;
  long long k = g_fail_alloc_in.load();
  while (k > 0 && !g_fail_alloc_in.compare_exchange_weak(k, k - 1)) {
  }
  if (k == 1) {
    *ptr = nullptr;
    set_error("device allocation of %s (%lld bytes) failed: injected by hpc_debug_fail_allocation", what,
              (long long)(sizeof(T) * count));
    return HPC_ERR_OOM;
  }
  cudaStream_t as = alloc_stream();
  cudaError_t e = cudaMallocAsync((void **)ptr, sizeof(T) * (size_t)count, as);
  if (e == cudaSuccess) e = cudaStreamSynchronize(as);
  if (e != cudaSuccess) {
    *ptr = nullptr;
    cudaGetLastError();
    set_error("device allocation of %s (%lld bytes) failed: %s", what, (long long)(sizeof(T) * count),
              cudaGetErrorString(e));
    return HPC_ERR_OOM;
  }
  g_live_allocs.fetch_add(1);
  return HPC_OK;
}

// Only after the context's own work that used ptr has completed.
template <typename T>
void dev_free(T *&ptr) {
  if (ptr) {
    cudaFreeAsync((void *)ptr, alloc_stream());
    g_live_allocs.fetch_sub(1);
  }
  ptr = nullptr;
}

hpc_status check_ctx(hpc_ctx *c) {
  if (!c) {
    set_error("null context");
    return HPC_ERR_INVALID_ARG;
  }
  HPC_CUDA(cudaSetDevice(c->device));
  return HPC_OK;
}

hpc_status check_index(hpc_ctx *c, int idx) {
  if (idx < 0 || idx >= c->count) {
    set_error("instance %d out of range [0, %d)", idx, c->count);
    return HPC_ERR_INVALID_ARG;
  }
  return HPC_OK;
}

double denom_of(const hpc_ctx *c, int64_t n) {
  return c->opts.ref_compat_sd ? (double)((float)n - 1.f) : (double)(n - 1);
}

// The device instance table from the host bookkeeping and the current buffers.
hpc_status write_inst_table(hpc_ctx *c) {
  std::vector<Inst> t((size_t)c->count);
  for (int b = 0; b < c->count; ++b) {
    const InstHost &h = c->ih[b];
    Inst &I = t[b];
    std::memset(&I, 0, sizeof(I));
    I.p = h.p;
    I.W = h.W;
    I.n_obs = (int)h.n;
    I.alpha = h.alpha;
    const double rc = h.r_crit >= 1.5 ? 2.0 : h.r_crit;
    const double sqrt_n3 = std::sqrt((double)h.n - 3.0);
    I.r_c = (float)rc;
    I.margin_r = rc >= 1.5 ? 0.f : (float)(c->opts.retest_margin * h.zc * (1.0 - rc * rc) / sqrt_n3);
    const double eps_in = c->cor32_rounded ? 1.2e-7 : tc_entry_err(h.n);
    I.ke_a = (float)(4.0 * eps_in * (1.0 + std::min(rc, 1.0)));
    I.ke_b = (float)(2.4e-7 * (1.0 + std::min(rc, 1.0)));
    I.r_lo = rc >= 1.5 ? 2.0 : rc * (1.0 - 1e-7);
    I.r_hi = rc >= 1.5 ? 2.0 : rc * (1.0 + 1e-7);
    const double d0 = tc_entry_err(h.n) + 1e-6 * rc;
    I.lo32 = rc >= 1.5 ? 2.f : (float)(rc - d0);
    I.hi32 = rc >= 1.5 ? 2.f : (float)(rc + d0);
    I.cor64 = (c->cor64_valid && c->cor64) ? c->cor64 + h.cor_off : nullptr;
    I.cor32 = c->cor32 ? c->cor32 + h.cor_off : nullptr;
    I.Z = c->z_valid ? c->Z + h.z_off : nullptr;
    I.zh = (!c->z_valid && c->zpair_valid) ? c->zpair + h.z_off : nullptr;
    I.zl = (!c->z_valid && c->zpair_valid) ? c->zpair + c->ztot + h.z_off : nullptr;
    I.ec = (c->ecache && I.zh) ? c->ecache + h.cor_off : nullptr;
    I.ev = (c->ecache && I.zh) ? c->evalid : nullptr;
    I.ev_off = h.cor_off;
    I.n_z = h.n;
    I.denom = denom_of(c, h.n);
    I.adj = c->adj + h.adj_off;
    I.deg = c->deg + h.row_off;
    I.rowptr = c->rowptr + h.row_off;
    I.row_work = c->row_work + h.row_off;
    I.colidx = c->colidx ? c->colidx + h.colidx_off : nullptr;
    I.colidx_cap = c->colidx ? h.colidx_cap : 0;
    I.recs = c->recs ? c->recs + h.rec_off : nullptr;
    I.rec_cap = c->recs ? h.rec_cap : 0;
    I.rec_ids = c->rec_ids;
    I.rec_stride = rec_stride_words(c->rec_ids);
    I.ctr = c->ctr + (size_t)b * kLevels;
    I.g = c->gctr + b;
    I.dirty = c->row_dirty ? c->row_dirty + h.row_off : nullptr;
    I.snap_epoch = c->snap_epoch;
  }
  if (c->inst_host.size() == t.size() && std::memcmp(c->inst_host.data(), t.data(), sizeof(Inst) * t.size()) == 0)
    return HPC_OK;  // unchanged: captured graphs stay valid
  // a new table (new arrays or capacities) invalidates every neighbour-list snapshot
  ++c->snap_epoch;
  for (auto &I : t) I.snap_epoch = c->snap_epoch;
  c->inst_host = t;
  HPC_CUDA(cudaMemcpyAsync(c->inst, c->inst_host.data(), sizeof(Inst) * t.size(), cudaMemcpyHostToDevice, c->stream));
  HPC_CUDA(cudaStreamSynchronize(c->stream));
  ++c->inst_version;
  return HPC_OK;
}

// The lowest set-order level in effect for a context (0: the edge order throughout):
// the process-wide setting, where the context's re-tests are queued (no FP64 matrix),
// the set order was not turned off by a re-test queue overflow, and the levels run in
// a whole-skeleton call (hpc_run_level cannot repeat a run after an overflow).
int effective_set_from(const hpc_ctx *c) {
  if (c->opts.precision == HPC_PREC_FP64 || c->cor64_valid || c->set_off || c->level_by_level) return 0;
  return set_order_from();
}

// Whether level l runs in the set order: from the lowest set-order level in effect, and
// only where the largest degree at the level's start in the context's last run (else
// the level before it; unknown before a first run) fits kSetDegMax.
bool set_at(const hpc_ctx *c, int level) {
  if (!uses_set_order(effective_set_from(c), level)) return false;
  int d = c->deg_seen[level];
  if (d < 0) d = c->deg_seen[level - 1];
  return d <= kSetDegMax;
}

unsigned int set_mask(const hpc_ctx *c, int last) {
  unsigned int m = 0;
  for (int l = 2; l <= last && l <= kSetTop; ++l)
    if (set_at(c, l)) m |= 1u << l;
  return m;
}

Launch make_launch(hpc_ctx *c, int level) {
  Launch L{};
  L.inst = c->inst;
  L.count = c->count;
  L.level = level;
  L.word_prefix = c->prefixes;
  L.tile_prefix = c->prefixes + (c->count + 1);
  L.row_prefix = c->prefixes + 2 * (c->count + 1);
  L.work_prefix = c->work_prefix + (size_t)level * (c->count + 1);
  L.lc = c->lc + level;
  L.rq = c->rq;
  L.rq_cap = c->rq_cap;
  L.rq_val = c->rq_val;
  L.rq_done = c->rq_done;
  L.rq_vcap = c->rq_vcap;
  L.seg_prefix = c->prefixes + 3 * (c->count + 1);
  L.seg = c->seg + (size_t)level * c->total_segs;
  L.row_cache = c->count == 1 && c->ih[0].p + 1 <= kRowCache;
  L.total_rows = c->total_rows;
  L.total_segs = c->total_segs;
  L.tune = c->tune_dev;
  L.force = c->tune_force;
  L.p_bucket = c->p_bucket;
  L.row_work_limit = std::min<unsigned long long>(1ull << 56, 0x7FFFFFFFFFFFFFFFull /
                                                                  (unsigned long long)std::max<long long>(1, c->total_rows));
  L.inst0 = c->inst_host[0];
  L.wait_ns = c->wait_ns;
  L.bar_extra = c->bar_extra;
  return L;
}

hpc_status pull_counters(hpc_ctx *c) {
  HPC_CUDA(cudaMemcpyAsync(c->ctr_host, c->ctr, sizeof(DevCounters) * (size_t)c->count * kLevels,
                           cudaMemcpyDeviceToHost, c->stream));
  if (!c->last_run_graph)  // the level kernels' phase times
    HPC_CUDA(cudaMemcpyAsync(c->lc_host, c->lc, sizeof(LaunchCounters) * kLevels, cudaMemcpyDeviceToHost, c->stream));
  HPC_CUDA(cudaMemcpyAsync(c->gctr_host, c->gctr, sizeof(DevGlobal) * (size_t)c->count, cudaMemcpyDeviceToHost,
                           c->stream));
  HPC_CUDA(cudaStreamSynchronize(c->stream));
  return HPC_OK;
}

// Queue all device work of one level on the context stream (no host sync).
// `timed` records the per-level events (not inside a graph capture: events recorded
// by graph nodes cannot be timed).
hpc_status enqueue_level(hpc_ctx *c, int level, bool timed) {
  hpc_status s;
  const Launch L = make_launch(c, level);
  cudaEvent_t *ev = c->evl[level];
  const bool queue = !c->cor64_valid;  // FP64 re-tests deferred to the re-test kernel
  if (timed) HPC_CUDA(cudaEventRecord(ev[0], c->stream));
  if (level == 0) {
    if (timed) HPC_CUDA(cudaEventRecord(ev[1], c->stream));
    if ((s = launch_level0(L, c->total_tiles, c->stream)) != HPC_OK) return s;
    if (queue && (s = launch_retest(L, c->sm_count, c->stream)) != HPC_OK) return s;
    if (timed) HPC_CUDA(cudaEventRecord(ev[2], c->stream));
    if ((s = launch_degrees(L, c->total_rows, c->stream)) != HPC_OK) return s;
    if ((s = launch_scan(L, c->stream)) != HPC_OK) return s;
    c->timings.launches += queue ? 4 : 3;
    return HPC_OK;
  }
  // snapshot rebuild, test-count scan and CI tests in one launch
  if (timed) HPC_CUDA(cudaEventRecord(ev[1], c->stream));
  const bool set = set_at(c, level);
  // level 1: the queue-only build of the interleaved variants where the re-tests are
  // queued and a queue overflow can be rerun
  const bool qo = level == 1 && c->l1v_now != kL1Chunked && effective_set_from(c) > 0;
  const int var = level == 1 ? (qo ? c->l1v_now | kQueueOnly : c->l1v_now) : set ? kSetOrder : kL1Interleaved;
  const int grid = level == 1 ? (qo ? c->citest_grid_l1q[c->l1v_now] : c->citest_grid_l1[var])
                   : set      ? c->citest_grid_set[level]
                              : c->citest_grid[level];
  if ((s = launch_level(L, c->opts.precision, grid, var, c->stream)) != HPC_OK) return s;
  if (timed) HPC_CUDA(cudaEventRecord(ev[3], c->stream));
  if (queue && (s = launch_retest(L, c->sm_count, c->stream)) != HPC_OK) return s;
  if (timed) HPC_CUDA(cudaEventRecord(ev[2], c->stream));
  c->timings.launches += queue ? 2 : 1;
  return HPC_OK;
}

// Neighbour-list and record buffers sized from the level-0 result (counters pulled):
// an instance needs room for the edges alive after level 0.
hpc_status ensure_capacity(hpc_ctx *c, bool *changed) {
  *changed = false;
  bool grow = !c->colidx || !c->recs;
  for (int b = 0; b < c->count && !grow; ++b) {
    const long long e2 = (long long)c->ctr_host[(size_t)b * kLevels].edges2;
    if (e2 > c->ih[b].colidx_cap || e2 / 2 > c->ih[b].rec_cap) grow = true;
  }
  if (!grow) return HPC_OK;
  long long ct = 0, rt = 0;  // neighbour ids, record words
  const long long stride = rec_stride_words(c->rec_ids);
  for (int b = 0; b < c->count; ++b) {
    InstHost &h = c->ih[b];
    const long long e2 = (long long)c->ctr_host[(size_t)b * kLevels].edges2;
    h.colidx_cap = std::max<long long>(std::max<long long>(h.colidx_cap, e2), 1);
    h.rec_cap = std::max<long long>(std::max<long long>(h.rec_cap, e2 / 2), 1);
    h.colidx_off = ct;
    h.rec_off = rt;
    ct += h.colidx_cap;
    rt += h.rec_cap * stride;
  }
  hpc_status s;
  if (ct > c->colidx_total || !c->colidx) {
    dev_free(c->colidx);
    c->colidx_total = 0;
    if ((s = dev_alloc(&c->colidx, ct, "neighbour lists")) != HPC_OK) return s;
    c->colidx_total = ct;
  }
  if (rt > c->rec_total || !c->recs) {
    dev_free(c->recs);
    c->rec_total = 0;
    if ((s = dev_alloc(&c->recs, rt, "separation-set records")) != HPC_OK) return s;
    c->rec_total = rt;
  }
  *changed = true;
  return write_inst_table(c);
}

// Statistics of one level, summed over the instances (or of one instance).
hpc_level_stats level_stats_of(hpc_ctx *c, int level, int only) {
  hpc_level_stats st{};
  st.level = level;
  for (int b = 0; b < c->count; ++b) {
    if (only >= 0 && b != only) continue;
    const DevCounters &h = c->ctr_host[(size_t)b * kLevels + level];
    const InstHost &ih = c->ih[b];
    const int64_t before = level == 0 ? ih.p * (ih.p - 1) / 2 : 0;
    st.max_degree = std::max(st.max_degree, level == 0 ? (int)(ih.p - 1) : h.max_deg);
    if (level == 0) {
      st.rows += ih.p;
      st.potential_tests += before;
      st.executed_tests += before;
      st.edges_before += before;
      st.edges_after += (int64_t)(h.edges2 / 2);
    } else {
      st.rows += h.rows;
      st.potential_tests += (int64_t)h.work_total;
      st.executed_tests += (int64_t)h.tests;
      st.retests += (int64_t)h.retests;
      st.edges_before += (int64_t)(h.edges2 / 2);
      st.edges_after += (int64_t)(h.edges2 / 2) - (int64_t)h.deleted;
    }
  }
  return st;
}

// Per-level statistics and timings after a level ran (counters pulled).
hpc_status collect_level(hpc_ctx *c, int level, hpc_level_stats *out) {
  hpc_level_stats st = level_stats_of(c, level, -1);
  if (level == 1) c->l1_max_deg = st.max_degree;
  if (level >= 1) c->deg_seen[level] = st.max_degree;
  float t_all = 0.f, t_snap = 0.f, t_test = 0.f, t_re = 0.f;
  if (!c->last_run_graph) {
    HPC_CUDA(cudaEventElapsedTime(&t_snap, c->evl[level][0], c->evl[level][1]));
    if (level >= 1) {  // the level kernel, then its re-tests
      HPC_CUDA(cudaEventElapsedTime(&t_test, c->evl[level][1], c->evl[level][3]));
      HPC_CUDA(cudaEventElapsedTime(&t_re, c->evl[level][3], c->evl[level][2]));
    } else {
      HPC_CUDA(cudaEventElapsedTime(&t_test, c->evl[level][1], c->evl[level][2]));
    }
    HPC_CUDA(cudaEventElapsedTime(&t_all, c->evl[level][0], level < HPC_MAX_LEVEL && level + 1 < c->next_level
                                                                ? c->evl[level + 1][0] : c->evl[level][2]));
  }
  st.ms = t_all;
  c->timings.level_ms[level] = t_all;
  c->timings.compact_ms[level] = t_snap;
  c->timings.test_ms[level] = t_test;
  c->timings.retest_ms[level] = t_re;
  {  // phases of the level kernel by %globaltimer (kernel-by-kernel runs)
    const LaunchCounters &lc = c->lc_host[level];
    const bool ok = !c->last_run_graph && level >= 1 && lc.t_entry && lc.t_rebuilt >= lc.t_entry &&
                    lc.t_scanned >= lc.t_rebuilt;
    c->timings.rebuild_ms[level] = ok ? 1e-6 * (double)(lc.t_rebuilt - lc.t_entry) : 0.0;
    c->timings.scan_ms[level] = ok ? 1e-6 * (double)(lc.t_scanned - lc.t_rebuilt) : 0.0;
  }
  for (int b = 0; b < c->count; ++b) {
    const DevCounters &h = c->ctr_host[(size_t)b * kLevels + level];
    c->ih[b].edges = level == 0 ? (int64_t)(h.edges2 / 2) : (int64_t)(h.edges2 / 2) - (int64_t)h.deleted;
    if (h.band_violations) {
      set_error("instance %d level %d: %llu FP32 removals not confirmed in FP64 (error bound violated)", b, level,
                (unsigned long long)h.band_violations);
      return HPC_ERR_NUMERIC;
    }
  }
  if (c->opts.verbose)
    printf("level %d: max degree %d, tests %lld of %lld, FP64 re-tests %lld, edges %lld -> %lld, %.3f ms\n", level,
           st.max_degree, (long long)st.executed_tests, (long long)st.potential_tests, (long long)st.retests,
           (long long)st.edges_before, (long long)st.edges_after, st.ms);
  if (out) *out = st;
  return HPC_OK;
}

hpc_status global_errors(hpc_ctx *c) {
  for (int b = 0; b < c->count; ++b) {
    const int err = c->gctr_host[b].err;
    if (err & kErrWorkOverflow) {
      set_error("instance %d: a row's CI tests at this level exceed the limit of 2^63 / (rows of the context); "
                "run fewer levels (max_level)", b);
      return HPC_ERR_CAPACITY;
    }
    if (err & kErrRecOverflow) {
      set_error("instance %d: separation-set record buffer overflow", b);
      return HPC_ERR_CAPACITY;
    }
    if (err & kErrTimeout) {
      set_error("instance %d: a bounded device wait timed out", b);
      return HPC_ERR_TIMEOUT;
    }
    if (err & kErrBandViolation) {
      set_error("instance %d: an FP32 removal was not confirmed in FP64 (error bound violated)", b);
      return HPC_ERR_NUMERIC;
    }
  }
  return HPC_OK;
}

// A run to repeat from level 0: the neighbour lists were too small (the data changed
// since they were sized), or the set order found the re-test queue full (the rerun
// keeps the edge order, whose tests re-test inline when the queue is full).
bool needs_rerun(hpc_ctx *c) {
  bool again = false;
  for (int b = 0; b < c->count; ++b) {
    const int err = c->gctr_host[b].err;
    if (err & kErrRetestOverflow) c->set_off = true;
    if (err & (kErrCsrOverflow | kErrRetestOverflow)) again = true;
  }
  return again;
}

bool any_work(hpc_ctx *c, int level) {
  for (int b = 0; b < c->count; ++b)
    if (c->ctr_host[(size_t)b * kLevels + level].work_total) return true;
  return false;
}

bool capturable(cudaStream_t s) { return s != nullptr && s != cudaStreamLegacy && s != cudaStreamPerThread; }

// Level 1's kernel variant (kL1*; the kernel is chosen on the host, the tile sizes on
// the device): from the forced policy, else from the table entry for the level-1
// degree of the context's last run (the default, interleaved, before any run).
int l1_variant_of(const TuneEntry &e) {
  if (e.tile_cap <= 0) return kL1Interleaved;
  if (e.edge_lanes == 1) return kL1Chunked;
  return e.l1_prefetch ? kL1Prefetch : kL1Interleaved;
}

int level1_variant(hpc_ctx *c) {
  if (c->tune_force.tile_cap > 0) return l1_variant_of(c->tune_force);
  if (c->l1_max_deg < 0) return kL1Interleaved;
  return l1_variant_of(tune_get(c->p_bucket, 1, tune_bucket(c->l1_max_deg, kTuneDB)));
}

// The context's device copy of the tile-policy table, refreshed when the table
// changed (before any capture: graphs keep the pointer and read the current entries).
hpc_status sync_tune(hpc_ctx *c) {
  if (c->tune_dev && c->tune_version_dev == tune_version()) return HPC_OK;
  std::vector<TuneEntry> t;
  long long v = 0;
  tune_snapshot(&t, &v);
  hpc_status s;
  if (!c->tune_dev) {
    if ((s = dev_alloc(&c->tune_dev, (int64_t)t.size(), "tile-policy table")) != HPC_OK) return s;
    ++c->inst_version;  // a graph captured before holds no table pointer
  }
  HPC_CUDA(cudaMemcpyAsync(c->tune_dev, t.data(), sizeof(TuneEntry) * t.size(), cudaMemcpyHostToDevice, c->stream));
  HPC_CUDA(cudaStreamSynchronize(c->stream));  // t is released on return
  c->tune_version_dev = v;
  return HPC_OK;
}

// Run levels first..last with one host sync at the end; the whole sequence 0..last
// is captured once into a CUDA graph and replayed while the buffers stay in place.
// `finalize` appends the FP64 p-values of the FP32-decided removals (and their FP64
// confirmation where the instance has an FP64 matrix) to the sequence, as the
// reference writes pMax inside its levels (src/executor/testing/cpuUtil.cpp:23-48);
// the kernel skips records already finalised, so every chunk of a run may end with it.
hpc_status run_levels(hpc_ctx *c, int first, int last, bool use_graph, bool wait = true, bool finalize = false) {
  hpc_status s;
  if ((s = sync_tune(c)) != HPC_OK) return s;
  c->l1v_now = level1_variant(c);
  finalize = finalize && last >= 1 && c->recs;
  auto enqueue_all = [&](bool timed) -> hpc_status {
    if (first == 0) {  // a skeleton from the start: its counters and records begin at zero
      HPC_CUDA(cudaMemsetAsync(c->ctr, 0, sizeof(DevCounters) * (size_t)c->count * kLevels, c->stream));
      HPC_CUDA(cudaMemsetAsync(c->gctr, 0, sizeof(DevGlobal) * (size_t)c->count, c->stream));
    }
    HPC_CUDA(cudaMemsetAsync(c->lc + first, 0, sizeof(LaunchCounters) * (size_t)(last - first + 1), c->stream));
    HPC_CUDA(cudaMemsetAsync(c->seg + (size_t)first * c->total_segs, 0,
                             sizeof(SegAgg) * (size_t)c->total_segs * (size_t)(last - first + 1), c->stream));
    for (int l = first; l <= last; ++l)
      if ((s = enqueue_level(c, l, timed)) != HPC_OK) return s;
    if (finalize) {
      if ((s = launch_finalize_records(c->inst, c->count, c->stream)) != HPC_OK) return s;
      c->timings.launches += 1;
    }
    return HPC_OK;
  };
  if (last >= 1) c->records_final = finalize;
  if (use_graph && c->graphs_enabled && first == 0 && capturable(c->stream)) {
    const bool valid = c->graph && c->graph_top == last && c->graph_stream == c->stream &&
                       c->graph_version == c->inst_version && c->graph_l1v == c->l1v_now &&
                       c->graph_set_mask == set_mask(c, last) &&
                       c->graph_final == finalize;
    if (!valid) {
      if (c->graph) cudaGraphExecDestroy(c->graph);
      c->graph = nullptr;
      cudaGraph_t g = nullptr;
      const int64_t launches = c->timings.launches;
      HPC_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      if ((s = enqueue_all(false)) != HPC_OK) {
        cudaStreamEndCapture(c->stream, &g);
        if (g) cudaGraphDestroy(g);
        return s;
      }
      HPC_CUDA(cudaStreamEndCapture(c->stream, &g));
      c->graph_launches = c->timings.launches - launches;
      c->timings.launches = launches;  // counted when the graph runs
      const cudaError_t e = cudaGraphInstantiate(&c->graph, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) {
        c->graph = nullptr;
        return cuda_fail(e, "cudaGraphInstantiate", __FILE__, __LINE__);
      }
      c->graph_top = last;
      c->graph_stream = c->stream;
      c->graph_version = c->inst_version;
      c->graph_l1v = c->l1v_now;
      c->graph_set_mask = set_mask(c, last);
      c->graph_final = finalize;
    }
    HPC_CUDA(cudaGraphLaunch(c->graph, c->stream));
    c->timings.launches += c->graph_launches;
    c->last_run_graph = true;
  } else {
    if ((s = enqueue_all(true)) != HPC_OK) return s;
    c->last_run_graph = false;
  }
  return wait ? pull_counters(c) : HPC_OK;
}

// ---- correlation ----------------------------------------------------------

// Shape metadata of the grouped correlation kernels (device arrays), built once.
hpc_status ensure_meta(hpc_ctx *c) {
  if (c->meta) return HPC_OK;
  const int C = c->count;
  // layout: row_prefix (C+1) | x_off | z_off | n | tc_off | n_pad | kdim | tile64 (C+1) | c_off | p | tiletc (C+1)
  std::vector<long long> m((size_t)(11 * C + 3), 0);
  long long *row_prefix = m.data(), *x_off = row_prefix + (C + 1), *z_off = x_off + C, *n = z_off + C;
  long long *tc_off = n + C, *n_pad = tc_off + C, *kdim = n_pad + C, *tile64 = kdim + C;
  long long *c_off = tile64 + (C + 1), *p = c_off + C, *tiletc = p + C;
  long long rows = 0, xo = 0, t64 = 0, ttc = 0;
  for (int b = 0; b < C; ++b) {
    const InstHost &h = c->ih[b];
    row_prefix[b] = rows;
    rows += h.p;
    x_off[b] = xo;
    z_off[b] = h.z_off;
    xo += h.n * h.p;
    n[b] = h.n;
    tc_off[b] = h.tc_off;
    n_pad[b] = tc_n_pad(h.n);
    kdim[b] = tc_k(h.n);
    tile64[b] = t64;
    t64 += gram_f64_tiles(h.p);
    c_off[b] = h.cor_off;
    p[b] = h.p;
    tiletc[b] = ttc;
    ttc += gram_tc_tiles(h.p);
  }
  row_prefix[C] = rows;
  tile64[C] = t64;
  tiletc[C] = ttc;
  c->tiles64 = t64;
  c->tiles_tc = ttc;
  std::vector<double> den((size_t)C);
  for (int b = 0; b < C; ++b) den[b] = denom_of(c, c->ih[b].n);
  hpc_status s;
  if ((s = dev_alloc(&c->meta, (int64_t)m.size(), "correlation metadata")) != HPC_OK) return s;
  if ((s = dev_alloc(&c->meta_denom, C, "correlation metadata")) != HPC_OK) return s;
  HPC_CUDA(cudaMemcpyAsync(c->meta, m.data(), sizeof(long long) * m.size(), cudaMemcpyHostToDevice, c->stream));
  HPC_CUDA(cudaMemcpyAsync(c->meta_denom, den.data(), sizeof(double) * den.size(), cudaMemcpyHostToDevice, c->stream));
  HPC_CUDA(cudaStreamSynchronize(c->stream));
  return HPC_OK;
}

StdArgs std_args(hpc_ctx *c) {
  const int C = c->count;
  long long *m = c->meta;
  StdArgs a{};
  a.count = C;
  a.row_prefix = m;
  a.x_off = m + (C + 1);
  a.z_off = a.x_off + C;
  a.n = a.z_off + C;
  a.tc_off = a.n + C;
  a.n_pad = a.tc_off + C;
  a.kdim = a.n_pad + C;
  a.ref_compat = c->opts.ref_compat_sd;
  return a;
}

GramArgs gram_args(hpc_ctx *c) {
  const StdArgs sa = std_args(c);
  GramArgs g{};
  g.count = c->count;
  g.tile_prefix = sa.kdim + c->count;
  g.z_off = sa.z_off;
  g.c_off = g.tile_prefix + (c->count + 1);
  g.n = sa.n;
  g.p = g.c_off + c->count;
  g.denom = c->meta_denom;
  return g;
}

// Entries of the deferred FP64 re-test queue (tensor-core mode): a test is queued when
// its FP32 |r| lies within the band around r_crit, about 4e-5 of the tests of a wide
// level 1 (4.7 M of 1.1e11 at p = 15000), so the queue grows with sum p^2 / 16, from 1 Mi
// to 16 Mi entries (144 B each). Tests beyond it are re-tested in place.
long long retest_queue_cap(long long sum_p2) {
  return std::min<long long>(64ll << 20, std::max<long long>(1ll << 20, sum_p2 / 16));
}

// The deferred FP64 re-test queue, allocated before the first run of a context
// without an FP64 matrix (tensor-core mode); contexts whose levels run elsewhere (the
// server's shared launches bring their own queue) never allocate it.
// queue of `cap` items with its entry scratch and zeroed done counters
hpc_status alloc_rq(hpc_ctx *c, long long cap) {
  hpc_status s;
  if ((s = dev_alloc(&c->rq, cap, "re-test queue")) != HPC_OK) return s;
  c->rq_cap = cap;
  const long long vcap = retest_scratch_entries(cap);
  if ((s = dev_alloc(&c->rq_val, vcap, "re-test entries")) != HPC_OK) return s;
  if ((s = dev_alloc(&c->rq_done, cap, "re-test counters")) != HPC_OK) return s;
  c->rq_vcap = vcap;
  HPC_CUDA(cudaMemsetAsync(c->rq_done, 0, sizeof(unsigned int) * (size_t)cap, c->stream));
  ++c->inst_version;  // a captured graph holds the queue pointers
  return HPC_OK;
}

hpc_status ensure_rq(hpc_ctx *c) {
  if (c->rq || c->cor64_valid) return HPC_OK;
  long long p2 = 0;
  for (const auto &h : c->ih) p2 += h.p * h.p;
  return alloc_rq(c, retest_queue_cap(p2));
}

hpc_status after_correlation(hpc_ctx *c) {
  c->have_cor = true;
  hpc_status s = write_inst_table(c);
  if (s != HPC_OK) return s;
  return hpc_ctx_reset(c);
}

hpc_status correlation_device(hpc_ctx *c, const void *X, bool f32) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if (!X) {
    set_error("null observation pointer");
    return HPC_ERR_INVALID_ARG;
  }
  if ((s = ensure_meta(c)) != HPC_OK) return s;
  long long ztot = 0;
  for (const auto &h : c->ih) ztot += h.n * h.p;
  const bool tc = c->opts.precision == HPC_PREC_MIXED_TC;
  // Tensor-core mode with FP32 observations keeps the standardised data as FP32 pairs
  // (zh + zl, FP64-grade, formed without FP64 arithmetic) instead of FP64: the FP64
  // entries of the re-tests are dot products of those.
  const bool pair = tc && f32;
  c->z_valid = false;
  c->zpair_valid = false;
  c->ztot = ztot;
  if (!pair && !c->Z && (s = dev_alloc(&c->Z, ztot, "standardised data")) != HPC_OK) return s;
  if (pair && !c->zpair && (s = dev_alloc(&c->zpair, 2 * ztot, "standardised data (FP32 pairs)")) != HPC_OK) return s;
  if (pair) {
    // the re-tests' entry store: sum p^2 doubles (instance b at its cor_off) and one bit
    // each, the bits cleared for the new data
    long long ent = 0;
    for (const auto &h : c->ih) ent = std::max(ent, h.cor_off + h.p * h.p);
    const long long words = (ent + 31) / 32 + 1;
    if (!c->ecache) {
      if ((s = dev_alloc(&c->ecache, ent, "re-test entries")) != HPC_OK) return s;
      if ((s = dev_alloc(&c->evalid, words, "re-test entry bits")) != HPC_OK) return s;
      c->evalid_words = words;
    }
    HPC_CUDA(cudaMemsetAsync(c->evalid, 0, sizeof(uint32_t) * (size_t)c->evalid_words, c->stream));
  }
  StdArgs sa = std_args(c);
  HPC_CUDA(cudaEventRecord(c->evc[0], c->stream));
  if (tc) {
    if (!c->tcP) {
      long long tt = 0;
      for (const auto &h : c->ih) tt += tc_p_pad(h.p) * tc_k(h.n);
      if ((s = dev_alloc(&c->tcP, tt, "tensor-core operand")) != HPC_OK) return s;
      HPC_CUDA(cudaMemsetAsync(c->tcP, 0, sizeof(__nv_bfloat16) * tt, c->stream));
      std::vector<CUtensorMap> maps((size_t)(2 * c->count));
      for (int b = 0; b < c->count; ++b) {
        const InstHost &h = c->ih[b];
        if ((s = tc_make_maps(&maps[2 * b], &maps[2 * b + 1], c->tcP + h.tc_off, c->tcP + h.tc_off, h.p, h.n)) !=
            HPC_OK)
          return s;
      }
      if ((s = dev_alloc(&c->tc_maps, 2 * c->count, "tensor maps")) != HPC_OK) return s;
      HPC_CUDA(cudaMemcpyAsync(c->tc_maps, maps.data(), sizeof(CUtensorMap) * maps.size(), cudaMemcpyHostToDevice,
                               c->stream));
      HPC_CUDA(cudaStreamSynchronize(c->stream));
    }
    if ((s = launch_standardise(X, f32, sa, sa.count ? c->total_rows : 0, pair ? nullptr : c->Z,
                                pair ? c->zpair : nullptr, ztot, c->tcP, c->stream)) != HPC_OK)
      return s;
    c->z_valid = !pair;
    c->zpair_valid = pair;
    HPC_CUDA(cudaEventRecord(c->evc[1], c->stream));
    TcArgs ta{};
    ta.count = c->count;
    ta.tile_prefix = gram_args(c).p + c->count;
    ta.maps = c->tc_maps;
    ta.c_off = gram_args(c).c_off;
    ta.p = gram_args(c).p;
    ta.n = sa.n;
    ta.err = &c->gctr[0].err;
    if ((s = launch_gram_tc(c->cor32, ta, c->tiles_tc, c->stream)) != HPC_OK) return s;
    HPC_CUDA(cudaEventRecord(c->evc[2], c->stream));
    c->cor64_valid = false;  // FP64 entries come from standardised dot products in the re-test kernels
    c->cor32_rounded = false;
    c->timings.launches += 2;
  } else {
    if ((s = launch_standardise(X, f32, sa, c->total_rows, c->Z, nullptr, 0, nullptr, c->stream)) != HPC_OK)
      return s;
    c->z_valid = true;
    HPC_CUDA(cudaEventRecord(c->evc[1], c->stream));
    c->cor64_valid = true;
    c->cor32_rounded = true;
    // FP64-accurate correlation: on the tensor cores by exact digits where that serves
    // (mixed precision, one instance of a few hundred variables or more), else the
    // FP64 SIMT Gram (the plain path, batches, small problems)
    const InstHost &h0 = c->ih[0];
    if (c->opts.precision == HPC_PREC_MIXED && c->count == 1 && emu_eligible(h0.p, h0.n)) {
      if (!c->emuD && (s = dev_alloc(&c->emuD, emu_digit_elems(h0.p, h0.n), "digit planes")) != HPC_OK) return s;
      if (!c->emuE && (s = dev_alloc(&c->emuE, emu_p_pad(h0.p), "digit exponents")) != HPC_OK) return s;
      if ((s = launch_gram_emu(c->Z, h0.p, h0.n, denom_of(c, h0.n), c->emuD, c->emuE, nullptr, c->cor64, c->cor32,
                               &c->gctr[0].err, c->stream)) != HPC_OK)
        return s;
      HPC_CUDA(cudaEventRecord(c->evc[2], c->stream));
      c->timings.launches += 3;
    } else {
      if ((s = launch_gram_f64(c->Z, c->cor64, gram_args(c), c->tiles64, c->stream)) != HPC_OK) return s;
      HPC_CUDA(cudaEventRecord(c->evc[2], c->stream));
      c->timings.launches += 2;
      if (c->opts.precision == HPC_PREC_MIXED) {
        long long tot = 0;
        for (const auto &h : c->ih) tot += h.p * h.p;
        if ((s = launch_to_f32(c->cor64, tot, c->cor32, c->stream)) != HPC_OK) return s;
        c->timings.launches += 1;
      }
    }
  }
  HPC_CUDA(cudaEventRecord(c->evc[3], c->stream));
  c->cor_timed = true;
  return after_correlation(c);
}

hpc_status correlation_host(hpc_ctx *c, const void *X, bool f32) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if (!X) {
    set_error("null observation pointer");
    return HPC_ERR_INVALID_ARG;
  }
  long long elems = 0;
  for (const auto &h : c->ih) elems += h.n * h.p;
  const int64_t bytes = elems * (f32 ? 4 : 8);
  if (c->X_stage_bytes < bytes) {
    HPC_CUDA(cudaStreamSynchronize(c->stream));
    uint8_t *old = (uint8_t *)c->X_stage;
    dev_free(old);
    c->X_stage = nullptr;
    c->X_stage_bytes = 0;
    uint8_t *buf = nullptr;
    if ((s = dev_alloc(&buf, bytes, "observation staging")) != HPC_OK) return s;
    c->X_stage = buf;
    c->X_stage_bytes = bytes;
  }
  HPC_CUDA(cudaMemcpyAsync(c->X_stage, X, (size_t)bytes, cudaMemcpyHostToDevice, c->stream));
  return correlation_device(c, c->X_stage, f32);
}

// A loaded FP64 matrix (every instance): the mixed modes test on its FP32 rounding.
hpc_status load_correlation(hpc_ctx *c, const double *C, cudaMemcpyKind kind) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if (!C) {
    set_error("null correlation pointer");
    return HPC_ERR_INVALID_ARG;
  }
  long long tot = 0;
  for (const auto &h : c->ih) tot += h.p * h.p;
  if (!c->cor64 && (s = dev_alloc(&c->cor64, tot, "cor64")) != HPC_OK) return s;
  if (c->opts.precision != HPC_PREC_FP64 && !c->cor32 && (s = dev_alloc(&c->cor32, tot, "cor32")) != HPC_OK)
    return s;
  HPC_CUDA(cudaMemcpyAsync(c->cor64, C, sizeof(double) * (size_t)tot, kind, c->stream));
  if (c->opts.precision != HPC_PREC_FP64) {
    if ((s = launch_to_f32(c->cor64, tot, c->cor32, c->stream)) != HPC_OK) return s;
    c->timings.launches += 1;
  }
  c->cor64_valid = true;
  c->cor32_rounded = true;
  return after_correlation(c);
}

hpc_status create(hpc_ctx **out, int count, const int64_t *p, const int64_t *n, const double *alpha,
                  const hpc_opts *opts);

}  // namespace

int set_order_from() { return g_set_from.load(); }
long long retest_scratch_entries(long long cap) { return std::min<long long>(32ll << 20, 3 * cap); }
bool uses_set_order(int set_from, int level) {
  return set_from > 0 && level >= 2 && level <= kSetTop && level >= set_from;
}

// for the server's shared launches (serve.cu)
hpc_status ctx_size_after_level0(hpc_ctx *c) {
  bool changed = false;
  return ensure_capacity(c, &changed);
}
long long ctx_retest_queue_bytes(long long sum_p2) {
  return retest_queue_cap(sum_p2) * (long long)sizeof(RetestItem);
}

}  // namespace hpc

using namespace hpc;

extern "C" {

const char *hpc_last_error_string(void) { return g_last_error.c_str(); }

const char *hpc_status_string(hpc_status s) {
  switch (s) {
    case HPC_OK: return "HPC_OK";
    case HPC_ERR_INVALID_ARG: return "HPC_ERR_INVALID_ARG";
    case HPC_ERR_OOM: return "HPC_ERR_OOM";
    case HPC_ERR_CUDA: return "HPC_ERR_CUDA";
    case HPC_ERR_TIMEOUT: return "HPC_ERR_TIMEOUT";
    case HPC_ERR_NUMERIC: return "HPC_ERR_NUMERIC";
    case HPC_ERR_STATE: return "HPC_ERR_STATE";
    case HPC_ERR_CAPACITY: return "HPC_ERR_CAPACITY";
    case HPC_ERR_NO_DEVICE: return "HPC_ERR_NO_DEVICE";
  }
  return "HPC_ERR_UNKNOWN";
}

hpc_status hpc_opts_default(hpc_opts *o) {
  if (!o) return HPC_ERR_INVALID_ARG;
  std::memset(o, 0, sizeof(*o));
  o->device = 0;
  o->alpha = 0.05;   // src/main.cpp:26
  o->max_level = 4;  // src/main.cpp:31
  o->precision = HPC_PREC_MIXED;
  o->retest_margin = 1e-3;
  o->ref_compat_sd = 0;
  o->verbose = 0;
  return HPC_OK;
}

hpc_status hpc_ctx_footprint(int64_t p, int64_t n, const hpc_opts *o, int64_t *bytes) {
  if (!o || !bytes || p < 2 || n < 4) return HPC_ERR_INVALID_ARG;
  const int64_t W = (p + 31) / 32;
  int64_t b = 0;
  if (o->precision != HPC_PREC_MIXED_TC) b += p * p * 8;           // cor64
  if (o->precision != HPC_PREC_FP64) b += p * p * 4;               // cor32
  if (o->precision == HPC_PREC_MIXED_TC) b += tc_p_pad(p) * tc_k(n) * 2;      // split operand planes
  if (o->precision == HPC_PREC_MIXED_TC) b += p * p * 8 + p * p / 8 + 8;     // re-test entry store and its bits
  b += n * p * 8;                                                  // standardised data (FP64 or FP32 pairs)
  b += n * p * 4;                                                  // observation staging
  b += p * W * 4 + p * p;                                          // adjacency bits + bytes
  b += (p + 1) * (4 + 4 + 8 + 1);                                  // deg, rowptr, row_work, stale-row marks
  b += (int64_t)(HPC_MAX_LEVEL + 1) * ((p + kSegRows - 1) / kSegRows) * (int64_t)sizeof(SegAgg);  // scan sums
  // neighbour lists and records are sized after level 0; budget an average degree of 64
  const int64_t e = std::min<int64_t>(p * (p - 1) / 2, p * 32);
  const int rec_ids = o->max_level < 0 ? HPC_MAX_LEVEL : std::min(std::max(o->max_level, 1), HPC_MAX_LEVEL);
  b += 2 * e * 4 + e * 4 * (int64_t)rec_stride_words(rec_ids);
  if (o->precision == HPC_PREC_MIXED_TC) {
    const int64_t cap = retest_queue_cap(p * p);
    b += cap * ((int64_t)sizeof(RetestItem) + 4) + retest_scratch_entries(cap) * 8;  // queue, counters, entries
  }
  *bytes = b;
  return HPC_OK;
}

hpc_status hpc_ctx_create(hpc_ctx **out, int64_t p, int64_t n, const hpc_opts *opts) {
  return create(out, 1, &p, &n, nullptr, opts);
}

hpc_status hpc_batch_create(hpc_ctx **out, int count, const int64_t *p, const int64_t *n, const double *alpha,
                            const hpc_opts *opts) {
  if (count < 1 || !p || !n) {
    set_error("batch needs count >= 1 and p, n arrays");
    return HPC_ERR_INVALID_ARG;
  }
  return create(out, count, p, n, alpha, opts);
}

hpc_status hpc_batch_size(hpc_ctx *c, int *count) {
  if (!c || !count) {
    set_error("null argument");
    return HPC_ERR_INVALID_ARG;
  }
  *count = c->count;
  return HPC_OK;
}

hpc_status hpc_ctx_destroy(hpc_ctx *c) {
  if (!c) return HPC_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  dev_free(c->cor64);
  dev_free(c->cor32);
  dev_free(c->Z);
  dev_free(c->zpair);
  dev_free(c->ecache);
  dev_free(c->evalid);
  dev_free(c->tcP);
  dev_free(c->emuD);
  dev_free(c->emuE);
  dev_free(c->tc_maps);
  {
    uint8_t *xs = (uint8_t *)c->X_stage;
    dev_free(xs);
    c->X_stage = nullptr;
  }
  dev_free(c->adj);
  dev_free(c->adj_bytes);
  dev_free(c->deg);
  dev_free(c->rowptr);
  dev_free(c->row_work);
  dev_free(c->row_dirty);
  dev_free(c->colidx);
  dev_free(c->recs);
  dev_free(c->rq);
  dev_free(c->rq_val);
  dev_free(c->rq_done);
  dev_free(c->ctr);
  dev_free(c->gctr);
  dev_free(c->lc);
  dev_free(c->inst);
  dev_free(c->prefixes);
  dev_free(c->work_prefix);
  dev_free(c->seg);
  dev_free(c->meta);
  dev_free(c->meta_denom);
  dev_free(c->tune_dev);
  dev_free(c->rec_stage);
  dev_free(c->rec_prefix_dev);
  dev_free(c->rec_seg);
  delete[] c->ctr_host;
  delete[] c->gctr_host;
  if (c->graph) cudaGraphExecDestroy(c->graph);
  for (auto &e : c->evc)
    if (e) cudaEventDestroy(e);
  for (auto &e : c->evr)
    if (e) cudaEventDestroy(e);
  for (auto &lv : c->evl)
    for (auto &e : lv)
      if (e) cudaEventDestroy(e);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  cudaGetLastError();
  delete c;
  return HPC_OK;
}

hpc_status hpc_ctx_reset(hpc_ctx *c) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  HPC_CUDA(cudaMemsetAsync(c->ctr, 0, sizeof(DevCounters) * (size_t)c->count * kLevels, c->stream));
  HPC_CUDA(cudaMemsetAsync(c->gctr, 0, sizeof(DevGlobal) * (size_t)c->count, c->stream));
  c->next_level = 0;
  for (auto &h : c->ih) h.edges = h.p * (h.p - 1) / 2;
  return HPC_OK;
}

hpc_status hpc_ctx_set_stream(hpc_ctx *c, void *stream) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  HPC_CUDA(cudaStreamSynchronize(c->stream));
  c->stream = stream ? (cudaStream_t)stream : c->own_stream;
  return HPC_OK;
}

hpc_status hpc_ctx_set_graphs(hpc_ctx *c, int enable) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  c->graphs_enabled = enable != 0;
  return HPC_OK;
}

hpc_status settle(hpc_ctx *c);

hpc_status hpc_ctx_set_tune(hpc_ctx *c, const hpc_tune_params *force) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if (force && !tune_params_valid(force)) {
    set_error("tile policy needs 1 <= tile_cap <= %d, 1 <= tiles_per_lane <= 64, edge_lanes 1 or 32, l1_prefetch 0 or 1",
              kTuneMaxCap);
    return HPC_ERR_INVALID_ARG;
  }
  if ((s = settle(c)) != HPC_OK) return s;
  c->tune_force = force ? tune_entry_of(*force) : TuneEntry{0, 0, 0, 0};
  ++c->inst_version;  // the policy is a launch parameter: graphs are captured anew
  return HPC_OK;
}

hpc_status hpc_autotune(hpc_ctx *c, const hpc_tune_params *cands, int ncands, int reps, hpc_tune_params *chosen,
                        int *entries) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if ((s = settle(c)) != HPC_OK) return s;
  if (!c->have_cor) {
    set_error("autotune before a correlation matrix was computed or loaded");
    return HPC_ERR_STATE;
  }
  if (reps < 1 || (cands && ncands < 1)) {
    set_error("autotune needs reps >= 1 and ncands >= 1");
    return HPC_ERR_INVALID_ARG;
  }
  std::vector<hpc_tune_params> grid;
  if (cands) {
    for (int q = 0; q < ncands; ++q) {
      if (!tune_params_valid(&cands[q])) {
        set_error("autotune candidate %d is not a valid tile policy", q);
        return HPC_ERR_INVALID_ARG;
      }
      grid.push_back(cands[q]);
    }
  } else {
    for (int v = 0; v < 3; ++v)  // level-1 variants: interleaved, interleaved with prefetch, chunked
      for (int cap : {16, 64, 256, 1024})
        for (int tpl : {2, 4, 8}) grid.push_back(hpc_tune_params{cap, tpl, v == 2 ? 1 : 32, v == 1 ? 1 : 0});
  }
  const bool graphs = c->graphs_enabled;
  const TuneEntry force0 = c->tune_force;
  c->graphs_enabled = false;  // kernel by kernel: every level's kernels are timed
  // every candidate's level times, the candidates taken in turn within each round (so
  // that a drift over the tuning run touches them alike); per level the candidate with
  // the smallest median over the rounds wins, not the one with the luckiest sample
  std::vector<std::vector<double>> ms_of(grid.size() * kLevels);
  int best[kLevels], max_deg[kLevels];
  for (int l = 0; l < kLevels; ++l) {
    best[l] = -1;
    max_deg[l] = -1;
  }
  hpc_level_stats st[kLevels];
  for (int r = 0; r < reps && s == HPC_OK; ++r) {
    for (size_t q = 0; q < grid.size() && s == HPC_OK; ++q) {
      c->tune_force = tune_entry_of(grid[q]);
      ++c->inst_version;
      int ran = 0;
      if ((s = hpc_ctx_reset(c)) != HPC_OK) break;
      if ((s = hpc_run_skeleton(c, st, kLevels, &ran)) != HPC_OK) break;
      for (int k = 0; k < ran; ++k) {
        const int l = st[k].level;
        if (l < 1 || st[k].potential_tests == 0) continue;
        max_deg[l] = st[k].max_degree;
        ms_of[q * kLevels + l].push_back(c->timings.test_ms[l]);
      }
    }
  }
  for (int l = 0; l < kLevels && s == HPC_OK; ++l) {
    double best_ms = 1e300;
    for (size_t q = 0; q < grid.size(); ++q) {
      std::vector<double> v = ms_of[q * kLevels + l];
      if (v.empty()) continue;
      std::sort(v.begin(), v.end());
      const double med = v.size() % 2 ? v[v.size() / 2] : 0.5 * (v[v.size() / 2 - 1] + v[v.size() / 2]);
      if (med < best_ms) {
        best_ms = med;
        best[l] = (int)q;
      }
    }
  }
  c->tune_force = force0;
  c->graphs_enabled = graphs;
  ++c->inst_version;
  const hpc_status reset = hpc_ctx_reset(c);
  if (s != HPC_OK) return s;
  if (reset != HPC_OK) return reset;
  int64_t pmax = 0;
  for (const auto &h : c->ih) pmax = std::max<int64_t>(pmax, h.p);
  int written = 0;
  for (int l = 0; l < kLevels; ++l) {
    if (chosen) chosen[l] = best[l] >= 0 ? grid[(size_t)best[l]] : hpc_tune_params{0, 0, 0, 0};
    if (best[l] < 0) continue;
    tune_store(pmax, l, max_deg[l], tune_entry_of(grid[(size_t)best[l]]));
    ++written;
  }
  if (entries) *entries = written;
  return HPC_OK;
}

hpc_status hpc_get_timings(hpc_ctx *c, hpc_timings *out) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if (!out) {
    set_error("null output pointer");
    return HPC_ERR_INVALID_ARG;
  }
  if (c->cor_timed) {
    HPC_CUDA(cudaEventSynchronize(c->evc[3]));
    float a = 0.f, b = 0.f, d = 0.f;
    HPC_CUDA(cudaEventElapsedTime(&a, c->evc[0], c->evc[1]));
    HPC_CUDA(cudaEventElapsedTime(&b, c->evc[1], c->evc[2]));
    HPC_CUDA(cudaEventElapsedTime(&d, c->evc[2], c->evc[3]));
    c->timings.standardise_ms = a;
    c->timings.gram_ms = b;
    c->timings.convert_ms = d;
  }
  *out = c->timings;
  return HPC_OK;
}

hpc_status hpc_correlation_f64(hpc_ctx *c, const double *X) { return correlation_host(c, X, false); }
hpc_status hpc_correlation_f32(hpc_ctx *c, const float *X) { return correlation_host(c, X, true); }
hpc_status hpc_correlation_device_f64(hpc_ctx *c, const double *X) { return correlation_device(c, X, false); }
hpc_status hpc_correlation_device_f32(hpc_ctx *c, const float *X) { return correlation_device(c, X, true); }
hpc_status hpc_load_correlation(hpc_ctx *c, const double *C) { return load_correlation(c, C, cudaMemcpyHostToDevice); }
hpc_status hpc_load_correlation_device(hpc_ctx *c, const double *C) {
  return load_correlation(c, C, cudaMemcpyDeviceToDevice);
}

hpc_status hpc_batch_offsets(hpc_ctx *c, int64_t *obs_offsets, int64_t *cor_offsets) {
  if (!c) {
    set_error("null context");
    return HPC_ERR_INVALID_ARG;
  }
  long long xo = 0;
  for (int b = 0; b < c->count; ++b) {
    if (obs_offsets) obs_offsets[b] = xo;
    if (cor_offsets) cor_offsets[b] = c->ih[b].cor_off;
    xo += c->ih[b].n * c->ih[b].p;
  }
  if (obs_offsets) obs_offsets[c->count] = xo;
  if (cor_offsets) cor_offsets[c->count] = c->ih.back().cor_off + c->ih.back().p * c->ih.back().p;
  return HPC_OK;
}

hpc_status hpc_get_correlation(hpc_ctx *c, double *C) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if (!C || !c->have_cor) {
    set_error(!C ? "null output pointer" : "no correlation matrix yet");
    return !C ? HPC_ERR_INVALID_ARG : HPC_ERR_STATE;
  }
  long long tot = 0;
  for (const auto &h : c->ih) tot += h.p * h.p;
  if (!c->cor64_valid) {
    // tensor-core mode keeps no FP64 matrix: form it from the standardised data (FP64
    // from the FP32 pairs where the context keeps those: the values the re-tests use)
    if (!c->cor64 && (s = dev_alloc(&c->cor64, tot, "cor64")) != HPC_OK) return s;
    if (!c->z_valid) {
      if (!c->zpair_valid) return HPC_ERR_STATE;
      if (!c->Z && (s = dev_alloc(&c->Z, c->ztot, "standardised data")) != HPC_OK) return s;
      if ((s = launch_pair_to_f64(c->zpair, c->zpair + c->ztot, c->ztot, c->Z, c->stream)) != HPC_OK) return s;
      c->z_valid = true;
    }
    if ((s = launch_gram_f64(c->Z, c->cor64, gram_args(c), c->tiles64, c->stream)) != HPC_OK) return s;
    c->cor64_valid = true;
    if ((s = write_inst_table(c)) != HPC_OK) return s;
  }
  HPC_CUDA(cudaMemcpyAsync(C, c->cor64, sizeof(double) * (size_t)tot, cudaMemcpyDeviceToHost, c->stream));
  HPC_CUDA(cudaStreamSynchronize(c->stream));
  return HPC_OK;
}

hpc_status hpc_get_correlation_f32(hpc_ctx *c, float *C) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if (!C || !c->have_cor || !c->cor32) {
    set_error(!C ? "null output pointer" : "no FP32 correlation (plain FP64 precision or none computed)");
    return !C ? HPC_ERR_INVALID_ARG : HPC_ERR_STATE;
  }
  long long tot = 0;
  for (const auto &h : c->ih) tot += h.p * h.p;
  HPC_CUDA(cudaMemcpyAsync(C, c->cor32, sizeof(float) * (size_t)tot, cudaMemcpyDeviceToHost, c->stream));
  HPC_CUDA(cudaStreamSynchronize(c->stream));
  return HPC_OK;
}

// results and further runs first collect a pending asynchronous run
hpc_status settle(hpc_ctx *c) { return c->async_pending ? hpc_wait(c, nullptr, 0, nullptr) : HPC_OK; }

hpc_status hpc_run_level(hpc_ctx *c, int level, hpc_level_stats *st) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if ((s = settle(c)) != HPC_OK) return s;
  if (!c->have_cor) {
    set_error("run before a correlation matrix was computed or loaded");
    return HPC_ERR_STATE;
  }
  if (level != c->next_level) {
    set_error("level %d requested, next level is %d", level, c->next_level);
    return HPC_ERR_STATE;
  }
  if (level > HPC_MAX_LEVEL) {
    set_error("level %d above HPC_MAX_LEVEL", level);
    return HPC_ERR_INVALID_ARG;
  }
  if (level > c->rec_ids) {  // the records hold ids up to the context's max_level
    set_error("level %d above the context's max_level %d", level, c->opts.max_level);
    return HPC_ERR_INVALID_ARG;
  }
  if ((s = ensure_rq(c)) != HPC_OK) return s;
  if (level == 1) {
    bool changed = false;
    if ((s = ensure_capacity(c, &changed)) != HPC_OK) return s;
  }
  c->level_by_level = true;
  s = run_levels(c, level, level, false);
  c->level_by_level = false;
  if (s != HPC_OK) return s;
  if ((s = global_errors(c)) != HPC_OK) return s;
  if (needs_rerun(c)) {
    set_error("neighbour-list buffer too small");
    return HPC_ERR_CAPACITY;
  }
  c->next_level = level + 1;
  return collect_level(c, level, st);
}

// Levels first..top in chunks with a host check in between, until a level has no
// tests: a known max level runs as one chunk (one graph replay from level 0); "until
// exhausted" starts with the previous run's extent (exhaust_top) as one chunk and
// continues four levels at a time. *last_run: the last level run; *overflow: the
// neighbour lists were too small (the caller resizes and reruns).
static hpc_status run_chunks(hpc_ctx *c, int first, int top, int *last_run, bool *overflow) {
  hpc_status s;
  const bool known = c->opts.max_level >= 0;
  *overflow = false;
  *last_run = first - 1;
  bool done = false;
  while (!done && first <= top) {
    int last = std::min(top, first + 3);
    if (known) last = top;
    else if (first == 0 && c->exhaust_top >= 1) last = std::min(top, c->exhaust_top);
    if ((s = run_levels(c, first, last, known || first == 0, true, true)) != HPC_OK) return s;
    *last_run = last;
    if (needs_rerun(c)) {
      *overflow = true;
      return HPC_OK;
    }
    if ((s = global_errors(c)) != HPC_OK) return s;
    done = last >= 1 && !any_work(c, last);
    first = last + 1;
  }
  return HPC_OK;
}

// the first level >= 1 without tests (where a run until exhausted stops), else last
static int exhausted_at(hpc_ctx *c, int last) {
  for (int l = 1; l <= last; ++l)
    if (!any_work(c, l)) return l;
  return last;
}

hpc_status hpc_run_skeleton(hpc_ctx *c, hpc_level_stats *stats, int cap, int *levels_run) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if ((s = settle(c)) != HPC_OK) return s;
  if (!c->have_cor) {
    set_error("run before a correlation matrix was computed or loaded");
    return HPC_ERR_STATE;
  }
  const int top = c->opts.max_level < 0 ? HPC_MAX_LEVEL : c->opts.max_level;
  int ran = 0;
  auto emit = [&](int l) -> hpc_status {
    hpc_level_stats st{};
    const hpc_status e = collect_level(c, l, &st);
    if (e != HPC_OK) return e;
    if (stats && ran < cap) stats[ran] = st;
    ++ran;
    return HPC_OK;
  };
  // levels run one by one through hpc_run_level before: continue the same way
  if (c->next_level != 0) {
    for (int l = c->next_level; l <= top; ++l) {
      if ((s = hpc_run_level(c, l, nullptr)) != HPC_OK) return s;
      if ((s = emit(l)) != HPC_OK) return s;
      if (l >= 1 && !any_work(c, l)) break;
    }
    if (levels_run) *levels_run = ran;
    return HPC_OK;
  }
  if ((s = ensure_rq(c)) != HPC_OK) return s;
  HPC_CUDA(cudaEventRecord(c->evr[0], c->stream));
  for (int attempt = 0; attempt < 3; ++attempt) {
    ran = 0;
    for (auto &h : c->ih) h.edges = h.p * (h.p - 1) / 2;
    const bool sized = c->colidx && c->recs;
    int first = 0;
    if (!sized) {
      // first run: level 0 alone sizes the neighbour-list and record buffers
      if ((s = run_levels(c, 0, 0, false)) != HPC_OK) return s;
      bool changed;
      if ((s = ensure_capacity(c, &changed)) != HPC_OK) return s;
      first = 1;
    }
    bool overflow = false;
    int last_run = first - 1;
    if ((s = run_chunks(c, first, top, &last_run, &overflow)) != HPC_OK) return s;
    if (overflow) {
      // the data changed since the buffers were sized: resize from level 0 and rerun
      bool changed;
      if ((s = ensure_capacity(c, &changed)) != HPC_OK) return s;
      if ((s = hpc_ctx_reset(c)) != HPC_OK) return s;
      continue;
    }
    c->next_level = last_run + 1;
    if (c->opts.max_level < 0) c->exhaust_top = exhausted_at(c, last_run);
    HPC_CUDA(cudaEventRecord(c->evr[1], c->stream));
    HPC_CUDA(cudaEventSynchronize(c->evr[1]));
    float tr = 0.f;
    HPC_CUDA(cudaEventElapsedTime(&tr, c->evr[0], c->evr[1]));
    c->timings.skeleton_ms = tr;
    for (int l = 0; l <= last_run; ++l) {
      if ((s = emit(l)) != HPC_OK) return s;
      if (l >= 1 && !any_work(c, l)) break;
    }
    if (levels_run) *levels_run = ran;
    return HPC_OK;
  }
  set_error("neighbour-list buffer still too small after resizing");
  return HPC_ERR_CAPACITY;
}

hpc_status hpc_run_skeleton_async(hpc_ctx *c) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if (!c->have_cor) {
    set_error("run before a correlation matrix was computed or loaded");
    return HPC_ERR_STATE;
  }
  const bool known = c->opts.max_level >= 0;
  if (!(c->colidx && c->recs) || !c->graphs_enabled || !capturable(c->stream) || (!known && c->exhaust_top < 1)) {
    // the first run sizes the neighbour lists (and, until exhausted, finds the extent
    // of the levels); uncapturable streams run eagerly
    c->async_pending = false;
    if ((s = hpc_ctx_reset(c)) != HPC_OK) return s;
    return hpc_run_skeleton(c, nullptr, 0, nullptr);
  }
  if ((s = ensure_rq(c)) != HPC_OK) return s;
  // until exhausted: the previous run's extent, continued by hpc_wait if the data now
  // reach further
  const int top = known ? c->opts.max_level : c->exhaust_top;
  for (auto &h : c->ih) h.edges = h.p * (h.p - 1) / 2;
  HPC_CUDA(cudaEventRecord(c->evr[0], c->stream));
  if ((s = run_levels(c, 0, top, true, false, true)) != HPC_OK) return s;
  HPC_CUDA(cudaEventRecord(c->evr[1], c->stream));
  c->async_pending = true;
  c->async_top = top;
  c->next_level = 0;
  return HPC_OK;
}

hpc_status hpc_wait(hpc_ctx *c, hpc_level_stats *stats, int cap, int *levels_run) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  int ran = 0;
  if (c->async_pending) {
    c->async_pending = false;
    if ((s = pull_counters(c)) != HPC_OK) return s;
    if (needs_rerun(c)) {
      // the data changed since the neighbour lists were sized: resize and rerun
      bool changed;
      if ((s = ensure_capacity(c, &changed)) != HPC_OK) return s;
      if ((s = hpc_ctx_reset(c)) != HPC_OK) return s;
      return hpc_run_skeleton(c, stats, cap, levels_run);
    }
    if ((s = global_errors(c)) != HPC_OK) return s;
    int last_run = c->async_top;
    if (c->opts.max_level < 0) {
      if (last_run < HPC_MAX_LEVEL && any_work(c, last_run)) {
        // the data reach beyond the previous run's extent: continue from here
        bool overflow = false;
        if ((s = run_chunks(c, c->async_top + 1, HPC_MAX_LEVEL, &last_run, &overflow)) != HPC_OK) return s;
        if (overflow) {
          bool changed;
          if ((s = ensure_capacity(c, &changed)) != HPC_OK) return s;
          if ((s = hpc_ctx_reset(c)) != HPC_OK) return s;
          return hpc_run_skeleton(c, stats, cap, levels_run);
        }
        HPC_CUDA(cudaEventRecord(c->evr[1], c->stream));
        HPC_CUDA(cudaEventSynchronize(c->evr[1]));
      }
      c->exhaust_top = exhausted_at(c, last_run);
    }
    c->next_level = last_run + 1;
    float tr = 0.f;
    HPC_CUDA(cudaEventElapsedTime(&tr, c->evr[0], c->evr[1]));
    c->timings.skeleton_ms = tr;
  }
  for (int l = 0; l < c->next_level; ++l) {
    hpc_level_stats st{};
    if ((s = collect_level(c, l, &st)) != HPC_OK) return s;
    if (stats && ran < cap) stats[ran] = st;
    ++ran;
    if (l >= 1 && !any_work(c, l)) break;
  }
  if (levels_run) *levels_run = ran;
  return HPC_OK;
}

hpc_status hpc_batch_level_stats(hpc_ctx *c, int idx, hpc_level_stats *out, int cap, int *levels) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if ((s = settle(c)) != HPC_OK) return s;
  if ((s = check_index(c, idx)) != HPC_OK) return s;
  int k = 0;
  for (int l = 0; l < c->next_level && l <= HPC_MAX_LEVEL; ++l) {
    if (out && k < cap) out[k] = level_stats_of(c, l, idx);
    ++k;
  }
  if (levels) *levels = k;
  return HPC_OK;
}

hpc_status hpc_batch_get_adjacency(hpc_ctx *c, int idx, uint8_t *out) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if ((s = settle(c)) != HPC_OK) return s;
  if ((s = check_index(c, idx)) != HPC_OK) return s;
  if (!out) {
    set_error("null output pointer");
    return HPC_ERR_INVALID_ARG;
  }
  const InstHost &h = c->ih[idx];
  if (c->next_level == 0) {
    for (int64_t i = 0; i < h.p; ++i)
      for (int64_t j = 0; j < h.p; ++j) out[i * h.p + j] = (uint8_t)(i != j);
    return HPC_OK;
  }
  if (!c->adj_bytes) {
    int64_t pm = 0;
    for (const auto &x : c->ih) pm = std::max(pm, x.p);
    if ((s = dev_alloc(&c->adj_bytes, pm * pm, "adjacency bytes")) != HPC_OK) return s;
  }
  if ((s = launch_expand_adjacency(c->adj + h.adj_off, h.p, h.W, c->adj_bytes, c->stream)) != HPC_OK) return s;
  c->timings.launches += 1;
  HPC_CUDA(cudaMemcpyAsync(out, c->adj_bytes, (size_t)(h.p * h.p), cudaMemcpyDeviceToHost, c->stream));
  HPC_CUDA(cudaStreamSynchronize(c->stream));
  return HPC_OK;
}

hpc_status hpc_get_adjacency(hpc_ctx *c, uint8_t *out) { return hpc_batch_get_adjacency(c, 0, out); }

hpc_status hpc_batch_edge_count(hpc_ctx *c, int idx, int64_t *edges) {
  if (!c || !edges) {
    set_error("null argument");
    return HPC_ERR_INVALID_ARG;
  }
  hpc_status s = check_index(c, idx);
  if (s != HPC_OK) return s;
  if ((s = settle(c)) != HPC_OK) return s;
  *edges = c->ih[idx].edges;
  return HPC_OK;
}

hpc_status hpc_edge_count(hpc_ctx *c, int64_t *edges) { return hpc_batch_edge_count(c, 0, edges); }

// FP64 p-values of the FP32-decided removals of every instance, once per run.
static hpc_status finalize_records(hpc_ctx *c) {
  if (c->records_final || !c->recs) return HPC_OK;
  hpc_status s;
  if ((s = launch_finalize_records(c->inst, c->count, c->stream)) != HPC_OK) return s;
  c->timings.launches += 1;
  HPC_CUDA(cudaMemcpyAsync(c->gctr_host, c->gctr, sizeof(DevGlobal) * (size_t)c->count, cudaMemcpyDeviceToHost,
                           c->stream));
  HPC_CUDA(cudaStreamSynchronize(c->stream));
  c->records_final = true;
  for (int b = 0; b < c->count; ++b)
    if (c->gctr_host[b].err & kErrBandViolation) {
      set_error("instance %d: an FP32 removal was not confirmed in FP64 (error bound violated)", b);
      return HPC_ERR_NUMERIC;
    }
  return HPC_OK;
}

hpc_status hpc_batch_get_sepset_records_from(hpc_ctx *c, int idx, int64_t first, hpc_sepset_record *out, int64_t cap,
                                             int64_t *count) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if ((s = settle(c)) != HPC_OK) return s;
  if ((s = check_index(c, idx)) != HPC_OK) return s;
  if (!count || first < 0) {
    set_error(!count ? "null count pointer" : "negative first record");
    return HPC_ERR_INVALID_ARG;
  }
  if ((s = finalize_records(c)) != HPC_OK) return s;
  DevGlobal g{};
  HPC_CUDA(cudaMemcpyAsync(&g, c->gctr + idx, sizeof(g), cudaMemcpyDeviceToHost, c->stream));
  HPC_CUDA(cudaStreamSynchronize(c->stream));
  const InstHost &h = c->ih[idx];
  const long long n = c->recs ? std::min<long long>((long long)g.rec_count, h.rec_cap) : 0;
  *count = n;
  if (out && cap > 0 && first < n) {
    const int64_t k = std::min<int64_t>(cap, n - first);
    const int stride = rec_stride_words(c->rec_ids);
    std::vector<int32_t> raw((size_t)k * stride);
    HPC_CUDA(cudaMemcpyAsync(raw.data(), c->recs + h.rec_off + first * stride, sizeof(int32_t) * raw.size(),
                             cudaMemcpyDeviceToHost, c->stream));
    HPC_CUDA(cudaStreamSynchronize(c->stream));
    for (int64_t r = 0; r < k; ++r) {  // packed records -> hpc_sepset_record
      const int32_t *rec = raw.data() + (size_t)r * stride;
      RecHead head;
      std::memcpy(&head, rec, sizeof(head));
      hpc_sepset_record &o = out[r];
      o.i = head.i;
      o.j = head.j;
      o.level = head.level;
      o.pad = 0;
      o.pmax = head.pmax;
      for (int q = 0; q < HPC_MAX_LEVEL; ++q) o.ids[q] = q < c->rec_ids ? rec[kRecHeadWords + q] : -1;
    }
  }
  return HPC_OK;
}

hpc_status hpc_batch_get_sepset_records(hpc_ctx *c, int idx, hpc_sepset_record *out, int64_t cap, int64_t *count) {
  return hpc_batch_get_sepset_records_from(c, idx, 0, out, cap, count);
}

hpc_status hpc_get_sepset_records(hpc_ctx *c, hpc_sepset_record *out, int64_t cap, int64_t *count) {
  return hpc_batch_get_sepset_records(c, 0, out, cap, count);
}

hpc_status hpc_batch_get_records_packed(hpc_ctx *c, int32_t *out, int64_t cap_words, int64_t *inst_words) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if ((s = settle(c)) != HPC_OK) return s;
  if (!inst_words) {
    set_error("null inst_words pointer");
    return HPC_ERR_INVALID_ARG;
  }
  if ((s = finalize_records(c)) != HPC_OK) return s;
  if ((s = pull_counters(c)) != HPC_OK) return s;
  // records and packed words per instance, from its removals per level (a level's
  // removals are its records; level 0 writes none)
  std::vector<long long> pre((size_t)c->count + 1, 0), wpre((size_t)c->count + 1, 0);
  for (int b = 0; b < c->count; ++b) {
    long long n = 0, w = 0;
    for (int l = 1; l < kLevels && l < c->next_level; ++l) {
      const long long d = (long long)c->ctr_host[(size_t)b * kLevels + l].deleted;
      n += d;
      w += d * (6 + ((l + 1) & ~1));
    }
    if (c->recs && n > std::min<long long>((long long)c->gctr_host[b].rec_count, c->ih[b].rec_cap)) {
      set_error("instance %d: record counts disagree (%lld removals, %lld records)", b, n,
                (long long)c->gctr_host[b].rec_count);
      return HPC_ERR_STATE;
    }
    pre[b + 1] = pre[b] + (c->recs ? n : 0);
    wpre[b + 1] = wpre[b] + (c->recs ? w : 0);
  }
  for (int b = 0; b <= c->count; ++b) inst_words[b] = wpre[b];
  const long long total = pre[c->count], words = wpre[c->count];
  if (!out || cap_words <= 0 || total == 0) return HPC_OK;
  if (c->rec_stage_words < words) {
    dev_free(c->rec_stage);
    c->rec_stage_words = 0;
    if ((s = dev_alloc(&c->rec_stage, words, "record staging")) != HPC_OK) return s;
    c->rec_stage_words = words;
  }
  // one segment per (instance, level) with removals: a contiguous run of records
  std::vector<RecSegment> segs;
  for (int b = 0; b < c->count; ++b) {
    long long src = 0, dst = wpre[b];
    for (int l = 1; l < kLevels && l < c->next_level; ++l) {
      const long long d = (long long)c->ctr_host[(size_t)b * kLevels + l].deleted;
      if (d == 0) continue;
      segs.push_back(RecSegment{src, d, dst, b, l});
      src += d;
      dst += d * (6 + ((l + 1) & ~1));
    }
  }
  if ((long long)segs.size() > c->rec_seg_cap) {
    dev_free(c->rec_seg);
    c->rec_seg = nullptr;
    c->rec_seg_cap = 0;
    if ((s = dev_alloc(&c->rec_seg, (int64_t)segs.size(), "record segments")) != HPC_OK) return s;
    c->rec_seg_cap = (long long)segs.size();
  }
  HPC_CUDA(cudaMemcpyAsync(c->rec_seg, segs.data(), sizeof(RecSegment) * segs.size(), cudaMemcpyHostToDevice,
                           c->stream));
  if ((s = launch_pack_records(c->inst, c->rec_seg, (int)segs.size(), c->rec_stage, c->stream)) != HPC_OK) return s;
  c->timings.launches += 1;
  HPC_CUDA(cudaMemcpyAsync(out, c->rec_stage, sizeof(int32_t) * (size_t)std::min<long long>(cap_words, words),
                           cudaMemcpyDeviceToHost, c->stream));
  HPC_CUDA(cudaStreamSynchronize(c->stream));
  return HPC_OK;
}

hpc_status hpc_batch_adjacency_words(hpc_ctx *c, int64_t *word_offsets) {
  if (!c || !word_offsets) {
    set_error("null argument");
    return HPC_ERR_INVALID_ARG;
  }
  for (int b = 0; b < c->count; ++b) word_offsets[b] = c->ih[b].adj_off;
  word_offsets[c->count] = c->total_words;
  return HPC_OK;
}

hpc_status hpc_batch_get_adjacency_bits(hpc_ctx *c, uint32_t *out, int64_t words) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if ((s = settle(c)) != HPC_OK) return s;
  if (!out || words < c->total_words) {
    set_error(!out ? "null output pointer" : "output holds %lld words, the adjacency needs %lld", (long long)words,
              (long long)c->total_words);
    return HPC_ERR_INVALID_ARG;
  }
  if (c->next_level == 0) {  // nothing run yet: the complete graph
    for (int b = 0; b < c->count; ++b) {
      const InstHost &h = c->ih[b];
      for (int64_t i = 0; i < h.p; ++i)
        for (int w = 0; w < h.W; ++w) {
          uint32_t v = 0;
          for (int q = 0; q < 32; ++q) {
            const int64_t j = (int64_t)w * 32 + q;
            if (j < h.p && j != i) v |= 1u << q;
          }
          out[h.adj_off + i * h.W + w] = v;
        }
    }
    return HPC_OK;
  }
  HPC_CUDA(cudaMemcpyAsync(out, c->adj, sizeof(uint32_t) * (size_t)c->total_words, cudaMemcpyDeviceToHost, c->stream));
  HPC_CUDA(cudaStreamSynchronize(c->stream));
  return HPC_OK;
}

hpc_status hpc_batch_get_all_sepset_records(hpc_ctx *c, hpc_sepset_record *out, int64_t cap, int64_t *prefix) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if ((s = settle(c)) != HPC_OK) return s;
  if (!prefix) {
    set_error("null prefix pointer");
    return HPC_ERR_INVALID_ARG;
  }
  if ((s = finalize_records(c)) != HPC_OK) return s;
  HPC_CUDA(cudaMemcpyAsync(c->gctr_host, c->gctr, sizeof(DevGlobal) * (size_t)c->count, cudaMemcpyDeviceToHost,
                           c->stream));
  HPC_CUDA(cudaStreamSynchronize(c->stream));
  std::vector<long long> pre((size_t)c->count + 1, 0);
  for (int b = 0; b < c->count; ++b) {
    const long long n = c->recs ? std::min<long long>((long long)c->gctr_host[b].rec_count, c->ih[b].rec_cap) : 0;
    pre[b + 1] = pre[b] + n;
  }
  for (int b = 0; b <= c->count; ++b) prefix[b] = pre[b];
  const long long total = pre[c->count];
  if (!out || cap <= 0 || total == 0) return HPC_OK;
  const int stride = rec_stride_words(c->rec_ids);
  if (c->rec_stage_words < total * stride) {
    dev_free(c->rec_stage);
    c->rec_stage_words = 0;
    if ((s = dev_alloc(&c->rec_stage, total * stride, "record staging")) != HPC_OK) return s;
    c->rec_stage_words = total * stride;
  }
  if (!c->rec_prefix_dev && (s = dev_alloc(&c->rec_prefix_dev, 2 * (c->count + 1), "record prefix")) != HPC_OK)
    return s;
  HPC_CUDA(cudaMemcpyAsync(c->rec_prefix_dev, pre.data(), sizeof(long long) * pre.size(), cudaMemcpyHostToDevice,
                           c->stream));
  if ((s = launch_gather_records(c->inst, c->count, c->rec_prefix_dev, total, stride, c->rec_stage, c->stream)) !=
      HPC_OK)
    return s;
  c->timings.launches += 1;
  const long long k = std::min<long long>(cap, total);
  std::vector<int32_t> raw((size_t)(k * stride));
  HPC_CUDA(cudaMemcpyAsync(raw.data(), c->rec_stage, sizeof(int32_t) * raw.size(), cudaMemcpyDeviceToHost, c->stream));
  HPC_CUDA(cudaStreamSynchronize(c->stream));
  for (long long r = 0; r < k; ++r) {
    const int32_t *rec = raw.data() + (size_t)r * stride;
    RecHead head;
    std::memcpy(&head, rec, sizeof(head));
    hpc_sepset_record &o = out[r];
    o.i = head.i;
    o.j = head.j;
    o.level = head.level;
    o.pad = 0;
    o.pmax = head.pmax;
    for (int q = 0; q < HPC_MAX_LEVEL; ++q) o.ids[q] = q < c->rec_ids ? rec[kRecHeadWords + q] : -1;
  }
  return HPC_OK;
}

hpc_status hpc_get_sepsets(hpc_ctx *c, int32_t *out, int max_cond) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if ((s = settle(c)) != HPC_OK) return s;
  if (!out || max_cond < 1) {
    set_error("null output or max_cond < 1");
    return HPC_ERR_INVALID_ARG;
  }
  const int64_t p = c->ih[0].p;
  std::fill(out, out + p * p * max_cond, -1);
  if (c->next_level == 0) return HPC_OK;
  std::vector<uint8_t> adj((size_t)(p * p));
  if ((s = hpc_get_adjacency(c, adj.data())) != HPC_OK) return s;
  int64_t nrec = 0;
  if ((s = hpc_get_sepset_records(c, nullptr, 0, &nrec)) != HPC_OK) return s;
  std::vector<hpc_sepset_record> recs((size_t)nrec);
  if (nrec && (s = hpc_get_sepset_records(c, recs.data(), nrec, &nrec)) != HPC_OK) return s;
  std::vector<uint8_t> later((size_t)(p * p), 0);
  for (const auto &r : recs) {
    later[(int64_t)r.i * p + r.j] = 1;
    for (int k = 0; k < std::min(r.level, max_cond); ++k) out[((int64_t)r.i * p + r.j) * max_cond + k] = r.ids[k];
  }
  for (int64_t i = 0; i < p; ++i)
    for (int64_t j = i + 1; j < p; ++j)
      if (!adj[i * p + j] && !later[i * p + j]) out[(i * p + j) * max_cond] = -2;
  return HPC_OK;
}

hpc_status hpc_debug_fail_allocation(int64_t k) {
  if (k < 0) return HPC_ERR_INVALID_ARG;
  g_fail_alloc_in.store(k);
  return HPC_OK;
}

int64_t hpc_debug_live_allocations(void) { return g_live_allocs.load(); }


hpc_status hpc_debug_set_retest_queue(hpc_ctx *c, int64_t entries) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if (entries < 1) {
    set_error("re-test queue of %lld entries", (long long)entries);
    return HPC_ERR_INVALID_ARG;
  }
  HPC_CUDA(cudaStreamSynchronize(c->stream));
  dev_free(c->rq);
  dev_free(c->rq_val);
  dev_free(c->rq_done);
  c->rq = nullptr;
  c->rq_val = nullptr;
  c->rq_done = nullptr;
  if ((s = alloc_rq(c, entries)) != HPC_OK) return s;
  c->set_off = false;
  return HPC_OK;
}

int hpc_debug_set_order_active(hpc_ctx *c) { return c && !c->set_off ? 1 : 0; }

hpc_status hpc_debug_set_order_from(int level) {
  if (level != 0 && (level < 2 || level > HPC_MAX_LEVEL)) {
    set_error("set order from level %d: 0 or 2..%d", level, HPC_MAX_LEVEL);
    return HPC_ERR_INVALID_ARG;
  }
  g_set_from.store(level);
  return HPC_OK;
}

hpc_status hpc_debug_set_barrier(hpc_ctx *c, int64_t wait_ns, int extra_arrivals) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if (wait_ns < 1000 || wait_ns > 10000000000ll || extra_arrivals < 0 || extra_arrivals > 1) {
    set_error("barrier wait needs 1 us <= wait_ns <= 10 s and extra_arrivals 0 or 1");
    return HPC_ERR_INVALID_ARG;
  }
  if ((s = settle(c)) != HPC_OK) return s;
  c->wait_ns = (unsigned long long)wait_ns;
  c->bar_extra = (unsigned int)extra_arrivals;
  ++c->inst_version;  // launch parameters: graphs are captured anew
  return HPC_OK;
}

double hpc_calc_pvalue(double r, int n) { return calc_pvalue64(r, n); }
double hpc_pval_l1(double x1, double x2, double x3, int n) { return pval_l1_64(x1, x2, x3, n); }
double hpc_pval_ln(const double *M, int k, int n) {
  if (!M || k < 2 || k > HPC_MAX_LEVEL + 2) return std::nan("");
  for (int i = 0; i < k * k; ++i)
    if (std::isnan(M[i])) return std::nan("");
  std::vector<double> a(M, M + k * k), v((size_t)(k * k));
  double p00, p01, p11;
  pinv_sym64_corner(a.data(), k, v.data(), &p00, &p01, &p11);
  return calc_pvalue64(-p01 / std::sqrt(p00 * p11), n);
}
double hpc_z_crit(double alpha) { return z_crit_of(alpha); }

}  // extern "C"

namespace hpc {
namespace {

hpc_status create(hpc_ctx **out, int count, const int64_t *p, const int64_t *n, const double *alpha,
                  const hpc_opts *opts) {
  if (!out) {
    set_error("null output pointer");
    return HPC_ERR_INVALID_ARG;
  }
  *out = nullptr;
  hpc_opts o;
  if (opts) o = *opts; else hpc_opts_default(&o);
  if (o.precision < HPC_PREC_FP64 || o.precision > HPC_PREC_MIXED_TC) {
    set_error("unknown precision %d", o.precision);
    return HPC_ERR_INVALID_ARG;
  }
  if (o.max_level > HPC_MAX_LEVEL) {
    set_error("max_level %d above HPC_MAX_LEVEL %d", o.max_level, HPC_MAX_LEVEL);
    return HPC_ERR_INVALID_ARG;
  }
  if (!(o.retest_margin >= 0.0)) o.retest_margin = 1e-3;
  for (int b = 0; b < count; ++b) {
    if (p[b] < 2 || p[b] > 46340) {
      set_error("instance %d: p = %lld out of range [2, 46340]", b, (long long)p[b]);
      return HPC_ERR_INVALID_ARG;
    }
    if (n[b] < 4 || n[b] > 0x7fffffff) {
      set_error("instance %d: n_obs = %lld out of range [4, 2^31)", b, (long long)n[b]);
      return HPC_ERR_INVALID_ARG;
    }
    const double a = alpha ? alpha[b] : o.alpha;
    if (!(a > 0.0 && a <= 1.0)) {
      set_error("instance %d: alpha = %g outside (0, 1]", b, a);
      return HPC_ERR_INVALID_ARG;
    }
  }
  int ndev = 0;
  const cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_error("no CUDA device available: %s", cudaGetErrorString(e));
    return HPC_ERR_NO_DEVICE;
  }
  if (o.device < 0 || o.device >= ndev) {
    set_error("device %d not present (%d devices)", o.device, ndev);
    return HPC_ERR_INVALID_ARG;
  }
  hpc_ctx *c = new hpc_ctx();
  c->count = count;
  c->opts = o;
  c->rec_ids = o.max_level < 0 ? HPC_MAX_LEVEL : std::min(std::max(o.max_level, 1), HPC_MAX_LEVEL);
  c->device = o.device;
  c->ih.resize((size_t)count);
  long long cor = 0, z = 0, adj = 0, rows = 0, tc = 0, words = 0, tiles = 0, nrows = 0;
  std::vector<long long> pre((size_t)(4 * (count + 1)), 0);
  long long segs = 0;
  for (int b = 0; b < count; ++b) {
    InstHost &h = c->ih[b];
    h.p = p[b];
    h.n = n[b];
    h.alpha = alpha ? alpha[b] : o.alpha;
    h.W = (int)((h.p + 31) / 32);
    h.zc = z_crit_of(h.alpha);
    h.r_crit = r_crit_of(h.alpha, (int)h.n);
    h.cor_off = cor;
    cor += h.p * h.p;
    h.z_off = z;
    z += h.n * h.p;
    h.adj_off = adj;
    adj += h.p * h.W;
    h.row_off = rows;
    rows += h.p + 1;
    h.tc_off = tc;
    tc += tc_p_pad(h.p) * tc_k(h.n);
    h.edges = h.p * (h.p - 1) / 2;
    pre[b] = words;
    words += h.p * h.W;
    pre[(count + 1) + b] = tiles;
    tiles += (long long)h.W * (h.W + 1) / 2;
    pre[2 * (count + 1) + b] = nrows;
    nrows += h.p;
    pre[3 * (count + 1) + b] = segs;
    segs += (h.p + kSegRows - 1) / kSegRows;
  }
  pre[count] = words;
  pre[(count + 1) + count] = tiles;
  pre[2 * (count + 1) + count] = nrows;
  pre[3 * (count + 1) + count] = segs;
  c->total_segs = segs;
  c->total_words = words;
  c->total_tiles = tiles;
  c->total_rows = nrows;
  c->p = c->ih[0].p;
  c->n = c->ih[0].n;
  {
    int64_t pmax = 0;
    for (const auto &h : c->ih) pmax = std::max<int64_t>(pmax, h.p);
    c->p_bucket = tune_bucket(pmax, kTunePB);
  }
  hpc_status s = HPC_OK;
  auto fail = [&](hpc_status st) {
    hpc_ctx_destroy(c);
    return st;
  };
  if (cudaSetDevice(c->device) != cudaSuccess) {
    cudaGetLastError();
    set_error("cudaSetDevice(%d) failed", c->device);
    delete c;
    return HPC_ERR_CUDA;
  }
  cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device);
  std::fill(std::begin(c->deg_seen), std::end(c->deg_seen), -1);
  bool ev_ok = true;
  for (auto &ev : c->evc) ev_ok = ev_ok && cudaEventCreate(&ev) == cudaSuccess;
  for (auto &ev : c->evr) ev_ok = ev_ok && cudaEventCreate(&ev) == cudaSuccess;
  for (auto &lv : c->evl)
    for (auto &ev : lv) ev_ok = ev_ok && cudaEventCreate(&ev) == cudaSuccess;
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess || !ev_ok) {
    cudaGetLastError();
    set_error("stream/event creation failed");
    return fail(HPC_ERR_CUDA);
  }
  c->stream = c->own_stream;
  // grids of the levels this context can run (up to its max_level): a context that stays
  // at low levels never loads the level-17..32 kernel, whose local-memory stack frame
  // (35 KB per thread) would otherwise be reserved for the whole device
  for (int l = 1; l <= c->rec_ids; ++l) c->citest_grid[l] = citest_grid(o.precision, l, c->device);
  if (o.precision != HPC_PREC_FP64)
    for (int l = 2; l <= std::min(c->rec_ids, kSetTop); ++l)
      c->citest_grid_set[l] = citest_grid(o.precision, l, c->device, kSetOrder);
  for (int v = 0; v < 3; ++v) c->citest_grid_l1[v] = citest_grid(o.precision, 1, c->device, v);
  if (o.precision != HPC_PREC_FP64)
    for (int v = 0; v < 2; ++v) c->citest_grid_l1q[v] = citest_grid(o.precision, 1, c->device, v | kQueueOnly);
  if (c->rec_ids > 16) retest_setup();  // the re-test kernel of levels 17-32
  if (o.precision != HPC_PREC_MIXED_TC && (s = dev_alloc(&c->cor64, cor, "cor64")) != HPC_OK) return fail(s);
  if (o.precision != HPC_PREC_FP64 && (s = dev_alloc(&c->cor32, cor, "cor32")) != HPC_OK) return fail(s);
  if ((s = dev_alloc(&c->adj, adj, "adjacency")) != HPC_OK) return fail(s);
  if ((s = dev_alloc(&c->deg, rows, "degrees")) != HPC_OK) return fail(s);
  if ((s = dev_alloc(&c->rowptr, rows, "row offsets")) != HPC_OK) return fail(s);
  if ((s = dev_alloc(&c->row_work, rows, "row work")) != HPC_OK) return fail(s);
  if ((s = dev_alloc(&c->row_dirty, rows, "stale-row marks")) != HPC_OK) return fail(s);
  if ((s = dev_alloc(&c->ctr, (int64_t)count * kLevels, "level counters")) != HPC_OK) return fail(s);
  if ((s = dev_alloc(&c->gctr, count, "counters")) != HPC_OK) return fail(s);
  if ((s = dev_alloc(&c->lc, kLevels, "launch counters")) != HPC_OK) return fail(s);
  if ((s = dev_alloc(&c->inst, count, "instance table")) != HPC_OK) return fail(s);
  if ((s = dev_alloc(&c->prefixes, (int64_t)pre.size(), "prefixes")) != HPC_OK) return fail(s);
  if ((s = dev_alloc(&c->work_prefix, (int64_t)kLevels * (count + 1), "work prefixes")) != HPC_OK) return fail(s);
  if ((s = dev_alloc(&c->seg, (int64_t)kLevels * segs, "segment sums")) != HPC_OK) return fail(s);
  c->ctr_host = new DevCounters[(size_t)count * kLevels];
  c->gctr_host = new DevGlobal[(size_t)count];
  if (cudaMemcpyAsync(c->prefixes, pre.data(), sizeof(long long) * pre.size(), cudaMemcpyHostToDevice, c->stream) !=
          cudaSuccess ||
      cudaMemsetAsync(c->ctr, 0, sizeof(DevCounters) * (size_t)count * kLevels, c->stream) != cudaSuccess ||
      cudaMemsetAsync(c->gctr, 0, sizeof(DevGlobal) * (size_t)count, c->stream) != cudaSuccess ||
      cudaMemsetAsync(c->lc, 0, sizeof(LaunchCounters) * kLevels, c->stream) != cudaSuccess) {
    cudaGetLastError();
    set_error("context initialisation failed");
    return fail(HPC_ERR_CUDA);
  }
  if ((s = write_inst_table(c)) != HPC_OK) return fail(s);
  *out = c;
  return HPC_OK;
}

}  // namespace
}  // namespace hpc
