// C ABI of libheterogpc: contexts, correlation entry points, the level loop and
// result retrieval. The reference equivalents are named beside each function in
// include/heterogpc.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
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

// z with erfc(z / sqrt 2) == alpha, by bisection in FP64 (host set-up only)
double z_crit_of(double alpha) {
  double lo = 0.0, hi = 40.0;
  for (int it = 0; it < 200; ++it) {
    double mid = 0.5 * (lo + hi);
    if (std::erfc(mid / 1.41421356237309504880) >= alpha) lo = mid; else hi = mid;
  }
  return 0.5 * (lo + hi);
}

// |r| with calc_pvalue64(r) == alpha (p is decreasing in |r|)
double r_crit_of(double alpha, int n) {
  double lo = 0.0, hi = kCutThr;
  if (calc_pvalue64(hi, n) >= alpha) return 2.0;  // every finite r is removed
  for (int it = 0; it < 200; ++it) {
    double mid = 0.5 * (lo + hi);
    if (calc_pvalue64(mid, n) >= alpha) lo = mid; else hi = mid;
  }
  return 0.5 * (lo + hi);
}

template <typename T>
hpc_status dev_alloc(T **ptr, int64_t count, const char *what) {
  if (count <= 0) count = 1;
  cudaError_t e = cudaMalloc((void **)ptr, sizeof(T) * (size_t)count);
  if (e != cudaSuccess) {
    *ptr = nullptr;
    cudaGetLastError();
    set_error("device allocation of %s (%lld bytes) failed: %s", what, (long long)(sizeof(T) * count),
              cudaGetErrorString(e));
    return HPC_ERR_OOM;
  }
  return HPC_OK;
}

template <typename T>
void dev_free(T *&ptr) {
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
}

// Absolute error bound of the tensor-core (split-BF16, FP32-accumulated) correlation
// entries used by the FP32 decision bands: the rounding of the low halves (2^-17
// relative per value) averages over the n samples, plus the FP32 accumulation;
// four times the model, which bounds the measured errors of tests/test_gpu_tensorcore.py.
double tc_entry_err(int64_t n) { return 4.0 * (1.6e-5 / std::sqrt((double)n) + 1e-7); }

LevelArgs make_args(hpc_ctx *c, int level) {
  LevelArgs a{};
  a.p = c->p;
  a.W = c->W;
  a.level = level;
  a.n_obs = (int)c->n;
  a.alpha = c->opts.alpha;
  a.sqrt_n3 = std::sqrt((double)c->n - 3.0);
  // FP32 decision: |r| against r_crit with a band of the configured relative |z|
  // margin (mapped to |r| through dz/dr = sqrt(n-3) / (1 - r^2)) plus an error bound
  // ke / (smallest pivot) from the rounding of the FP32 correlation entries and of
  // the factorisation
  const double rc = c->r_crit >= 1.5 ? 2.0 : c->r_crit;
  a.r_c = (float)rc;
  a.margin_r = rc >= 1.5 ? 0.f : (float)(c->opts.retest_margin * c->zc * (1.0 - rc * rc) / a.sqrt_n3);
  const double eps_in = c->cor32_rounded ? 1.2e-7 : tc_entry_err(c->n);
  a.ke = (float)((4.0 * eps_in + (level + 2) * 2.4e-7) * (1.0 + std::min(rc, 1.0)));
  a.cor64 = c->cor64_valid ? c->cor64 : nullptr;
  a.cor32 = c->cor32;
  a.Z = c->Z;
  a.n_z = c->n;
  a.denom = c->opts.ref_compat_sd ? (double)((float)c->n - 1.f) : (double)(c->n - 1);
  a.rq = c->rq;
  a.rq_cap = c->rq_cap;
  a.adj = c->adj;
  a.deg = c->deg;
  a.rowptr = c->rowptr;
  a.colidx = c->colidx;
  a.row_work = c->row_work;
  a.recs = c->recs;
  a.rec_cap = c->rec_cap;
  a.colidx_cap = c->colidx_cap;
  a.ctr = c->ctr + level;
  a.gctr = c->gctr;
  return a;
}

hpc_status check_ctx(hpc_ctx *c) {
  if (!c) {
    set_error("null context");
    return HPC_ERR_INVALID_ARG;
  }
  HPC_CUDA(cudaSetDevice(c->device));
  return HPC_OK;
}

hpc_status pull_counters(hpc_ctx *c) {
  HPC_CUDA(cudaMemcpyAsync(c->ctr_host, c->ctr, sizeof(DevCounters) * (HPC_MAX_LEVEL + 1), cudaMemcpyDeviceToHost,
                           c->stream));
  HPC_CUDA(cudaMemcpyAsync(c->gctr_host, c->gctr, sizeof(DevGlobal), cudaMemcpyDeviceToHost, c->stream));
  HPC_CUDA(cudaStreamSynchronize(c->stream));
  return HPC_OK;
}

// Queue all device work of one level on the context stream (no host sync).
// `timed` records the per-level events (not inside a graph capture: events
// recorded by graph nodes cannot be timed).
hpc_status enqueue_level(hpc_ctx *c, int level, bool timed) {
  hpc_status s;
  LevelArgs a = make_args(c, level);
  cudaEvent_t *ev = c->evl[level];
  if (timed) HPC_CUDA(cudaEventRecord(ev[0], c->stream));
  if (level == 0) {
    const double rc = c->r_crit;
    if (timed) HPC_CUDA(cudaEventRecord(ev[1], c->stream));
    if (c->cor64_valid) {
      const double r_lo = rc >= 1.5 ? 2.0 : rc * (1.0 - 1e-7), r_hi = rc >= 1.5 ? 2.0 : rc * (1.0 + 1e-7);
      if ((s = launch_level0(a, r_lo, r_hi, c->stream)) != HPC_OK) return s;
    } else {
      // FP32 tensor-core entries: band of the entry error bound, FP64 re-tests queued
      const double d0 = tc_entry_err(c->n) + 1e-6 * rc;
      const float lo = rc >= 1.5 ? 2.f : (float)(rc - d0), hi = rc >= 1.5 ? 2.f : (float)(rc + d0);
      HPC_CUDA(cudaMemsetAsync(&a.ctr->rq_count, 0, sizeof(unsigned long long), c->stream));
      if ((s = launch_level0_f32(a, lo, hi, c->stream)) != HPC_OK) return s;
      if ((s = launch_retest(a, c->sm_count, c->stream)) != HPC_OK) return s;
      if ((s = launch_mirror(a, c->stream)) != HPC_OK) return s;
      c->timings.launches += 1;
    }
    if (timed) HPC_CUDA(cudaEventRecord(ev[2], c->stream));
    if ((s = launch_degrees(a, c->deg, c->stream)) != HPC_OK) return s;
    if ((s = launch_scan(c->p, 0, c->deg, c->rowptr, c->row_work, a.ctr, c->gctr, c->stream)) != HPC_OK) return s;
    c->timings.launches += 4;
    return HPC_OK;
  }
  if ((s = launch_degrees(a, c->deg, c->stream)) != HPC_OK) return s;
  if ((s = launch_scan(c->p, level, c->deg, c->rowptr, c->row_work, a.ctr, c->gctr, c->stream)) != HPC_OK) return s;
  if ((s = launch_fill_csr(a, c->colidx, c->stream)) != HPC_OK) return s;
  if (timed) HPC_CUDA(cudaEventRecord(ev[1], c->stream));
  if ((s = launch_citest(a, c->opts.precision, c->citest_grid[level], c->stream)) != HPC_OK) return s;
  if (!c->cor64_valid) {
    if ((s = launch_retest(a, c->sm_count, c->stream)) != HPC_OK) return s;
    c->timings.launches += 1;
  }
  if (timed) HPC_CUDA(cudaEventRecord(ev[2], c->stream));
  c->timings.launches += 4;
  if (c->opts.precision != HPC_PREC_FP64) {
    if ((s = launch_finalize_records(a, c->stream)) != HPC_OK) return s;
    c->timings.launches += 1;
  }
  return HPC_OK;
}

// Neighbour-list and record buffers sized from the level-0 result (counters pulled).
hpc_status ensure_capacity(hpc_ctx *c, bool *changed) {
  const int64_t e2 = (int64_t)c->ctr_host[0].edges2;
  hpc_status s;
  *changed = false;
  if (e2 > c->colidx_cap) {
    dev_free(c->colidx);
    c->colidx_cap = 0;
    if ((s = dev_alloc(&c->colidx, std::max<int64_t>(1, e2), "neighbour lists")) != HPC_OK) return s;
    c->colidx_cap = std::max<int64_t>(1, e2);
    *changed = true;
  }
  if (e2 / 2 > c->rec_cap) {
    dev_free(c->recs);
    c->rec_cap = 0;
    if ((s = dev_alloc(&c->recs, std::max<int64_t>(1, e2 / 2), "separation-set records")) != HPC_OK) return s;
    c->rec_cap = std::max<int64_t>(1, e2 / 2);
    *changed = true;
  }
  return HPC_OK;
}

// Per-level statistics and timings from the pulled counters and events.
hpc_status collect_level(hpc_ctx *c, int level, hpc_level_stats *out) {
  const DevCounters &h = c->ctr_host[level];
  hpc_level_stats st{};
  st.level = level;
  st.edges_before = c->edges;
  st.max_degree = level == 0 ? (int)(c->p - 1) : h.max_deg;
  st.rows = level == 0 ? c->p : h.rows;
  if (level == 0) {
    st.potential_tests = st.executed_tests = c->p * (c->p - 1) / 2;
    st.edges_after = (int64_t)(h.edges2 / 2);
  } else {
    st.potential_tests = (int64_t)h.work_total;
    st.executed_tests = (int64_t)h.tests;
    st.retests = (int64_t)h.retests;
    st.edges_after = st.edges_before - (int64_t)h.deleted;
  }
  float t_all = 0.f, t_snap = 0.f, t_test = 0.f;
  if (!c->last_run_graph) {
    HPC_CUDA(cudaEventElapsedTime(&t_snap, c->evl[level][0], c->evl[level][1]));
    HPC_CUDA(cudaEventElapsedTime(&t_test, c->evl[level][1], c->evl[level][2]));
    HPC_CUDA(cudaEventElapsedTime(&t_all, c->evl[level][0], level < HPC_MAX_LEVEL && level + 1 < c->next_level
                                                                ? c->evl[level + 1][0] : c->evl[level][2]));
  }
  st.ms = t_all;
  c->timings.level_ms[level] = t_all;
  c->timings.compact_ms[level] = t_snap;
  c->timings.test_ms[level] = t_test;
  c->edges = st.edges_after;
  if (h.band_violations) {
    set_error("level %d: %llu FP32 removals not confirmed in FP64 (error bound violated)", level,
              (unsigned long long)h.band_violations);
    return HPC_ERR_NUMERIC;
  }
  if (c->opts.verbose)
    printf("level %d: max degree %d, tests %lld of %lld, FP64 re-tests %lld, edges %lld -> %lld, %.3f ms\n", level,
           st.max_degree, (long long)st.executed_tests, (long long)st.potential_tests, (long long)st.retests,
           (long long)st.edges_before, (long long)st.edges_after, st.ms);
  if (out) *out = st;
  return HPC_OK;
}

hpc_status global_errors(hpc_ctx *c) {
  const int err = c->gctr_host->err;
  if (err & kErrWorkOverflow) {
    set_error("the number of CI tests of a level overflows 64 bits");
    return HPC_ERR_CAPACITY;
  }
  if (err & kErrRecOverflow) {
    set_error("separation-set record buffer overflow");
    return HPC_ERR_CAPACITY;
  }
  return HPC_OK;
}

hpc_status after_correlation(hpc_ctx *c) {
  if (c->opts.precision == HPC_PREC_MIXED) {
    hpc_status s = launch_to_f32(c->cor64, c->p * c->p, c->cor32, c->stream);
    if (s != HPC_OK) return s;
    c->timings.launches += 1;
  }
  c->have_cor = true;
  c->cor32_rounded = c->opts.precision != HPC_PREC_MIXED_TC;
  return hpc_ctx_reset(c);
}

// A loaded FP64 matrix: every mixed mode tests on its FP32 rounding.
hpc_status after_loaded_correlation(hpc_ctx *c) {
  if (c->opts.precision != HPC_PREC_FP64) {
    hpc_status s = launch_to_f32(c->cor64, c->p * c->p, c->cor32, c->stream);
    if (s != HPC_OK) return s;
    c->timings.launches += 1;
  }
  c->have_cor = true;
  c->cor32_rounded = true;
  c->cor64_valid = true;
  return hpc_ctx_reset(c);
}

template <typename T>
hpc_status correlation_device(hpc_ctx *c, const T *X) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if (!X) {
    set_error("null observation pointer");
    return HPC_ERR_INVALID_ARG;
  }
  const int64_t elems = c->n * c->p;
  if (c->Z_elems < elems) {
    dev_free(c->Z);
    if ((s = dev_alloc(&c->Z, elems, "standardised data")) != HPC_OK) return s;
    c->Z_elems = elems;
  }
  HPC_CUDA(cudaEventRecord(c->evc[0], c->stream));
  const double denom = c->opts.ref_compat_sd ? (double)((float)c->n - 1.f) : (double)(c->n - 1);
  if (c->opts.precision == HPC_PREC_MIXED_TC) {
    // split-BF16 operands + FP64 standardised copy, tensor-core Gram into cor32
    const int64_t tc = tc_p_pad(c->p) * tc_k(c->n);
    if (c->tc_elems < tc) {
      dev_free(c->tcP);
      dev_free(c->tcQ);
      c->tc_elems = 0;
      if ((s = dev_alloc(&c->tcP, tc, "tensor-core operand P")) != HPC_OK) return s;
      if ((s = dev_alloc(&c->tcQ, tc, "tensor-core operand Q")) != HPC_OK) return s;
      HPC_CUDA(cudaMemsetAsync(c->tcP, 0, sizeof(__nv_bfloat16) * tc, c->stream));
      HPC_CUDA(cudaMemsetAsync(c->tcQ, 0, sizeof(__nv_bfloat16) * tc, c->stream));
      c->tc_elems = tc;
    }
    if (sizeof(T) == 8)
      s = launch_standardise_split_f64((const double *)X, c->n, c->p, c->opts.ref_compat_sd, c->Z, c->tcP, c->tcQ,
                                       c->stream);
    else
      s = launch_standardise_split_f32((const float *)X, c->n, c->p, c->opts.ref_compat_sd, c->Z, c->tcP, c->tcQ,
                                       c->stream);
    if (s != HPC_OK) return s;
    HPC_CUDA(cudaEventRecord(c->evc[1], c->stream));
    if ((s = launch_gram_tc(c->tcP, c->tcQ, c->n, c->p, c->cor32, &c->gctr->err, c->stream)) != HPC_OK) return s;
    HPC_CUDA(cudaEventRecord(c->evc[2], c->stream));
    // FP64 entries come from dot products of Z in the re-test kernels: no FP64 matrix
    if (!c->rq) {
      const int64_t cap = 1 << 20;
      if ((s = dev_alloc(&c->rq, cap, "re-test queue")) != HPC_OK) return s;
      c->rq_cap = cap;
    }
    c->cor64_valid = false;
    c->timings.launches += 2;
  } else {
    if (sizeof(T) == 8)
      s = launch_standardise_f64((const double *)X, c->n, c->p, c->opts.ref_compat_sd, c->Z, c->stream);
    else
      s = launch_standardise_f32((const float *)X, c->n, c->p, c->opts.ref_compat_sd, c->Z, c->stream);
    if (s != HPC_OK) return s;
    HPC_CUDA(cudaEventRecord(c->evc[1], c->stream));
    if ((s = launch_gram_f64(c->Z, c->n, c->p, denom, c->cor64, c->stream)) != HPC_OK) return s;
    HPC_CUDA(cudaEventRecord(c->evc[2], c->stream));
    c->cor64_valid = true;
    c->timings.launches += 2;
  }
  if ((s = after_correlation(c)) != HPC_OK) return s;
  HPC_CUDA(cudaEventRecord(c->evc[3], c->stream));
  c->cor_timed = true;
  return HPC_OK;
}

template <typename T>
hpc_status correlation_host(hpc_ctx *c, const T *X) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if (!X) {
    set_error("null observation pointer");
    return HPC_ERR_INVALID_ARG;
  }
  const int64_t bytes = c->n * c->p * (int64_t)sizeof(T);
  if (c->X_stage_bytes < bytes) {
    if (c->X_stage) cudaFree(c->X_stage);
    c->X_stage = nullptr;
    uint8_t *buf = nullptr;
    if ((s = dev_alloc(&buf, bytes, "observation staging")) != HPC_OK) return s;
    c->X_stage = buf;
    c->X_stage_bytes = bytes;
  }
  HPC_CUDA(cudaMemcpyAsync(c->X_stage, X, (size_t)bytes, cudaMemcpyHostToDevice, c->stream));
  return correlation_device(c, (const T *)c->X_stage);
}

}  // namespace
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
  o->alpha = 0.05;  // src/main.cpp:26
  o->max_level = 4; // src/main.cpp:31
  o->precision = HPC_PREC_MIXED;
  o->retest_margin = 1e-3;
  o->ref_compat_sd = 0;
  o->verbose = 0;
  return HPC_OK;
}

hpc_status hpc_ctx_footprint(int64_t p, int64_t n, const hpc_opts *o, int64_t *bytes) {
  if (!o || !bytes || p < 2 || n < 4) return HPC_ERR_INVALID_ARG;
  const int64_t W = (p + 31) / 32;
  int64_t b = p * p * 8;                                  // cor64
  if (o->precision != HPC_PREC_FP64) b += p * p * 4;      // cor32
  b += p * W * 4;                                         // adjacency bits
  b += (p + 1) * (4 + 4 + 8);                             // deg, rowptr, row_work
  b += n * p * 8;                                         // standardised data
  // neighbour lists and records are sized at level 1 from the surviving edges;
  // budget them for an average degree of 64
  const int64_t e = std::min<int64_t>(p * (p - 1) / 2, p * 32);
  b += 2 * e * 4 + e * (int64_t)sizeof(hpc_sepset_record);
  *bytes = b;
  return HPC_OK;
}

hpc_status hpc_ctx_create(hpc_ctx **out, int64_t p, int64_t n, const hpc_opts *opts) {
  if (!out) {
    set_error("null output pointer");
    return HPC_ERR_INVALID_ARG;
  }
  *out = nullptr;
  hpc_opts o;
  if (opts) o = *opts; else hpc_opts_default(&o);
  if (p < 2 || p > 46340) {
    set_error("p = %lld out of range [2, 46340]", (long long)p);
    return HPC_ERR_INVALID_ARG;
  }
  if (n < 4 || n > 0x7fffffff) {
    set_error("n_obs = %lld out of range [4, 2^31)", (long long)n);
    return HPC_ERR_INVALID_ARG;
  }
  if (!(o.alpha > 0.0 && o.alpha <= 1.0)) {
    set_error("alpha = %g outside (0, 1]", o.alpha);
    return HPC_ERR_INVALID_ARG;
  }
  if (o.precision < HPC_PREC_FP64 || o.precision > HPC_PREC_MIXED_TC) {
    set_error("unknown precision %d", o.precision);
    return HPC_ERR_INVALID_ARG;
  }
  if (o.max_level > HPC_MAX_LEVEL) {
    set_error("max_level %d above HPC_MAX_LEVEL %d", o.max_level, HPC_MAX_LEVEL);
    return HPC_ERR_INVALID_ARG;
  }
  if (!(o.retest_margin >= 0.0)) o.retest_margin = 1e-3;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
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
  c->p = p;
  c->n = n;
  c->opts = o;
  c->device = o.device;
  c->W = (int)((p + 31) / 32);
  c->zc = z_crit_of(o.alpha);
  c->r_crit = r_crit_of(o.alpha, (int)n);
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
  c->stream = nullptr;
  bool ev_ok = true;
  for (auto &e : c->evc) ev_ok = ev_ok && cudaEventCreate(&e) == cudaSuccess;
  for (auto &e : c->evr) ev_ok = ev_ok && cudaEventCreate(&e) == cudaSuccess;
  for (auto &lv : c->evl)
    for (auto &e : lv) ev_ok = ev_ok && cudaEventCreate(&e) == cudaSuccess;
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess || !ev_ok) {
    cudaGetLastError();
    set_error("stream/event creation failed");
    return fail(HPC_ERR_CUDA);
  }
  c->stream = c->own_stream;
  for (int l = 1; l <= HPC_MAX_LEVEL; ++l) c->citest_grid[l] = citest_grid(o.precision, l, c->device);
  if (o.precision != HPC_PREC_MIXED_TC && (s = dev_alloc(&c->cor64, p * p, "cor64")) != HPC_OK) return fail(s);
  if (o.precision != HPC_PREC_FP64 && (s = dev_alloc(&c->cor32, p * p, "cor32")) != HPC_OK) return fail(s);
  if ((s = dev_alloc(&c->adj, p * (int64_t)c->W, "adjacency")) != HPC_OK) return fail(s);
  if ((s = dev_alloc(&c->deg, p, "degrees")) != HPC_OK) return fail(s);
  if ((s = dev_alloc(&c->rowptr, p + 1, "row offsets")) != HPC_OK) return fail(s);
  if ((s = dev_alloc(&c->row_work, p + 1, "row work")) != HPC_OK) return fail(s);
  if ((s = dev_alloc(&c->ctr, HPC_MAX_LEVEL + 1, "level counters")) != HPC_OK) return fail(s);
  if ((s = dev_alloc(&c->gctr, 1, "counters")) != HPC_OK) return fail(s);
  if (cudaMallocHost((void **)&c->ctr_host, sizeof(DevCounters) * (HPC_MAX_LEVEL + 1)) != cudaSuccess ||
      cudaMallocHost((void **)&c->gctr_host, sizeof(DevGlobal)) != cudaSuccess) {
    cudaGetLastError();
    set_error("pinned counter allocation failed");
    return fail(HPC_ERR_OOM);
  }
  if (cudaMemsetAsync(c->ctr, 0, sizeof(DevCounters) * (HPC_MAX_LEVEL + 1), c->stream) != cudaSuccess ||
      cudaMemsetAsync(c->gctr, 0, sizeof(DevGlobal), c->stream) != cudaSuccess)
    return fail(HPC_ERR_CUDA);
  *out = c;
  return HPC_OK;
}

hpc_status hpc_ctx_destroy(hpc_ctx *c) {
  if (!c) return HPC_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  dev_free(c->cor64);
  dev_free(c->cor32);
  dev_free(c->Z);
  dev_free(c->tcP);
  dev_free(c->tcQ);
  if (c->X_stage) cudaFree(c->X_stage);
  dev_free(c->adj);
  dev_free(c->adj_bytes);
  dev_free(c->rq);
  dev_free(c->deg);
  dev_free(c->rowptr);
  dev_free(c->colidx);
  dev_free(c->row_work);
  dev_free(c->recs);
  dev_free(c->ctr);
  dev_free(c->gctr);
  if (c->ctr_host) cudaFreeHost(c->ctr_host);
  if (c->gctr_host) cudaFreeHost(c->gctr_host);
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

hpc_status hpc_ctx_reset(hpc_ctx *c) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  HPC_CUDA(cudaMemsetAsync(c->ctr, 0, sizeof(DevCounters) * (HPC_MAX_LEVEL + 1), c->stream));
  HPC_CUDA(cudaMemsetAsync(c->gctr, 0, sizeof(DevGlobal), c->stream));
  c->next_level = 0;
  c->edges = c->p * (c->p - 1) / 2;
  return HPC_OK;
}

hpc_status hpc_correlation_f64(hpc_ctx *c, const double *X) { return correlation_host(c, X); }
hpc_status hpc_correlation_f32(hpc_ctx *c, const float *X) { return correlation_host(c, X); }
hpc_status hpc_correlation_device_f64(hpc_ctx *c, const double *X) { return correlation_device(c, X); }
hpc_status hpc_correlation_device_f32(hpc_ctx *c, const float *X) { return correlation_device(c, X); }

hpc_status hpc_load_correlation(hpc_ctx *c, const double *C) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if (!C) {
    set_error("null correlation pointer");
    return HPC_ERR_INVALID_ARG;
  }
  if (!c->cor64 && (s = dev_alloc(&c->cor64, c->p * c->p, "cor64")) != HPC_OK) return s;
  HPC_CUDA(cudaMemcpyAsync(c->cor64, C, sizeof(double) * (size_t)(c->p * c->p), cudaMemcpyHostToDevice, c->stream));
  return after_loaded_correlation(c);
}

hpc_status hpc_load_correlation_device(hpc_ctx *c, const double *C) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if (!C) {
    set_error("null correlation pointer");
    return HPC_ERR_INVALID_ARG;
  }
  if (!c->cor64 && (s = dev_alloc(&c->cor64, c->p * c->p, "cor64")) != HPC_OK) return s;
  HPC_CUDA(cudaMemcpyAsync(c->cor64, C, sizeof(double) * (size_t)(c->p * c->p), cudaMemcpyDeviceToDevice, c->stream));
  return after_loaded_correlation(c);
}

hpc_status hpc_get_correlation(hpc_ctx *c, double *C) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if (!C || !c->have_cor) {
    set_error(!C ? "null output pointer" : "no correlation matrix yet");
    return !C ? HPC_ERR_INVALID_ARG : HPC_ERR_STATE;
  }
  if (!c->cor64_valid) {
    // tensor-core mode keeps no FP64 matrix: form it from the standardised data
    if (!c->cor64 && (s = dev_alloc(&c->cor64, c->p * c->p, "cor64")) != HPC_OK) return s;
    const double denom = c->opts.ref_compat_sd ? (double)((float)c->n - 1.f) : (double)(c->n - 1);
    if ((s = launch_gram_f64(c->Z, c->n, c->p, denom, c->cor64, c->stream)) != HPC_OK) return s;
    c->cor64_valid = true;
  }
  HPC_CUDA(cudaMemcpyAsync(C, c->cor64, sizeof(double) * (size_t)(c->p * c->p), cudaMemcpyDeviceToHost, c->stream));
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
  HPC_CUDA(cudaMemcpyAsync(C, c->cor32, sizeof(float) * (size_t)(c->p * c->p), cudaMemcpyDeviceToHost, c->stream));
  HPC_CUDA(cudaStreamSynchronize(c->stream));
  return HPC_OK;
}

hpc_status hpc_run_level(hpc_ctx *c, int level, hpc_level_stats *st) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
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
  if (level == 1) {
    bool changed = false;
    if ((s = ensure_capacity(c, &changed)) != HPC_OK) return s;
  }
  if ((s = enqueue_level(c, level, true)) != HPC_OK) return s;
  c->last_run_graph = false;
  if ((s = pull_counters(c)) != HPC_OK) return s;
  if ((s = global_errors(c)) != HPC_OK) return s;
  c->next_level = level + 1;
  return collect_level(c, level, st);
}

namespace {
bool capturable(cudaStream_t s) {
  return s != nullptr && s != cudaStreamLegacy && s != cudaStreamPerThread;
}

// Run levels first..last (already validated) with one host sync at the end; the
// whole sequence 0..last is captured once into a CUDA graph and replayed.
hpc_status run_levels(hpc_ctx *c, int first, int last, bool use_graph) {
  hpc_status s;
  if (use_graph && c->graphs_enabled && first == 0 && capturable(c->stream)) {
    const bool valid = c->graph && c->graph_top == last && c->graph_stream == c->stream &&
                       c->graph_cor64_valid == c->cor64_valid &&
                       c->graph_colidx_cap == c->colidx_cap && c->graph_rec_cap == c->rec_cap;
    if (!valid) {
      if (c->graph) cudaGraphExecDestroy(c->graph);
      c->graph = nullptr;
      cudaGraph_t g = nullptr;
      HPC_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      const int64_t launches = c->timings.launches;
      for (int l = first; l <= last; ++l) {
        if ((s = enqueue_level(c, l, false)) != HPC_OK) {
          cudaStreamEndCapture(c->stream, &g);
          if (g) cudaGraphDestroy(g);
          return s;
        }
      }
      c->timings.launches = launches;  // counted when the graph runs
      HPC_CUDA(cudaStreamEndCapture(c->stream, &g));
      cudaError_t e = cudaGraphInstantiate(&c->graph, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) {
        c->graph = nullptr;
        return cuda_fail(e, "cudaGraphInstantiate", __FILE__, __LINE__);
      }
      c->graph_top = last;
      c->graph_stream = c->stream;
      c->graph_cor64_valid = c->cor64_valid;
      c->graph_colidx_cap = c->colidx_cap;
      c->graph_rec_cap = c->rec_cap;
      // launches of one replay
      c->graph_launches = 0;
      for (int l = first; l <= last; ++l) c->graph_launches += l == 0 ? 4 : (c->opts.precision != HPC_PREC_FP64 ? 5 : 4);
    }
    HPC_CUDA(cudaGraphLaunch(c->graph, c->stream));
    c->timings.launches += c->graph_launches;
    c->last_run_graph = true;
  } else {
    for (int l = first; l <= last; ++l)
      if ((s = enqueue_level(c, l, true)) != HPC_OK) return s;
    c->last_run_graph = false;
  }
  return pull_counters(c);
}
}  // namespace

hpc_status hpc_run_skeleton(hpc_ctx *c, hpc_level_stats *stats, int cap, int *levels_run) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if (!c->have_cor) {
    set_error("run before a correlation matrix was computed or loaded");
    return HPC_ERR_STATE;
  }
  const int top = c->opts.max_level < 0 ? HPC_MAX_LEVEL : c->opts.max_level;
  int ran = 0;
  auto emit = [&](int l) -> hpc_status {
    hpc_level_stats st{};
    hpc_status e = collect_level(c, l, &st);
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
      if (l >= 1 && c->ctr_host[l].work_total == 0) break;
    }
    if (levels_run) *levels_run = ran;
    return HPC_OK;
  }
  // A known max level runs as one sequence (one graph replay, one sync); "until
  // exhausted" runs in chunks of four levels with a check in between.
  const bool known = c->opts.max_level >= 0;
  const int chunk = known ? top + 1 : 4;
  const int64_t edges0 = c->edges;
  HPC_CUDA(cudaEventRecord(c->evr[0], c->stream));
  for (int attempt = 0; attempt < 2; ++attempt) {
    ran = 0;
    c->edges = edges0;
    bool sized = c->colidx_cap > 0 && c->rec_cap > 0;
    int first = 0;
    if (!sized) {
      // first run: level 0 alone sizes the neighbour-list and record buffers
      if ((s = run_levels(c, 0, 0, false)) != HPC_OK) return s;
      bool changed;
      if ((s = ensure_capacity(c, &changed)) != HPC_OK) return s;
      first = 1;
    }
    bool overflow = false, done = false;
    int last_run = first - 1;
    while (!done && first <= top) {
      const int last = std::min(top, first + chunk - 1);
      if ((s = run_levels(c, first, last, known)) != HPC_OK) return s;
      last_run = last;
      if (c->gctr_host->err & kErrCsrOverflow) {
        overflow = true;
        break;
      }
      if ((s = global_errors(c)) != HPC_OK) return s;
      done = last >= 1 && c->ctr_host[last].work_total == 0;
      first = last + 1;
    }
    if (overflow) {
      // the data changed since the buffers were sized: resize from level 0 and rerun
      bool changed;
      if ((s = ensure_capacity(c, &changed)) != HPC_OK) return s;
      if ((s = hpc_ctx_reset(c)) != HPC_OK) return s;
      continue;
    }
    c->next_level = last_run + 1;
    HPC_CUDA(cudaEventRecord(c->evr[1], c->stream));
    HPC_CUDA(cudaEventSynchronize(c->evr[1]));
    float tr = 0.f;
    HPC_CUDA(cudaEventElapsedTime(&tr, c->evr[0], c->evr[1]));
    c->timings.skeleton_ms = tr;
    // a first run sized its buffers with level 0 alone: the events of that part
    // are of the eager kind, the rest may be a graph replay
    for (int l = 0; l <= last_run; ++l) {
      if ((s = emit(l)) != HPC_OK) return s;
      if (l >= 1 && c->ctr_host[l].work_total == 0) break;
    }
    if (levels_run) *levels_run = ran;
    return HPC_OK;
  }
  set_error("neighbour-list buffer still too small after resizing");
  return HPC_ERR_CAPACITY;
}

hpc_status hpc_get_adjacency(hpc_ctx *c, uint8_t *out) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if (!out) {
    set_error("null output pointer");
    return HPC_ERR_INVALID_ARG;
  }
  if (c->next_level == 0) {
    for (int64_t i = 0; i < c->p; ++i)
      for (int64_t j = 0; j < c->p; ++j) out[i * c->p + j] = (uint8_t)(i != j);
    return HPC_OK;
  }
  if (!c->adj_bytes && (s = dev_alloc(&c->adj_bytes, c->p * c->p, "adjacency bytes")) != HPC_OK) return s;
  if ((s = launch_expand_adjacency(c->adj, c->p, c->W, c->adj_bytes, c->stream)) != HPC_OK) return s;
  c->timings.launches += 1;
  HPC_CUDA(cudaMemcpyAsync(out, c->adj_bytes, (size_t)(c->p * c->p), cudaMemcpyDeviceToHost, c->stream));
  HPC_CUDA(cudaStreamSynchronize(c->stream));
  return HPC_OK;
}

hpc_status hpc_edge_count(hpc_ctx *c, int64_t *edges) {
  if (!c || !edges) {
    set_error("null argument");
    return HPC_ERR_INVALID_ARG;
  }
  *edges = c->edges;
  return HPC_OK;
}

hpc_status hpc_get_sepset_records(hpc_ctx *c, hpc_sepset_record *out, int64_t cap, int64_t *count) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if (!count) {
    set_error("null count pointer");
    return HPC_ERR_INVALID_ARG;
  }
  unsigned long long n = 0;
  HPC_CUDA(cudaMemcpyAsync(&n, &c->gctr->rec_count, sizeof(n), cudaMemcpyDeviceToHost, c->stream));
  HPC_CUDA(cudaStreamSynchronize(c->stream));
  n = std::min<unsigned long long>(n, (unsigned long long)std::max<int64_t>(c->rec_cap, 0));
  *count = (int64_t)n;
  if (out && cap > 0 && n > 0) {
    const int64_t k = std::min<int64_t>(cap, (int64_t)n);
    HPC_CUDA(cudaMemcpyAsync(out, c->recs, sizeof(hpc_sepset_record) * (size_t)k, cudaMemcpyDeviceToHost, c->stream));
    HPC_CUDA(cudaStreamSynchronize(c->stream));
  }
  return HPC_OK;
}

hpc_status hpc_get_sepsets(hpc_ctx *c, int32_t *out, int max_cond) {
  hpc_status s = check_ctx(c);
  if (s != HPC_OK) return s;
  if (!out || max_cond < 1) {
    set_error("null output or max_cond < 1");
    return HPC_ERR_INVALID_ARG;
  }
  const int64_t p = c->p;
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
