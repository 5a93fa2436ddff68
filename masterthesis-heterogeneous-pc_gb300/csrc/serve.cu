// Skeleton serving with continuous batching (no reference counterpart: the reference
// answers one problem per process run, its level loop being
// src/independence/skeleton.cpp:152-190).
//
// One engine thread owns the device work. Each admitted request is an instance with
// its own device state (a single-instance context: correlation, adjacency bitmask,
// neighbour lists, records, counters) whose correlation is computed at admission. The
// engine then runs steps: in a step, the requests that stand at the same level share
// one launch of that level's kernels -- the kernels already run over a table of
// instances (rebuild, test-count scan and CI tests of every instance in one cooperative
// launch) -- and requests at different levels run as consecutive launches of the same
// step. After a step (one host sync) each request moves to its next level or
// completes; requests that arrived meanwhile are admitted, as device memory allows, and
// join at level 0 in the next step while the others continue. So a request never
// waits for a batch to drain: it joins the running launches at the next level
// boundary, and a batch no longer finishes with its slowest request.
//
// Admission: in arrival order while the device bytes of the admitted requests (the
// context footprint without the re-test queue, which the engine shares) stay within
// budget_bytes and fewer than max_batch requests are active; at most max_inflight
// requests are admitted between two steps, so that running requests keep advancing.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "internal.cuh"

namespace {

using clk = std::chrono::steady_clock;
using namespace hpc;

constexpr int kLevels = HPC_MAX_LEVEL + 1;

struct Request {
  int64_t id = 0;
  const float *X = nullptr;
  int64_t p = 0, n = 0;
  double alpha = 0.05;
  uint8_t *adj_out = nullptr;
  int64_t bytes = 0;
  clk::time_point t_submit, t_start, t_done;
  hpc_status status = HPC_OK;
  int levels = 0;
  int64_t edges = 0;
  int batch_size = 0;   // most requests in one of its level launches
  int joined = 0;       // requests already running when it was admitted
  // engine state
  hpc_ctx *ctx = nullptr;
  int next = 0;         // next level to run
};

// counters of one request's level, gathered after a step
struct StepCounters {
  DevCounters c;
  DevGlobal g;
};

__global__ void gather_counters_kernel(const Inst *__restrict__ inst, const int *__restrict__ level, int count,
                                       StepCounters *__restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < count) {
    out[t].c = inst[t].ctr[level[t]];
    out[t].g = *inst[t].g;
  }
}

template <typename T>
hpc_status grow(T **ptr, long long *cap, long long need, cudaStream_t st) {
  if (*cap >= need) return HPC_OK;
  if (*ptr) cudaFreeAsync(*ptr, st);
  *ptr = nullptr;
  *cap = 0;
  const long long n = std::max<long long>(need, 16);
  const cudaError_t e = cudaMallocAsync((void **)ptr, sizeof(T) * (size_t)n, st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error("server scratch allocation failed: %s", cudaGetErrorString(e));
    return HPC_ERR_OOM;
  }
  *cap = n;
  return HPC_OK;
}

}  // namespace

struct hpc_server {
  hpc_server_opts opts{};
  std::mutex mu;
  std::condition_variable cv;        // engine wake-up
  std::condition_variable cv_done;   // drain
  std::deque<Request *> pending;
  std::vector<Request *> done;
  int64_t next_id = 0;
  int64_t outstanding = 0;           // submitted, not yet completed
  bool stop = false;
  std::thread engine;
  // engine-owned (engine thread only)
  cudaStream_t st = nullptr;
  int sms = 0;
  std::vector<Request *> active;
  int64_t active_bytes = 0;
  float *stage = nullptr;            // observations of the request being admitted
  long long stage_cap = 0;
  Inst *d_inst = nullptr;            // the step's instance tables, one slice per level group
  long long d_inst_cap = 0;
  long long *d_pre = nullptr;        // per group: word, tile, row, segment prefixes
  long long d_pre_cap = 0;
  unsigned long long *d_work = nullptr;
  long long d_work_cap = 0;
  LaunchCounters *d_lc = nullptr;
  long long d_lc_cap = 0;
  SegAgg *d_seg = nullptr;
  long long d_seg_cap = 0;
  RetestItem *d_rq = nullptr;
  long long rq_cap = 0;
  double *d_rqv = nullptr;         // the re-tests' entry scratch and done counters
  long long rqv_cap = 0;
  unsigned int *d_rqd = nullptr;
  long long rqd_cap = 0;
  int *d_levels = nullptr;
  long long d_levels_cap = 0;
  StepCounters *d_out = nullptr;
  long long d_out_cap = 0;
  TuneEntry *d_tune = nullptr;
  long long d_tune_cap = 0;
  long long tune_version = -1;
  int grid[kLevels] = {};
  int grid_set[kLevels] = {};  // set-order kernels (levels 2-16)
  int grid_l1 = 0;
};

namespace {

// A request whose context exists: queue its observations' upload and correlation.
hpc_status admit(hpc_server *sv, Request *r) {
  hpc_opts o;
  hpc_opts_default(&o);
  o.device = sv->opts.device;
  o.precision = sv->opts.precision;
  o.max_level = sv->opts.max_level;
  o.alpha = r->alpha;
  hpc_status s = hpc_ctx_create(&r->ctx, r->p, r->n, &o);
  if (s != HPC_OK) return s;
  if ((s = hpc_ctx_set_stream(r->ctx, sv->st)) != HPC_OK) return s;
  if ((s = grow(&sv->stage, &sv->stage_cap, r->p * r->n, sv->st)) != HPC_OK) return s;
  HPC_CUDA(cudaMemcpyAsync(sv->stage, r->X, sizeof(float) * (size_t)(r->p * r->n), cudaMemcpyHostToDevice, sv->st));
  if ((s = hpc_correlation_device_f32(r->ctx, sv->stage)) != HPC_OK) return s;
  r->next = 0;
  return HPC_OK;
}

hpc_status sync_tune_table(hpc_server *sv) {
  if (sv->d_tune && sv->tune_version == tune_version()) return HPC_OK;
  std::vector<TuneEntry> t;
  long long v = 0;
  tune_snapshot(&t, &v);
  hpc_status s;
  if ((s = grow(&sv->d_tune, &sv->d_tune_cap, (long long)t.size(), sv->st)) != HPC_OK) return s;
  HPC_CUDA(cudaMemcpyAsync(sv->d_tune, t.data(), sizeof(TuneEntry) * t.size(), cudaMemcpyHostToDevice, sv->st));
  HPC_CUDA(cudaStreamSynchronize(sv->st));  // t is released on return
  sv->tune_version = v;
  return HPC_OK;
}

// One step: the active requests grouped by their next level, one launch sequence per
// group, then every request's counters of the level it ran in one copy.
hpc_status step(hpc_server *sv) {
  std::vector<Request *> &act = sv->active;
  const int A = (int)act.size();
  std::vector<int> order(A);
  for (int q = 0; q < A; ++q) order[q] = q;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return act[a]->next < act[b]->next; });
  std::vector<Inst> tab(A);
  std::vector<long long> pre;      // per group: 4 x (G + 1)
  std::vector<int> lv(A);
  struct Group {
    int level, first, count;
    long long pre_off, seg_off, words, tiles, rows, segs;
    int64_t pmax;
    int prev_deg;  // largest degree at the previous level's start over the group (the set-order choice)
  };
  std::vector<Group> groups;
  long long segs_all = 0;
  for (int q = 0; q < A;) {
    const int l = act[order[q]]->next;
    int e = q;
    while (e < A && act[order[e]]->next == l) ++e;
    Group g{l, q, e - q, (long long)pre.size(), segs_all, 0, 0, 0, 0, 0, 0};
    pre.resize(pre.size() + 4 * (size_t)(g.count + 1));
    long long *wp = pre.data() + g.pre_off, *tp = wp + (g.count + 1), *rp = tp + (g.count + 1),
              *sp = rp + (g.count + 1);
    for (int k = 0; k < g.count; ++k) {
      Request *r = act[order[q + k]];
      tab[q + k] = r->ctx->inst_host[0];
      lv[q + k] = l;
      const InstHost &h = r->ctx->ih[0];
      wp[k] = g.words;
      tp[k] = g.tiles;
      rp[k] = g.rows;
      sp[k] = g.segs;
      g.words += h.p * h.W;
      g.tiles += (long long)h.W * (h.W + 1) / 2;
      g.rows += h.p;
      g.segs += (h.p + kSegRows - 1) / kSegRows;
      g.pmax = std::max<int64_t>(g.pmax, h.p);
      g.prev_deg = std::max(g.prev_deg, l >= 2 ? r->ctx->ctr_host[l - 1].max_deg : 0);
      r->batch_size = std::max(r->batch_size, g.count);
    }
    wp[g.count] = g.words;
    tp[g.count] = g.tiles;
    rp[g.count] = g.rows;
    sp[g.count] = g.segs;
    segs_all += g.segs;
    groups.push_back(g);
    q = e;
  }
  const int G = (int)groups.size();
  hpc_status s;
  if ((s = sync_tune_table(sv)) != HPC_OK) return s;
  if ((s = grow(&sv->d_inst, &sv->d_inst_cap, A, sv->st)) != HPC_OK) return s;
  if ((s = grow(&sv->d_pre, &sv->d_pre_cap, (long long)pre.size(), sv->st)) != HPC_OK) return s;
  if ((s = grow(&sv->d_work, &sv->d_work_cap, A + G, sv->st)) != HPC_OK) return s;
  if ((s = grow(&sv->d_lc, &sv->d_lc_cap, G, sv->st)) != HPC_OK) return s;
  if ((s = grow(&sv->d_seg, &sv->d_seg_cap, std::max<long long>(segs_all, 1), sv->st)) != HPC_OK) return s;
  if ((s = grow(&sv->d_levels, &sv->d_levels_cap, A, sv->st)) != HPC_OK) return s;
  if ((s = grow(&sv->d_out, &sv->d_out_cap, A, sv->st)) != HPC_OK) return s;
  HPC_CUDA(cudaMemcpyAsync(sv->d_inst, tab.data(), sizeof(Inst) * (size_t)A, cudaMemcpyHostToDevice, sv->st));
  HPC_CUDA(cudaMemcpyAsync(sv->d_pre, pre.data(), sizeof(long long) * pre.size(), cudaMemcpyHostToDevice, sv->st));
  HPC_CUDA(cudaMemcpyAsync(sv->d_levels, lv.data(), sizeof(int) * (size_t)A, cudaMemcpyHostToDevice, sv->st));
  HPC_CUDA(cudaMemsetAsync(sv->d_lc, 0, sizeof(LaunchCounters) * (size_t)G, sv->st));
  HPC_CUDA(cudaMemsetAsync(sv->d_seg, 0, sizeof(SegAgg) * (size_t)std::max<long long>(segs_all, 1), sv->st));
  const bool tc = sv->opts.precision == HPC_PREC_MIXED_TC;
  for (int gi = 0; gi < G; ++gi) {
    const Group &g = groups[gi];
    Launch L{};
    L.inst = sv->d_inst + g.first;
    L.count = g.count;
    L.level = g.level;
    L.word_prefix = sv->d_pre + g.pre_off;
    L.tile_prefix = L.word_prefix + (g.count + 1);
    L.row_prefix = L.tile_prefix + (g.count + 1);
    L.seg_prefix = L.row_prefix + (g.count + 1);
    L.work_prefix = sv->d_work + g.first + gi;
    L.lc = sv->d_lc + gi;
    L.rq = sv->d_rq;
    L.rq_cap = sv->rq_cap;
    L.rq_val = sv->d_rqv;
    L.rq_done = sv->d_rqd;
    L.rq_vcap = sv->rqv_cap;
    L.seg = sv->d_seg + g.seg_off;
    L.row_cache = g.count == 1 && g.pmax + 1 <= kRowCache;
    L.total_rows = g.rows;
    L.total_segs = g.segs;
    L.tune = sv->d_tune;
    L.force = TuneEntry{0, 0, 0, 0};
    L.p_bucket = tune_bucket(g.pmax, kTunePB);
    L.row_work_limit =
        std::min<unsigned long long>(1ull << 56, 0x7FFFFFFFFFFFFFFFull / (unsigned long long)std::max(1ll, g.rows));
    L.inst0 = tab[g.first];
    L.wait_ns = 2000000000ull;
    L.bar_extra = 0;
    if (g.level == 0) {
      if ((s = launch_level0(L, g.tiles, sv->st)) != HPC_OK) return s;
      if (tc && (s = launch_retest(L, sv->sms, sv->st)) != HPC_OK) return s;
      if ((s = launch_degrees(L, g.rows, sv->st)) != HPC_OK) return s;
      if ((s = launch_scan(L, sv->st)) != HPC_OK) return s;
    } else {
      const bool set = tc && uses_set_order(set_order_from(), g.level) && g.prev_deg <= kSetDegMax;
      const int grid = g.level == 1 ? sv->grid_l1 : set ? sv->grid_set[g.level] : sv->grid[g.level];
      if ((s = launch_level(L, sv->opts.precision, grid, set ? kSetOrder : kL1Interleaved, sv->st)) != HPC_OK)
        return s;
      if (tc && (s = launch_retest(L, sv->sms, sv->st)) != HPC_OK) return s;
    }
  }
  // the counters of every request's level, in the step's order
  gather_counters_kernel<<<(A + 127) / 128, 128, 0, sv->st>>>(sv->d_inst, sv->d_levels, A, sv->d_out);
  HPC_LAUNCH_CHECK("gather_counters_kernel");
  std::vector<StepCounters> out((size_t)A);
  HPC_CUDA(cudaMemcpyAsync(out.data(), sv->d_out, sizeof(StepCounters) * (size_t)A, cudaMemcpyDeviceToHost, sv->st));
  HPC_CUDA(cudaStreamSynchronize(sv->st));
  for (int q = 0; q < A; ++q) {
    Request *r = act[order[q]];
    const int l = lv[q];
    r->ctx->ctr_host[l] = out[q].c;
    r->ctx->gctr_host[0] = out[q].g;
  }
  return HPC_OK;
}

// A request after the level it just ran: its next level, or completion (true).
bool advance(hpc_server *sv, Request *r) {
  hpc_ctx *c = r->ctx;
  const int l = r->next;
  const DevCounters &C = c->ctr_host[l];
  const int err = c->gctr_host[0].err;
  if (err & (kErrTimeout | kErrRecOverflow | kErrWorkOverflow | kErrCsrOverflow | kErrRetestOverflow)) {
    r->status = (err & kErrTimeout) ? HPC_ERR_TIMEOUT : HPC_ERR_CAPACITY;
    return true;
  }
  c->next_level = l + 1;
  r->levels = l + 1;
  r->edges = l == 0 ? (int64_t)(C.edges2 / 2) : (int64_t)(C.edges2 / 2) - (int64_t)C.deleted;
  c->ih[0].edges = r->edges;
  const int top = sv->opts.max_level < 0 ? HPC_MAX_LEVEL : sv->opts.max_level;
  if (l == 0) {
    if (top == 0) return true;
    const hpc_status s = ctx_size_after_level0(c);  // neighbour lists and records for the edges left
    if (s != HPC_OK) {
      r->status = s;
      return true;
    }
    r->next = 1;
    return false;
  }
  if (C.work_total == 0 || l >= top) return true;  // no edge had enough neighbours, or the last level
  r->next = l + 1;
  return false;
}

void finish(hpc_server *sv, Request *r, std::vector<Request *> *out) {
  if (r->status == HPC_OK && r->adj_out) r->status = hpc_get_adjacency(r->ctx, r->adj_out);
  if (r->ctx) hpc_ctx_destroy(r->ctx);
  r->ctx = nullptr;
  r->t_done = clk::now();
  sv->active_bytes -= r->bytes;
  out->push_back(r);
}

void engine_loop(hpc_server *sv) {
  cudaSetDevice(sv->opts.device);
  std::vector<Request *> finished;
  for (;;) {
    std::vector<Request *> admitted;
    {
      std::unique_lock<std::mutex> lk(sv->mu);
      sv->cv.wait(lk, [&] { return sv->stop || !sv->pending.empty() || !sv->active.empty(); });
      if (sv->stop && sv->pending.empty() && sv->active.empty()) break;
      // admission in arrival order (a request above the whole budget runs alone)
      while (!sv->pending.empty() && (int)admitted.size() < sv->opts.max_inflight &&
             (int)(sv->active.size() + admitted.size()) < sv->opts.max_batch) {
        Request *r = sv->pending.front();
        const bool empty = sv->active.empty() && admitted.empty();
        if (!empty && sv->active_bytes + r->bytes > sv->opts.budget_bytes) break;
        sv->pending.pop_front();
        sv->active_bytes += r->bytes;
        admitted.push_back(r);
      }
    }
    const int running = (int)sv->active.size();  // requests that have run steps already
    for (Request *r : admitted) {
      r->t_start = clk::now();
      r->joined = running;
      r->status = admit(sv, r);
      if (r->status != HPC_OK) finish(sv, r, &finished);
      else sv->active.push_back(r);
    }
    if (!sv->active.empty()) {
      hpc_status s = step(sv);
      std::vector<Request *> keep;
      for (Request *r : sv->active) {
        if (s != HPC_OK) r->status = s;
        if (s != HPC_OK || advance(sv, r)) finish(sv, r, &finished);
        else keep.push_back(r);
      }
      sv->active.swap(keep);
    }
    if (!finished.empty()) {
      std::lock_guard<std::mutex> g(sv->mu);
      for (Request *r : finished) sv->done.push_back(r);
      sv->outstanding -= (int64_t)finished.size();
      finished.clear();
      sv->cv_done.notify_all();
    }
  }
}

}  // namespace

extern "C" {

hpc_status hpc_server_opts_default(hpc_server_opts *o) {
  if (!o) return HPC_ERR_INVALID_ARG;
  std::memset(o, 0, sizeof(*o));
  o->device = 0;
  o->precision = HPC_PREC_MIXED_TC;
  o->max_level = 4;
  o->budget_bytes = 150LL * 1000 * 1000 * 1000;
  o->max_batch = 256;
  o->max_inflight = 32;
  return HPC_OK;
}

hpc_status hpc_server_create(hpc_server **out, const hpc_server_opts *opts) {
  if (!out) return HPC_ERR_INVALID_ARG;
  *out = nullptr;
  hpc_server_opts o;
  if (opts) o = *opts; else hpc_server_opts_default(&o);
  if (o.precision < HPC_PREC_FP64 || o.precision > HPC_PREC_MIXED_TC || o.max_level > HPC_MAX_LEVEL) {
    set_error("server: unknown precision or max_level above HPC_MAX_LEVEL");
    return HPC_ERR_INVALID_ARG;
  }
  if (o.max_batch < 1) o.max_batch = 1;
  if (o.max_inflight < 1) o.max_inflight = 1;
  HPC_CUDA(cudaSetDevice(o.device));
  hpc_server *sv = new hpc_server();
  sv->opts = o;
  cudaDeviceGetAttribute(&sv->sms, cudaDevAttrMultiProcessorCount, o.device);
  if (cudaStreamCreateWithFlags(&sv->st, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete sv;
    set_error("server: stream creation failed");
    return HPC_ERR_CUDA;
  }
  const int top = o.max_level < 0 ? HPC_MAX_LEVEL : o.max_level;
  for (int l = 2; l <= top; ++l) sv->grid[l] = citest_grid(o.precision, l, o.device);
  if (o.precision != HPC_PREC_FP64)
    for (int l = 2; l <= std::min(top, kSetTop); ++l) sv->grid_set[l] = citest_grid(o.precision, l, o.device, kSetOrder);
  if (top >= 1) sv->grid_l1 = citest_grid(o.precision, 1, o.device, kL1Interleaved);
  if (top > 16) retest_setup();
  if (o.precision == HPC_PREC_MIXED_TC) {
    // the shared FP64 re-test queue of every launch (4 Mi entries; a full queue re-tests
    // in place)
    hpc_status s = grow(&sv->d_rq, &sv->rq_cap, 4ll << 20, sv->st);
    if (s == HPC_OK) s = grow(&sv->d_rqv, &sv->rqv_cap, retest_scratch_entries(4ll << 20), sv->st);
    if (s == HPC_OK) s = grow(&sv->d_rqd, &sv->rqd_cap, 4ll << 20, sv->st);
    if (s == HPC_OK && cudaMemsetAsync(sv->d_rqd, 0, sizeof(unsigned int) * (size_t)sv->rqd_cap, sv->st) != cudaSuccess)
      s = HPC_ERR_CUDA;
    if (s != HPC_OK) {
      cudaStreamDestroy(sv->st);
      delete sv;
      return s;
    }
  }
  sv->engine = std::thread(engine_loop, sv);
  *out = sv;
  return HPC_OK;
}

hpc_status hpc_server_submit(hpc_server *sv, const float *X, int64_t p, int64_t n, double alpha, uint8_t *adj_out,
                             int64_t *id) {
  if (!sv || !X || p < 2 || p > 46340 || n < 4 || !(alpha > 0.0 && alpha <= 1.0)) {
    set_error("server: bad request (null data, p outside [2, 46340], n < 4 or alpha outside (0, 1])");
    return HPC_ERR_INVALID_ARG;
  }
  hpc_opts o;
  hpc_opts_default(&o);
  o.precision = sv->opts.precision;
  o.max_level = sv->opts.max_level;
  int64_t bytes = 0;
  hpc_ctx_footprint(p, n, &o, &bytes);
  if (o.precision == HPC_PREC_MIXED_TC) bytes -= ctx_retest_queue_bytes(p * p);  // the engine's queue is shared
  Request *r = new Request();
  r->X = X;
  r->p = p;
  r->n = n;
  r->alpha = alpha;
  r->adj_out = adj_out;
  r->bytes = bytes;
  r->t_submit = clk::now();
  {
    std::lock_guard<std::mutex> g(sv->mu);
    r->id = sv->next_id++;
    sv->pending.push_back(r);
    ++sv->outstanding;
  }
  if (id) *id = r->id;
  sv->cv.notify_all();
  return HPC_OK;
}

hpc_status hpc_server_poll(hpc_server *sv, hpc_served *out, int cap, int *count) {
  if (!sv || !count || (cap > 0 && !out)) return HPC_ERR_INVALID_ARG;
  std::vector<Request *> take;
  {
    std::lock_guard<std::mutex> g(sv->mu);
    const size_t k = std::min<size_t>(sv->done.size(), (size_t)std::max(cap, 0));
    take.assign(sv->done.begin(), sv->done.begin() + k);
    sv->done.erase(sv->done.begin(), sv->done.begin() + k);
  }
  auto ms = [](clk::time_point a, clk::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
  };
  for (size_t i = 0; i < take.size(); ++i) {
    const Request *r = take[i];
    hpc_served &d = out[i];
    d.id = r->id;
    d.status = r->status;
    d.levels = r->levels;
    d.edges = r->edges;
    d.batch_size = r->batch_size;
    d.joined = r->joined;
    d.queue_ms = ms(r->t_submit, r->t_start);
    d.run_ms = ms(r->t_start, r->t_done);
    d.latency_ms = ms(r->t_submit, r->t_done);
    delete r;
  }
  *count = (int)take.size();
  return HPC_OK;
}

hpc_status hpc_server_drain(hpc_server *sv) {
  if (!sv) return HPC_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(sv->mu);
  sv->cv_done.wait(lk, [&] { return sv->outstanding == 0; });
  return HPC_OK;
}

hpc_status hpc_server_destroy(hpc_server *sv) {
  if (!sv) return HPC_OK;
  hpc_server_drain(sv);
  {
    std::lock_guard<std::mutex> g(sv->mu);
    sv->stop = true;
  }
  sv->cv.notify_all();
  if (sv->engine.joinable()) sv->engine.join();
  for (Request *r : sv->done) delete r;
  cudaSetDevice(sv->opts.device);
  for (void *p : {(void *)sv->stage, (void *)sv->d_inst, (void *)sv->d_pre, (void *)sv->d_work, (void *)sv->d_lc,
                  (void *)sv->d_seg, (void *)sv->d_rq, (void *)sv->d_rqv, (void *)sv->d_rqd, (void *)sv->d_levels,
                  (void *)sv->d_out, (void *)sv->d_tune})
    if (p) cudaFreeAsync(p, sv->st);
  cudaStreamSynchronize(sv->st);
  cudaStreamDestroy(sv->st);
  cudaGetLastError();
  delete sv;
  return HPC_OK;
}

}  // extern "C"
