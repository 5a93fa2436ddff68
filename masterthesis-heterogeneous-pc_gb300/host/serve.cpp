// Skeleton serving with continuous batching (no reference counterpart: the
// reference answers one problem per process run).
//
// Requests (observations of one problem each) arrive at any time. A scheduler
// thread admits the requests that have arrived, in arrival order, as one batch --
// a context whose level kernels run once for all its instances -- as long as the
// device bytes of the batches in flight stay within the budget and fewer than
// `max_inflight` batches are running; each batch runs on a worker thread with its
// own CUDA stream, so batches admitted while others are on the GPU overlap with
// them. A request's correlation matrix and level state stay on the device until
// its batch finishes; then its edge count (and, on request, its adjacency) is
// copied out, the batch's memory is returned and waiting requests are admitted.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/heterogpc.h"

namespace {

using clk = std::chrono::steady_clock;

struct Request {
  int64_t id;
  const float *X;
  int64_t p, n;
  double alpha;
  uint8_t *adj_out;
  int64_t bytes;
  clk::time_point t_submit, t_start, t_done;
  hpc_status status = HPC_OK;
  int levels = 0;
  int64_t edges = 0;
  int batch_size = 0;
};

}  // namespace

struct hpc_server {
  hpc_server_opts opts{};
  std::mutex mu;
  std::condition_variable cv;        // scheduler wake-up
  std::condition_variable cv_done;   // drain
  std::deque<Request *> pending;
  std::vector<Request *> done;
  int64_t next_id = 0;
  int64_t inflight_bytes = 0;
  int inflight_batches = 0;
  int64_t outstanding = 0;           // submitted, not yet completed
  bool stop = false;
  std::thread scheduler;
  std::vector<std::thread> workers;
  clk::time_point t0 = clk::now();
};

namespace {

void run_batch(hpc_server *sv, std::vector<Request *> batch, int64_t bytes) {
  const auto t_start = clk::now();
  for (Request *r : batch) r->t_start = t_start;
  const int count = (int)batch.size();
  std::vector<int64_t> ps(count), ns(count);
  std::vector<double> alphas(count);
  for (int b = 0; b < count; ++b) {
    ps[b] = batch[b]->p;
    ns[b] = batch[b]->n;
    alphas[b] = batch[b]->alpha;
  }
  hpc_opts o;
  hpc_opts_default(&o);
  o.device = sv->opts.device;
  o.precision = sv->opts.precision;
  o.max_level = sv->opts.max_level;
  hpc_ctx *ctx = nullptr;
  hpc_status s = hpc_batch_create(&ctx, count, ps.data(), ns.data(), alphas.data(), &o);
  std::vector<int64_t> off(count + 1);
  float *staged = nullptr;
  cudaStream_t st = nullptr;
  if (s == HPC_OK) s = hpc_batch_offsets(ctx, off.data(), nullptr);
  if (s == HPC_OK) {
    // observations of every request into one packed device buffer, one copy each
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMallocAsync((void **)&staged, sizeof(float) * (size_t)off[count], st) != cudaSuccess) {
      cudaGetLastError();
      s = HPC_ERR_OOM;
    }
  }
  if (s == HPC_OK) {
    for (int b = 0; b < count && s == HPC_OK; ++b)
      if (cudaMemcpyAsync(staged + off[b], batch[b]->X, sizeof(float) * (size_t)(off[b + 1] - off[b]),
                          cudaMemcpyHostToDevice, st) != cudaSuccess)
        s = HPC_ERR_CUDA;
    if (s == HPC_OK) s = hpc_ctx_set_stream(ctx, st);
    if (s == HPC_OK) s = hpc_correlation_device_f32(ctx, staged);
    hpc_level_stats stats[HPC_MAX_LEVEL + 1];
    int levels = 0;
    if (s == HPC_OK) s = hpc_run_skeleton(ctx, stats, HPC_MAX_LEVEL + 1, &levels);
    for (int b = 0; b < count; ++b) {
      Request *r = batch[b];
      r->batch_size = count;
      r->status = s;
      if (s != HPC_OK) continue;
      hpc_batch_edge_count(ctx, b, &r->edges);
      int lv = 0;
      hpc_batch_level_stats(ctx, b, nullptr, 0, &lv);
      r->levels = lv;
      if (r->adj_out) r->status = hpc_batch_get_adjacency(ctx, b, r->adj_out);
    }
  } else {
    for (Request *r : batch) r->status = s;
  }
  if (staged) cudaFreeAsync(staged, st);
  if (ctx) hpc_ctx_destroy(ctx);
  if (st) {
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
  }
  const auto t_done = clk::now();
  std::lock_guard<std::mutex> g(sv->mu);
  for (Request *r : batch) {
    r->t_done = t_done;
    sv->done.push_back(r);
  }
  sv->inflight_bytes -= bytes;
  --sv->inflight_batches;
  sv->outstanding -= count;
  sv->cv.notify_all();
  sv->cv_done.notify_all();
}

void scheduler_loop(hpc_server *sv) {
  cudaSetDevice(sv->opts.device);
  std::unique_lock<std::mutex> lk(sv->mu);
  while (true) {
    sv->cv.wait(lk, [&] {
      return sv->stop || (!sv->pending.empty() && sv->inflight_batches < sv->opts.max_inflight &&
                          sv->inflight_bytes + sv->pending.front()->bytes <= sv->opts.budget_bytes) ||
             (!sv->pending.empty() && sv->inflight_batches == 0);
    });
    if (sv->stop && sv->pending.empty()) break;
    if (sv->pending.empty()) continue;
    // admit in arrival order while the budget allows (a request larger than the
    // whole budget runs alone once nothing else is in flight)
    std::vector<Request *> batch;
    int64_t bytes = 0;
    while (!sv->pending.empty() && (int)batch.size() < sv->opts.max_batch) {
      Request *r = sv->pending.front();
      if (!batch.empty() && sv->inflight_bytes + bytes + r->bytes > sv->opts.budget_bytes) break;
      if (batch.empty() && sv->inflight_batches > 0 && sv->inflight_bytes + r->bytes > sv->opts.budget_bytes) break;
      batch.push_back(r);
      bytes += r->bytes;
      sv->pending.pop_front();
    }
    if (batch.empty()) continue;
    sv->inflight_bytes += bytes;
    ++sv->inflight_batches;
    sv->workers.emplace_back([sv, batch, bytes]() {
      cudaSetDevice(sv->opts.device);
      run_batch(sv, batch, bytes);
    });
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
  o->max_batch = 64;
  o->max_inflight = 4;
  return HPC_OK;
}

hpc_status hpc_server_create(hpc_server **out, const hpc_server_opts *opts) {
  if (!out) return HPC_ERR_INVALID_ARG;
  hpc_server *sv = new hpc_server();
  if (opts) sv->opts = *opts; else hpc_server_opts_default(&sv->opts);
  if (sv->opts.max_batch < 1) sv->opts.max_batch = 1;
  if (sv->opts.max_inflight < 1) sv->opts.max_inflight = 1;
  sv->scheduler = std::thread(scheduler_loop, sv);
  *out = sv;
  return HPC_OK;
}

hpc_status hpc_server_submit(hpc_server *sv, const float *X, int64_t p, int64_t n, double alpha, uint8_t *adj_out,
                             int64_t *id) {
  if (!sv || !X || p < 2 || n < 4 || !(alpha > 0.0 && alpha <= 1.0)) return HPC_ERR_INVALID_ARG;
  hpc_opts o;
  hpc_opts_default(&o);
  o.precision = sv->opts.precision;
  int64_t bytes = 0;
  hpc_ctx_footprint(p, n, &o, &bytes);
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
  if (!sv || !count) return HPC_ERR_INVALID_ARG;
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
  if (sv->scheduler.joinable()) sv->scheduler.join();
  for (auto &w : sv->workers)
    if (w.joinable()) w.join();
  for (Request *r : sv->done) delete r;
  delete sv;
  return HPC_OK;
}

}  // extern "C"
