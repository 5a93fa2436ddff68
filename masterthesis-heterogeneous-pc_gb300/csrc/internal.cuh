// Internal declarations shared by the CUDA translation units of libheterogpc.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/heterogpc.h"

namespace hpc {

// ---------------------------------------------------------------------------
// error plumbing (thread-local last error, never exit())
void set_error(const char *fmt, ...);
hpc_status cuda_fail(cudaError_t e, const char *what, const char *file, int line);

#define HPC_CUDA(call)                                                   \
  do {                                                                   \
    cudaError_t e_ = (call);                                             \
    if (e_ != cudaSuccess) return hpc::cuda_fail(e_, #call, __FILE__, __LINE__); \
  } while (0)

#define HPC_LAUNCH_CHECK(what)                                           \
  do {                                                                   \
    cudaError_t e_ = cudaGetLastError();                                 \
    if (e_ != cudaSuccess) return hpc::cuda_fail(e_, what, __FILE__, __LINE__); \
  } while (0)

// ---------------------------------------------------------------------------
// constants of the statistic (src/executor/independence/cpuInd.cpp:6)
constexpr double kCutThr = 0.9999999;

// Device counters of one level (one slot per level, written by that level's kernels).
struct DevCounters {
  unsigned long long tests;        // executed CI tests
  unsigned long long retests;      // tests re-run in FP64 (band, conditioning, non-finite)
  unsigned long long deleted;      // edges removed
  unsigned long long tile_next;    // work-queue head
  unsigned long long work_total;   // T_l
  unsigned long long edges2;       // sum of degrees at the level start
  unsigned long long rec_begin;    // first separation-set record of the level
  unsigned long long band_violations;  // FP32 removals the FP64 post-pass did not confirm
  unsigned long long rq_count;     // FP64 re-tests queued (tensor-core mode)
  int max_deg;                     // at the level start
  int rows;                        // rows with work at this level
  int pad[2];
};
// Context-wide device counters.
struct DevGlobal {
  unsigned long long rec_count;    // separation-set records written (cumulative)
  int err;                         // error bits (kErr*)
  int pad;
};
constexpr int kErrRecOverflow = 1;
constexpr int kErrWorkOverflow = 2;
constexpr int kErrCsrOverflow = 4;
constexpr int kErrTimeout = 8;

// One deferred FP64 re-test: edge (i, j) given ids[0..level), or a level-0 pair (i > j).
struct RetestItem {
  int32_t i, j, level, pad;
  int32_t ids[HPC_MAX_LEVEL];
};

// Everything a level kernel needs, passed by value.
struct LevelArgs {
  int64_t p;
  int W;                 // 32-bit words per adjacency row
  int level;
  int n_obs;
  double alpha;
  double sqrt_n3;        // sqrt(n - 3)
  float r_c;             // |r| at which p == alpha (FP32)
  float margin_r;        // |r| half-width of the fixed re-test band
  float ke;              // error-bound coefficient: |r| error <= ke / (smallest pivot)
  const double *cor64;   // p x p row-major (FP64 correlation)
  const float *cor32;    // p x p row-major (FP32 copy) or null in plain mode
  uint32_t *adj;         // live bitmask p x W
  const int *deg;        // snapshot degrees
  const int *rowptr;     // snapshot CSR offsets (p+1)
  const int *colidx;     // snapshot neighbour ids, ascending per row
  const unsigned long long *row_work;  // exclusive prefix of tests per row (p+1)
  hpc_sepset_record *recs;
  long long rec_cap;
  long long colidx_cap;
  DevCounters *ctr;      // this level's counters
  DevGlobal *gctr;
  // FP64 entries without an FP64 matrix: dot products of the standardised columns
  const double *Z;       // n_z x p column-major (each variable contiguous) or null
  int64_t n_z;
  double denom;          // n - 1 (the Gram's divisor)
  RetestItem *rq;        // deferred FP64 re-tests (tensor-core mode)
  long long rq_cap;
};

// ---------------------------------------------------------------------------
// kernels' host launchers (defined in the .cu files)
hpc_status launch_standardise_f64(const double *X, int64_t n, int64_t p, int ref_compat, double *Z,
                                  cudaStream_t s);
hpc_status launch_standardise_f32(const float *X, int64_t n, int64_t p, int ref_compat, double *Z,
                                  cudaStream_t s);
hpc_status launch_gram_f64(const double *Z, int64_t n, int64_t p, double inv_denom, double *C,
                           cudaStream_t s);
hpc_status launch_to_f32(const double *C, int64_t count, float *C32, cudaStream_t s);
int64_t tc_n_pad(int64_t n);
int64_t tc_p_pad(int64_t p);
int64_t tc_k(int64_t n);
hpc_status launch_standardise_split_f64(const double *X, int64_t n, int64_t p, int ref_compat, double *Z64,
                                        __nv_bfloat16 *P, __nv_bfloat16 *Q, cudaStream_t s);
hpc_status launch_standardise_split_f32(const float *X, int64_t n, int64_t p, int ref_compat, double *Z64,
                                        __nv_bfloat16 *P, __nv_bfloat16 *Q, cudaStream_t s);
hpc_status launch_gram_tc(const __nv_bfloat16 *P, const __nv_bfloat16 *Q, int64_t n, int64_t p, float *C, int *err,
                          cudaStream_t s);
hpc_status launch_level0(const LevelArgs &a, double r_lo, double r_hi, cudaStream_t s);
hpc_status launch_degrees(const LevelArgs &a, int *deg, cudaStream_t s);
hpc_status launch_scan(int64_t p, int level, const int *deg, int *rowptr, unsigned long long *row_work,
                       DevCounters *ctr, DevGlobal *g, cudaStream_t s);
hpc_status launch_fill_csr(const LevelArgs &a, int *colidx, cudaStream_t s);
hpc_status launch_expand_adjacency(const uint32_t *adj, int64_t p, int W, uint8_t *out, cudaStream_t s);
hpc_status launch_citest(const LevelArgs &a, int precision, int grid, cudaStream_t s);
hpc_status launch_finalize_records(const LevelArgs &a, cudaStream_t s);
hpc_status launch_retest(const LevelArgs &a, int sms, cudaStream_t s);
hpc_status launch_level0_f32(const LevelArgs &a, float lo, float hi, cudaStream_t s);
hpc_status launch_mirror(const LevelArgs &a, cudaStream_t s);
int citest_grid(int precision, int level, int device);

}  // namespace hpc

// ---------------------------------------------------------------------------
// The context (opaque to callers).
struct hpc_ctx {
  int64_t p = 0, n = 0;
  hpc_opts opts{};
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  int W = 0;
  double *cor64 = nullptr;
  float *cor32 = nullptr;
  double *Z = nullptr;          // standardised data (n x p)
  int64_t Z_elems = 0;
  __nv_bfloat16 *tcP = nullptr, *tcQ = nullptr;  // split-BF16 operands of the tensor-core Gram
  int64_t tc_elems = 0;
  void *X_stage = nullptr;      // device copy of host observations
  int64_t X_stage_bytes = 0;
  uint32_t *adj = nullptr;
  uint8_t *adj_bytes = nullptr;  // p x p expansion for hpc_get_adjacency
  hpc::RetestItem *rq = nullptr;  // deferred FP64 re-tests (tensor-core mode)
  int64_t rq_cap = 0;
  bool cor64_valid = false;       // cor64 holds the current FP64 matrix
  int *deg = nullptr;
  int *rowptr = nullptr;
  int *colidx = nullptr;
  int64_t colidx_cap = 0;
  unsigned long long *row_work = nullptr;
  hpc_sepset_record *recs = nullptr;
  int64_t rec_cap = 0;
  hpc::DevCounters *ctr = nullptr;      // device, one slot per level (HPC_MAX_LEVEL + 1)
  hpc::DevCounters *ctr_host = nullptr; // pinned mirror
  hpc::DevGlobal *gctr = nullptr;       // device
  hpc::DevGlobal *gctr_host = nullptr;  // pinned mirror
  cudaStream_t own_stream = nullptr; // the context's stream; `stream` may be a caller's
  cudaEvent_t evc[4] = {nullptr, nullptr, nullptr, nullptr};  // correlation phases
  cudaEvent_t evl[HPC_MAX_LEVEL + 1][3] = {};  // per level: start, snapshot done, tests done
  // CUDA graph of the whole level sequence 0..graph_top, replayed while the
  // buffers it was captured with stay in place
  cudaGraphExec_t graph = nullptr;
  int graph_top = -1;
  cudaStream_t graph_stream = nullptr;
  int64_t graph_colidx_cap = 0, graph_rec_cap = 0;
  int64_t graph_launches = 0;
  bool graph_cor64_valid = false;
  bool graphs_enabled = true;
  bool last_run_graph = false;
  cudaEvent_t evr[2] = {nullptr, nullptr};  // whole skeleton run
  int citest_grid[HPC_MAX_LEVEL + 1] = {};  // persistent grid size per level
  bool cor_timed = false;
  hpc_timings timings{};
  bool have_cor = false;
  bool cor32_rounded = true;   // cor32 is the FP32 rounding of cor64 (else the tensor-core Gram)
  int next_level = 0;
  int64_t edges = 0;           // undirected edges after the last level
  double zc = 0.0;             // z_crit (FP64)
  double r_crit = 0.0;         // |r| at which p == alpha
};
