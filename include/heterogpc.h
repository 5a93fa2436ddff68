/*
 * heterogpc.h -- C ABI of the GB300 PC-stable skeleton library (libheterogpc.so).
 *
 * PC-stable skeleton discovery with Gaussian (Fisher-z partial-correlation)
 * conditional-independence tests on one GPU. Every entry point takes plain
 * pointers and sizes, returns an hpc_status and never exits the process
 * (the reference calls exit() on every CUDA error, src/util/cuda_util.cuh:28-50).
 *
 * Each function names the reference interface it replaces (paths are relative
 * to the milanpro/Masterthesis-Heterogeneous-PC source tree).
 *
 * Threading: a context is used by one host thread at a time; all its work is
 * ordered on the context's own CUDA stream.
 */
#ifndef HETEROGPC_H
#define HETEROGPC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HPC_ABI_VERSION 1
/* Highest conditioning-set size the kernels accept (levels 1-16 run unrolled kernels,
 * 17-32 one kernel with the level read at run time). A skeleton run "until exhausted"
 * (max_level = -1) stops after this level. */
#define HPC_MAX_LEVEL 32

typedef enum hpc_status {
  HPC_OK = 0,
  HPC_ERR_INVALID_ARG = 1, /* bad pointer, size or option */
  HPC_ERR_OOM = 2,         /* device or host allocation failed */
  HPC_ERR_CUDA = 3,        /* a CUDA runtime call failed */
  HPC_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up */
  HPC_ERR_NUMERIC = 5,     /* non-finite input where finite values are required */
  HPC_ERR_STATE = 6,       /* call out of order (e.g. run before correlation) */
  HPC_ERR_CAPACITY = 7,    /* a device work or record buffer would overflow */
  HPC_ERR_NO_DEVICE = 8    /* no CUDA device / extension not usable */
} hpc_status;

typedef enum hpc_precision {
  /* Plain path: FP64 correlation, every CI test in FP64. */
  HPC_PREC_FP64 = 0,
  /* FP64 correlation, CI tests in FP32; tests whose |z| lies within the margin
   * of z_crit, and ill-conditioned or non-finite ones, are re-run in FP64. */
  HPC_PREC_MIXED = 1,
  /* Split-BF16 tensor-core Gram (FP32 accumulation) for the FP32 correlation,
   * FP32 tests, FP64 re-tests on exact FP64 correlation entries computed on
   * demand from the FP64-standardised data. */
  HPC_PREC_MIXED_TC = 2
} hpc_precision;

typedef struct hpc_opts {
  int device;            /* CUDA device ordinal (default 0) */
  double alpha;          /* significance level; an edge is removed iff p >= alpha (default 0.05) */
  int max_level;         /* highest level run; -1 = until no edge has enough neighbours (default 4) */
  int precision;         /* hpc_precision (default HPC_PREC_MIXED) */
  double retest_margin;  /* relative |z| band around z_crit re-tested in FP64 (default 1e-3) */
  int ref_compat_sd;     /* 1: standard deviation rounded through float like src/correlation/corHelper.cu:75 */
  int verbose;           /* 1: per-level lines on stdout */
} hpc_opts;

typedef struct hpc_level_stats {
  int level;
  int max_degree;             /* largest neighbour count at the level start */
  int64_t rows;               /* rows with at least `level` neighbours */
  int64_t potential_tests;    /* T_l = sum over directed edges of C(d_i - 1, l) */
  int64_t executed_tests;     /* CI tests actually evaluated on the device */
  int64_t retests;            /* tests re-run in FP64 (band, conditioning, non-finite) */
  int64_t edges_before;       /* undirected edges at the level start */
  int64_t edges_after;        /* undirected edges after the level */
  double ms;                  /* device time of the level (compaction + tests), CUDA events */
} hpc_level_stats;

typedef struct hpc_sepset_record {
  int32_t i, j;               /* i < j, the removed edge */
  int32_t level;              /* conditioning-set size; 0 = marginal (reference marker -2) */
  int32_t pad;
  double pmax;                /* FP64 p-value of the removing test */
  int32_t ids[HPC_MAX_LEVEL]; /* ascending separating variables, `level` of them */
} hpc_sepset_record;

/* Device-time breakdown of the last calls, from CUDA events on the context stream. */
typedef struct hpc_timings {
  double standardise_ms;                 /* last correlation: column standardisation */
  double gram_ms;                        /* last correlation: Gram */
  double convert_ms;                     /* last correlation: FP32 copy */
  double level_ms[HPC_MAX_LEVEL + 1];    /* whole level (snapshot + tests) */
  double compact_ms[HPC_MAX_LEVEL + 1];  /* neighbour-list snapshot of the level */
  double test_ms[HPC_MAX_LEVEL + 1];     /* CI-test kernel of the level */
  int64_t launches;                      /* kernels launched by this context so far */
  double skeleton_ms;                    /* last hpc_run_skeleton as a whole */
  double retest_ms[HPC_MAX_LEVEL + 1];   /* FP64 re-test kernel of the level (tensor-core mode) */
  double rebuild_ms[HPC_MAX_LEVEL + 1];  /* level kernel, neighbour-list rebuild phase (device timer) */
  double scan_ms[HPC_MAX_LEVEL + 1];     /* level kernel, test-count scan phase (device timer) */
} hpc_timings;

typedef struct hpc_ctx hpc_ctx;

/* ---- errors ------------------------------------------------------------ */
/* Message for the last failing call on this host thread. */
const char *hpc_last_error_string(void);
/* Short name of a status code. */
const char *hpc_status_string(hpc_status s);

/* ---- context ------------------------------------------------------------
 * Replaces MMState's constructor (src/util/state.cu:3-44, struct at
 * src/util/state.cuh:29-56): all p x p state lives in device memory owned by
 * the context, not in managed memory. */
hpc_status hpc_opts_default(hpc_opts *opts);
hpc_status hpc_ctx_create(hpc_ctx **out, int64_t p, int64_t n_obs, const hpc_opts *opts);
hpc_status hpc_ctx_destroy(hpc_ctx *ctx);
/* Resets adjacency (complete graph minus diagonal) and separation sets, keeping
 * the correlation matrix (src/util/state.cu:31-43). */
hpc_status hpc_ctx_reset(hpc_ctx *ctx);
/* Orders all of the context's work on `stream` (a cudaStream_t of the same device,
 * owned by the caller) instead of the context's own stream; NULL restores it. */
hpc_status hpc_ctx_set_stream(hpc_ctx *ctx, void *stream);
/* hpc_run_skeleton captures its level sequence into a CUDA graph and replays it on
 * later runs (enable = 1, the default); 0 runs it kernel by kernel, which also
 * records the per-level kernel timings (graph replays time the whole skeleton only). */
hpc_status hpc_ctx_set_graphs(hpc_ctx *ctx, int enable);
/* Device-time breakdown of the context's last correlation and levels. */
hpc_status hpc_get_timings(hpc_ctx *ctx, hpc_timings *out);
/* Device bytes held by a context of this shape (admission control). */
hpc_status hpc_ctx_footprint(int64_t p, int64_t n_obs, const hpc_opts *opts, int64_t *bytes);

/* ---- correlation --------------------------------------------------------
 * Replaces gpuPMCC(h_mat, n, dim, cors, deviceId, verbose)
 * (src/correlation/corOwn.cuh:3, src/correlation/corOwn.cu:10-48).
 * X is column-major n_obs x p (each variable's samples contiguous), exactly the
 * arma::mat layout returned by CSVParser::read_csv_to_mat (src/util/csv_parser.cpp:64-77).
 * Host pointers are copied to the device on the context's stream: from pageable memory
 * the call returns once the data has left the caller's buffer; from pinned (page-locked)
 * memory it returns once the copy, the standardisation and the Gram are queued, and the
 * caller keeps X_host unchanged until a later call on the context that waits for its
 * stream (hpc_run_skeleton, hpc_wait, a result read) has returned. *_device variants
 * take device pointers already resident in HBM. */
hpc_status hpc_correlation_f64(hpc_ctx *ctx, const double *X_host);
hpc_status hpc_correlation_f32(hpc_ctx *ctx, const float *X_host);
hpc_status hpc_correlation_device_f64(hpc_ctx *ctx, const double *X_dev);
hpc_status hpc_correlation_device_f32(hpc_ctx *ctx, const float *X_dev);
/* Replaces SkeletonCalculator::add_correlation_matrix's memcpy into state.cor
 * (src/independence/skeleton.cpp:60-65). C is row-major p x p. */
hpc_status hpc_load_correlation(hpc_ctx *ctx, const double *C_host);
hpc_status hpc_load_correlation_device(hpc_ctx *ctx, const double *C_dev);
/* Copies the FP64 correlation matrix (row-major p x p) to the host. */
hpc_status hpc_get_correlation(hpc_ctx *ctx, double *C_host);
/* Copies the FP32 correlation the mixed-precision tests read (row-major p x p):
 * the tensor-core split-BF16 Gram in HPC_PREC_MIXED_TC, else the FP32 rounding. */
hpc_status hpc_get_correlation_f32(hpc_ctx *ctx, float *C_host);

/* Allocation-free correlation. No counterpart in the reference: it serves callers
 * that cannot allocate device memory when they need the matrix, such as a plugin
 * in a host application that owns all GPU memory through its own pool, or a
 * latency-critical caller that cannot afford the device-wide synchronisation that
 * cudaMalloc/cudaFree may cause. No context is needed. X_dev (column-major n_obs x p
 * FP64, device) and C_dev (row-major p x p FP64, device) are the caller's; the
 * standardised data lives in one library-wide __device__ array of
 * HPC_NOALLOC_MAX_ELEMS doubles (32 MiB, held by every GPU that loads the library
 * until the process exits), so n_obs * p above that limit returns HPC_ERR_CAPACITY.
 * Work is queued on `stream` (a cudaStream_t, NULL = default stream) and is not
 * waited for. The first call on a device looks up the array's device address;
 * make it before any stream capture. All calls share the array: calls that
 * overlap on the GPU race, so order them on one stream. Results equal those of
 * hpc_correlation_device_f64. */
#define HPC_NOALLOC_MAX_ELEMS (4LL * 1024 * 1024)
hpc_status hpc_correlation_noalloc_f64(const double *X_dev, int64_t n_obs, int64_t p, int ref_compat_sd,
                                       double *C_dev, void *stream);

/* ---- skeleton levels ----------------------------------------------------
 * hpc_run_level replaces SkeletonCalculator::calcLevel (src/independence/skeleton.cpp:104-150):
 * for level >= 1 it first snapshots the neighbour lists (callCompact,
 * src/independence/compact.cu:91-99), then runs every CI test of the level
 * (GPUExecutor::executeLevel, src/executor/gpuExecutor.cu:9-122, and the
 * testRowL0/L1/LN kernels, src/executor/testing/gpuRowTests.cu) for any level,
 * not only 0..3. Levels must be run in order 0, 1, 2, ...
 * Returns HPC_OK with stats->potential_tests == 0 when no edge has enough neighbours. */
hpc_status hpc_run_level(hpc_ctx *ctx, int level, hpc_level_stats *stats);
/* Replaces SkeletonCalculator::run's level loop (src/independence/skeleton.cpp:152-190):
 * levels 0..max_level (opts.max_level, -1 = until exhausted), stopping early once a
 * level has no tests. `stats` receives up to `cap` per-level records. */
hpc_status hpc_run_skeleton(hpc_ctx *ctx, hpc_level_stats *stats, int cap, int *levels_run);
/* hpc_run_skeleton from a fresh start (as after hpc_ctx_reset) without waiting: the
 * counter reset and the captured level sequence are queued on the context's stream
 * and the call returns; hpc_wait synchronises and returns what hpc_run_skeleton
 * would have. Runs of the same context queue behind each other, so a caller can keep
 * the GPU busy across skeletons. The first run of a context (which sizes the
 * neighbour lists and, with max_level = -1, finds how many levels the data need) and
 * runs that cannot be captured (legacy default stream, graphs disabled) are run
 * synchronously inside the call. With max_level = -1 later runs queue the levels the
 * previous run needed; hpc_wait continues level by level if the data reach further.
 * Every skeleton run ends with the FP64 p-values of its removals (pmax), so records
 * read afterwards need no further device work. No counterpart in the reference,
 * which runs one skeleton per process. */
hpc_status hpc_run_skeleton_async(hpc_ctx *ctx);
hpc_status hpc_wait(hpc_ctx *ctx, hpc_level_stats *stats, int cap, int *levels_run);

/* ---- tile policy and autotuner -------------------------------------------
 * No counterpart in the reference, whose launch shapes are fixed
 * (src/executor/gpuExecutor.cu:45-106). The CI tests of a level are a flattened
 * space of (row, neighbour, subset) indices that warps claim in tiles; a tile policy
 * sets how a launch cuts it:
 *   tile_cap        largest run of consecutive tests (subset chunk) a lane takes per tile
 *   tiles_per_lane  target number of tiles per lane of the grid (balance vs claim cost)
 *   edge_lanes      level 1 only: 32 = a warp's lanes interleaved over one edge's tests
 *                   (coalesced gathers), 1 = each lane a chunk of consecutive tests (the
 *                   mapping of the higher levels)
 *   l1_prefetch     level 1 with edge_lanes 32 only: 1 = the next step's entries are loaded
 *                   one step ahead (pays off on long neighbour lists)
 * Defaults: 64, 4, 32, 0. A process-wide table holds policies keyed by buckets of
 * (largest p of the launch, level, largest degree at the level start), buckets being
 * bit lengths; every level kernel reads its entry on the device after its test-count
 * scan, so the table also steers CUDA-graph replays. */
typedef struct hpc_tune_params {
  int tile_cap;        /* 1..65536 */
  int tiles_per_lane;  /* 1..64 */
  int edge_lanes;      /* 1 or 32 */
  int l1_prefetch;     /* 0 or 1 */
} hpc_tune_params;
/* Sets (prm != NULL) or erases (NULL) the table entry of the key's buckets. */
hpc_status hpc_tune_set(int64_t p, int level, int max_degree, const hpc_tune_params *prm);
/* The policy a launch with this key uses; *found (optional) = 0 when it is the default. */
hpc_status hpc_tune_lookup(int64_t p, int level, int max_degree, hpc_tune_params *out, int *found);
hpc_status hpc_tune_clear(void);
/* The table as a text file (entries only), and back: loaded entries replace those of
 * the same key. */
hpc_status hpc_tune_save(const char *path);
hpc_status hpc_tune_load(const char *path);
/* Forces one policy on every level of the context's runs (NULL = the table again). */
hpc_status hpc_ctx_set_tune(hpc_ctx *ctx, const hpc_tune_params *force);
/* Autotuner: runs the context's skeleton (on its current correlation, kernel by
 * kernel) once per candidate policy in each of `reps` rounds, times every level's
 * CI-test kernel with CUDA events, and stores for each level the candidate with the
 * smallest median time under the level's key. cands/ncands: the candidates (NULL = the built-in grid: tile_cap
 * 16, 64, 256, 1024 x tiles_per_lane 2, 4, 8 x level-1 kernel interleaved,
 * interleaved with prefetch, chunked). chosen (optional,
 * HPC_MAX_LEVEL + 1 entries) receives each level's choice (zeros for levels not run);
 * *entries (optional) the number of table entries written. Decisions, and so the
 * skeleton, do not depend on the policy; the context is reset afterwards. */
hpc_status hpc_autotune(hpc_ctx *ctx, const hpc_tune_params *cands, int ncands, int reps, hpc_tune_params *chosen,
                        int *entries);

/* ---- results ------------------------------------------------------------ */
/* adj (row-major p x p, 1 = edge kept), the reference's state.adj. */
hpc_status hpc_get_adjacency(hpc_ctx *ctx, uint8_t *adj_host);
/* Number of undirected edges left (printSepsets' count, src/util/sepset_util.hpp:9-60). */
hpc_status hpc_edge_count(hpc_ctx *ctx, int64_t *edges);
/* Separation sets in the reference layout (src/util/state.cu:7,25 and
 * src/executor/testing/cpuUtil.cpp:3-48): out[(i*p + j)*max_cond + k] for i < j,
 * -1 = none, -2 in slot 0 = removed at level 0. out holds p*p*max_cond ints. */
hpc_status hpc_get_sepsets(hpc_ctx *ctx, int32_t *out, int max_cond);
/* Records of every edge removed at level >= 1 (level-0 removals are implied by
 * the adjacency): *count receives the number available; at most cap are copied. */
hpc_status hpc_get_sepset_records(hpc_ctx *ctx, hpc_sepset_record *out, int64_t cap, int64_t *count);

/* ---- batches ----------------------------------------------------------------
 * Many independent skeleton problems (uneven p, n and alpha) in one context; no
 * counterpart in the reference, which runs one problem per process. Each kernel of
 * each level runs once for all instances (one shared launch per kernel), so
 * hundreds of small problems fill the GPU together. The correlation and run calls
 * above act on every instance of a batch: observations are packed (instance b's
 * column-major n_b x p_b block starts at element obs_offsets[b]) and loaded
 * correlation matrices likewise (row-major p_b x p_b at cor_offsets[b]); the
 * single-instance result calls act on instance 0. */
hpc_status hpc_batch_create(hpc_ctx **out, int count, const int64_t *p, const int64_t *n_obs, const double *alpha,
                            const hpc_opts *opts);
hpc_status hpc_batch_size(hpc_ctx *ctx, int *count);
/* count + 1 offsets each (the last is the total); either pointer may be NULL */
hpc_status hpc_batch_offsets(hpc_ctx *ctx, int64_t *obs_offsets, int64_t *cor_offsets);
/* per-level statistics of instance idx of the last run */
hpc_status hpc_batch_level_stats(hpc_ctx *ctx, int idx, hpc_level_stats *out, int cap, int *levels);
hpc_status hpc_batch_get_adjacency(hpc_ctx *ctx, int idx, uint8_t *adj_host);
hpc_status hpc_batch_edge_count(hpc_ctx *ctx, int idx, int64_t *edges);
hpc_status hpc_batch_get_sepset_records(hpc_ctx *ctx, int idx, hpc_sepset_record *out, int64_t cap,
                                        int64_t *count);
/* The same from record `first` on (for reading millions of records in chunks). */
hpc_status hpc_batch_get_sepset_records_from(hpc_ctx *ctx, int idx, int64_t first, hpc_sepset_record *out,
                                             int64_t cap, int64_t *count);
/* Results of every instance in one copy each, for callers that read a whole batch:
 * the live adjacency as bitmasks (instance b's p_b rows of W_b = ceil(p_b / 32) 32-bit
 * words start at word_offsets[b]; bit j % 32 of word j / 32 of row i set = edge i-j
 * kept; count + 1 offsets, the last the total) ... */
hpc_status hpc_batch_adjacency_words(hpc_ctx *ctx, int64_t *word_offsets);
hpc_status hpc_batch_get_adjacency_bits(hpc_ctx *ctx, uint32_t *bits_host, int64_t words);
/* ... and the separation-set records of all instances back to back: instance b's are
 * out[prefix[b] .. prefix[b + 1]) (prefix: count + 1 entries, always written; at most
 * cap records copied, none when out is NULL). */
hpc_status hpc_batch_get_all_sepset_records(hpc_ctx *ctx, hpc_sepset_record *out, int64_t cap, int64_t *prefix);
/* ... or packed, for bulk transfer: record after record (instance by instance, each
 * instance's in level order) the 32-bit words i, j, level, 0, pmax (a double in two
 * words), then the `level` separating ids padded with -1 to an even count, i.e.
 * 6 + 2 * ceil(level / 2) words per record; instance b's records start at word
 * inst_words[b] (count + 1 entries, always written; the last is the total). At most
 * cap_words words are copied, none when out is NULL. */
hpc_status hpc_batch_get_records_packed(hpc_ctx *ctx, int32_t *out, int64_t cap_words, int64_t *inst_words);

/* ---- serving ----------------------------------------------------------------
 * Continuous batching of skeleton requests (no reference counterpart; the
 * reference's level loop is src/independence/skeleton.cpp:152-190). One engine
 * thread runs steps: in a step, the requests standing at the same level share one
 * launch of that level's kernels (the kernels run over a table of instances), and
 * requests at different levels run as consecutive launches of the step. After each
 * step every request moves on to its next level or completes, and requests that
 * arrived meanwhile are admitted -- in arrival order, while the device bytes of the
 * admitted requests (hpc_ctx_footprint without the re-test queue, which the engine
 * shares) stay within budget_bytes -- and join at level 0 in the next step, while
 * the others continue. Each request's data stay resident on the device from its
 * admission to its completion. */
typedef struct hpc_server hpc_server;
typedef struct hpc_server_opts {
  int device;
  int precision;          /* default HPC_PREC_MIXED_TC */
  int max_level;          /* default 4; -1 = until no edge has enough neighbours */
  int64_t budget_bytes;   /* device bytes admitted at once (default 150 GB) */
  int max_batch;          /* most requests on the device at once (default 256) */
  int max_inflight;       /* most requests admitted between two steps (default 32) */
} hpc_server_opts;
typedef struct hpc_served {
  int64_t id;
  int32_t status;         /* hpc_status of the request */
  int32_t levels;         /* levels run */
  int64_t edges;          /* undirected edges of its skeleton */
  double queue_ms;        /* submit -> admitted */
  double run_ms;          /* admitted -> results copied */
  double latency_ms;      /* submit -> results copied */
  int32_t batch_size;     /* most requests that shared one of its level launches */
  int32_t joined;         /* requests already running when it was admitted */
} hpc_served;
hpc_status hpc_server_opts_default(hpc_server_opts *opts);
hpc_status hpc_server_create(hpc_server **out, const hpc_server_opts *opts);
/* X: host FP32, column-major n_obs x p; X and adj_out (optional, p x p bytes) must
 * stay valid until the request is returned by hpc_server_poll. */
hpc_status hpc_server_submit(hpc_server *sv, const float *X, int64_t p, int64_t n_obs, double alpha, uint8_t *adj_out,
                             int64_t *id);
/* completed requests since the last poll, at most cap */
hpc_status hpc_server_poll(hpc_server *sv, hpc_served *out, int cap, int *count);
hpc_status hpc_server_drain(hpc_server *sv);
hpc_status hpc_server_destroy(hpc_server *sv);

/* ---- independence statistics (FP64) -------------------------------------
 * Same semantics as CPU::calcPValue / CPU::pValL1 / CPU::pValLN
 * (src/executor/independence/cpuInd.hpp:3-10, cpuInd.cpp:8-38). M is the
 * row-major k x k correlation submatrix ordered (i, j, S...). These are the
 * device FP64 re-test formulas compiled for the host, for callers of that API. */
double hpc_calc_pvalue(double r, int n_obs);
double hpc_pval_l1(double x1, double x2, double x3, int n_obs);
double hpc_pval_ln(const double *M, int k, int n_obs);
/* z_crit = Phi^-1(1 - alpha/2): p >= alpha  <=>  |z| <= z_crit. */
double hpc_z_crit(double alpha);

/* ---- test hooks ------------------------------------------------------------
 * Failure injection on the host, for tests of the error paths (no counterpart in the
 * reference, which exits the process on any CUDA error, src/util/cuda_util.cuh:28-50).
 * hpc_debug_fail_allocation(k): the k-th device allocation of the library from now on
 * fails with HPC_ERR_OOM (k = 0 clears it). hpc_debug_live_allocations: the library's
 * device allocations currently held (a failed call must leave it unchanged).
 * hpc_debug_set_barrier: the bound of the level kernels' grid-barrier waits
 * (default 2e9 ns) and 0 or 1 arrivals added to their target -- with 1 the wait cannot
 * complete, runs out after wait_ns, and the run returns HPC_ERR_TIMEOUT; the context
 * works again after hpc_debug_set_barrier(ctx, 2000000000, 0) and hpc_ctx_reset. */
hpc_status hpc_debug_fail_allocation(int64_t k);
int64_t hpc_debug_live_allocations(void);
hpc_status hpc_debug_set_barrier(hpc_ctx *ctx, int64_t wait_ns, int extra_arrivals);
/* hpc_debug_set_order_from(level): the lowest level whose CI tests run in the set order
 * (one Cholesky factor of a conditioning set serves every neighbour outside it), 2..32,
 * or 0 for the edge order (each test factors its own set) at every level; process-wide,
 * read when a level is launched. Both orders give the same skeleton; the default is 3. */
hpc_status hpc_debug_set_order_from(int level);
/* hpc_debug_set_retest_queue(ctx, entries): replace the context's FP64 re-test queue by
 * one of `entries` entries (so that a test can make it overflow). When a set-order level
 * finds the queue full, the run is repeated from level 0 in the edge order, whose tests
 * re-test inline when the queue is full; hpc_debug_set_order_active then returns 0 for
 * the context (1 while the set order is in use). */
hpc_status hpc_debug_set_retest_queue(hpc_ctx *ctx, int64_t entries);
int hpc_debug_set_order_active(hpc_ctx *ctx);

/* ---- synthetic data ------------------------------------------------------
 * Seeded linear-Gaussian SEM (no reference counterpart; the reference reads
 * CSV files only). Bit-identical output on every host. */
typedef enum hpc_graph_kind { HPC_GRAPH_ER = 0, HPC_GRAPH_PA = 1 } hpc_graph_kind;
typedef struct hpc_sem_params {
  int64_t p, n;       /* variables, samples */
  int graph;          /* hpc_graph_kind */
  double degree;      /* ER: expected degree (edge probability degree/(p-1)) */
  int pa_parents;     /* PA: parents per new node */
  double w_lo, w_hi;  /* |weight| ~ U[w_lo, w_hi], random sign */
  uint64_t seed;
} hpc_sem_params;
/* X (n x p column-major, FP64) and/or X32 (FP32 copy); dag (p x p, parent->child)
 * and weights (p x p) optional; any output may be NULL. */
hpc_status hpc_sem_generate(const hpc_sem_params *prm, double *X, float *X32, uint8_t *dag,
                            double *weights);

#ifdef __cplusplus
}
#endif
#endif /* HETEROGPC_H */
