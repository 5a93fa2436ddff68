// Internal declarations shared by the CUDA translation units of libheterogpc.
//
// A context holds `count` independent skeleton problems ("instances"; a plain
// context has one). Every device buffer is packed over the instances, and every
// level kernel runs once per level over all of them: its flattened index space is
// split by per-launch prefix sums (words, bit tiles, rows, CI tests) and each
// thread or warp finds its instance by binary search over the prefix.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

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

// Device counters of one instance and level.
struct DevCounters {
  unsigned long long tests;        // executed CI tests
  unsigned long long retests;      // tests re-run in FP64 (band, conditioning, non-finite)
  unsigned long long deleted;      // edges removed
  unsigned long long work_total;   // T_l of the instance
  unsigned long long edges2;       // sum of degrees at the level start
  unsigned long long rec_begin;    // first separation-set record of the level
  unsigned long long band_violations;  // FP32 removals the FP64 post-pass did not confirm
  int max_deg;                     // at the level start
  int rows;                        // rows with work at this level
};
// Instance-wide device counters.
struct DevGlobal {
  unsigned long long rec_count;    // separation-set records written (cumulative)
  // the neighbour-list snapshot: Inst::snap_epoch while every row's list in colidx
  // matches the adjacency except the rows marked in Inst::dirty, else 0 (set by the
  // scan phase after a rebuild, cleared by level 0 and by every counter reset)
  unsigned long long snap;
  int err;                         // error bits (kErr*)
  int pad;
};
// Counters of one level's launch over all instances.
struct LaunchCounters {
  unsigned long long tile_next;    // CI-test work-queue head
  unsigned long long rq_count;     // FP64 re-tests queued
  unsigned int scan_done;          // scan blocks finished (the last one forms the prefix)
  unsigned int bar;                // grid-barrier arrivals of the level kernel
  int max_deg;                     // largest degree at the level start over all instances
  int pad;
  // %globaltimer (ns) of the level kernel's phases: block 0 at entry, after the rebuild
  // and after the scan; the last block to finish its tests
  unsigned long long t_entry, t_rebuilt, t_scanned, t_end;
};

// Tile policy of a level's CI tests (set by the autotuner, else the defaults):
// tile_cap bounds the consecutive tests a lane takes per tile (the subset chunk),
// tiles_per_lane is the target number of tiles per lane of the grid (balance), and
// edge_lanes picks level 1's mapping: 32 = the warp's lanes interleaved over one
// edge's tests, 1 = each lane a chunk of consecutive tests (the mapping of the higher
// levels).
struct TuneEntry {
  int tile_cap, tiles_per_lane, edge_lanes, l1_prefetch;
};
// level-1 kernel variants: lanes interleaved over an edge, the same with the next
// position's entries loaded a step ahead, each lane a chunk of consecutive tests
constexpr int kL1Interleaved = 0, kL1Prefetch = 1, kL1Chunked = 2;
// kernel variant of levels 2-16 (mixed precision): the CI tests in the set order
// (citest.cuh) instead of the edge order (variant 0)
constexpr int kSetOrder = 3;
constexpr int kSetTop = 24;  // the highest level with a set-order kernel (unrolled for its level)
// flag on the level-1 variants kL1Interleaved / kL1Prefetch: undecided tests only
// queued (mixed precision without an FP64 matrix), as the set order does
constexpr int kQueueOnly = 8;
constexpr int kTuneDefaultCap = 64, kTuneDefaultTpl = 4, kTuneDefaultEdgeLanes = 32, kTuneMaxCap = 65536;
// table of a context: [p bucket][level][degree bucket]; bucket = bit length, capped
constexpr int kTunePB = 32, kTuneDB = 18;
__host__ __device__ __forceinline__ int tune_bucket(long long v, int cap) {
  int b = 0;
  while (v > 0 && b < cap - 1) {
    ++b;
    v >>= 1;
  }
  return b;
}
// Rows per segment of the level kernel's test-count scan, and the per-segment sums
// the rebuild phase accumulates (one slice of segments per level).
constexpr int kSegRows = 256;
struct SegAgg {
  unsigned long long deg;   // sum of degrees
  unsigned long long work;  // sum of tests per row
  unsigned long long sets;  // sum of conditioning sets per row (the units of the set order)
  int max_deg;
  int rows;                 // rows with tests
  int over;                 // a row's test count does not fit
  int pad;
};
constexpr int kErrRecOverflow = 1;
constexpr int kErrWorkOverflow = 2;
constexpr int kErrCsrOverflow = 4;
constexpr int kErrTimeout = 8;
constexpr int kErrBandViolation = 16;
constexpr int kErrRetestOverflow = 32;  // the set order found the re-test queue full: rerun in the edge order

// Separation-set records on the device, packed: a head (the removed edge i < j, the
// level and the p-value) and then the context's `rec_ids` separating-variable slots,
// at a stride of rec_stride_words(rec_ids) 32-bit words (even, so that every head's
// double is 8-byte aligned). rec_ids is the highest level the context runs, so a
// skeleton run to level 4 stores 40-byte records; they are expanded to
// hpc_sepset_record when read.
struct RecHead {
  int32_t i, j, level, pad;
  double pmax;
};
constexpr int kRecHeadWords = 6;
__host__ __device__ __forceinline__ int rec_stride_words(int rec_ids) { return kRecHeadWords + ((rec_ids + 1) & ~1); }

// One deferred FP64 re-test: edge (i, j) of instance `inst` given ids[0..level),
// or a level-0 pair (i > j).
struct RetestItem {
  int32_t i, j, level, inst;
  int32_t ids[HPC_MAX_LEVEL];
};

// One skeleton problem, as the kernels see it (device-resident table).
struct Inst {
  int64_t p;
  int W;                  // 32-bit words per adjacency row
  int n_obs;
  double alpha;
  // FP32 decision: |r| against r_c with a band margin_r + 8 * ke(l) / pivot,
  // ke(l) = ke_a + (l + 2) * ke_b
  float r_c, margin_r, ke_a, ke_b;
  double r_lo, r_hi;      // level 0 on FP64 entries: exact formula inside [r_lo, r_hi]
  float lo32, hi32;       // level 0 on FP32 entries: FP64 re-test inside [lo32, hi32]
  const double *cor64;    // p x p FP64 or null (tensor-core mode: entries from Z)
  const float *cor32;     // p x p FP32 (mixed modes) or null
  const double *Z;        // FP64 standardised data, n_z x p column-major, or null
  const float *zh, *zl;   // ... else the same values as FP32 pairs zh + zl (same layout)
  double *ec;             // FP64 entries the re-tests formed (p x p, entry (a, b) at min * p + max), or null
  uint32_t *ev;           // ... and which of them are there: bit ev_off + index of the context's bitmap
  int64_t ev_off;
  int64_t n_z;
  double denom;           // the Gram's divisor n - 1
  uint32_t *adj;          // live bitmask p x W
  int *deg;               // snapshot degrees (p)
  int *rowptr;            // snapshot CSR offsets (p + 1)
  int *colidx;            // snapshot neighbour ids, ascending per row
  long long colidx_cap;
  uint8_t *dirty;         // per row: nonzero when the row lost an edge since its list was extracted
  unsigned long long snap_epoch;  // nonzero; changes whenever the table (pointers, capacities) does
  unsigned long long *row_work;  // exclusive prefix of tests per row (p + 1)
  int32_t *recs;          // packed records (RecHead + rec_ids slots each)
  long long rec_cap;      // records
  int rec_ids, rec_stride;  // id slots per record, words per record
  DevCounters *ctr;       // [HPC_MAX_LEVEL + 1]
  DevGlobal *g;
};

// The re-tests' FP64 entries, kept per instance once formed (the same entries recur in
// the re-tests of one edge and of neighbouring conditioning sets): entry (a, b) at
// min * p + max, present when its bit is set. The value is stored, fenced, then the bit
// set; a reader that sees the bit fences before reading the value.
__device__ __forceinline__ bool ecache_get(const Inst &I, int64_t a, int64_t b, double *v) {
  if (!I.ec) return false;
  const int64_t idx = (a < b ? a : b) * I.p + (a < b ? b : a), bit = I.ev_off + idx;
  const uint32_t w = __ldcg(I.ev + (bit >> 5));
  if (!((w >> (bit & 31)) & 1u)) return false;
  __threadfence();
  *v = __ldcg(I.ec + idx);
  return true;
}
__device__ __forceinline__ void ecache_put(const Inst &I, int64_t a, int64_t b, double v) {
  if (!I.ec) return;
  const int64_t idx = (a < b ? a : b) * I.p + (a < b ? b : a), bit = I.ev_off + idx;
  __stcg(I.ec + idx, v);
  __threadfence();
  atomicOr(I.ev + (bit >> 5), 1u << (bit & 31));
}

// Sum over samples k = k0, k0 + step, ... < n of z_a[k] * z_b[k], the FP64-standardised
// variables a and b of one instance. From Z: FP64 FMAs. From the FP32 pairs: each
// product zh_a zh_b with its exact rounding error (fmaf) and the cross terms, summed
// with compensation (TwoSum) in FP32 and carried into FP64 every 16 samples -- about
// 2^-45 relative per block, and FP32 arithmetic instead of this GPU's 1/64-rate FP64.
__device__ __forceinline__ double zdot(const Inst &I, int64_t a, int64_t b, int64_t k0, int64_t step) {
  const int64_t n = I.n_z;
  double s = 0.0;
  if (I.Z) {
    const double *x = I.Z + a * n, *y = I.Z + b * n;
    for (int64_t k = k0; k < n; k += step) s = fma(x[k], y[k], s);
    return s;
  }
  const float *xh = I.zh + a * n, *xl = I.zl + a * n, *yh = I.zh + b * n, *yl = I.zl + b * n;
  // one block of up to 16 samples: products compensated into (sh, sl)
  auto add = [&](int64_t k, float &sh, float &sl) {
    const float ah = xh[k], al = xl[k], bh = yh[k], bl = yl[k];
    const float p = ah * bh;
    float e = fmaf(ah, bh, -p);
    e = fmaf(ah, bl, fmaf(al, bh, e));
    const float t = sh + p;
    const float bb = t - sh;
    sl += ((sh - (t - bb)) + (p - bb)) + e;
    sh = t;
  };
  int64_t k = k0;
  // full blocks: no bounds test inside, so that all 64 loads of a block issue before the
  // arithmetic that waits for them
  for (; k + 15 * step < n; k += 16 * step) {
    float sh = 0.f, sl = 0.f;
#pragma unroll
    for (int u = 0; u < 16; ++u) add(k + u * step, sh, sl);
    s += (double)sh + (double)sl;
  }
  float sh = 0.f, sl = 0.f;
  for (; k < n; k += step) add(k, sh, sl);
  return s + ((double)sh + (double)sl);
}

// One level's launch over all instances, passed by value.
struct Launch {
  const Inst *inst;
  int count;
  int level;
  const long long *word_prefix;     // adjacency words  sum p * W   (count + 1)
  const long long *tile_prefix;     // 32x32 bit tiles  sum W(W+1)/2 (count + 1)
  const long long *row_prefix;      // rows             sum p       (count + 1)
  unsigned long long *work_prefix;  // CI tests of this level       (count + 1), written by the scan
  LaunchCounters *lc;               // this level's
  RetestItem *rq;                   // deferred FP64 re-tests
  long long rq_cap;
  double *rq_val;                   // their entries, rq_vcap doubles of scratch (or null)
  unsigned int *rq_done;            // entries done per item (rq_cap, zero between launches)
  long long rq_vcap;
  const long long *seg_prefix;      // scan segments  sum ceil(p / kSegRows) (count + 1)
  SegAgg *seg;                      // this level's segment sums (zeroed before the level)
  int row_cache;                    // the CI tests keep the row offsets in shared memory
  long long total_rows, total_segs; // row_prefix[count], seg_prefix[count]
  const TuneEntry *tune;            // the context's tile-policy table (kTunePB x kLevels x kTuneDB)
  TuneEntry force;                  // tile_cap > 0: this policy for the level, whatever the table says
  int p_bucket;                     // tune_bucket of the largest p of the launch
  unsigned long long row_work_limit;  // a row with this many CI tests or more is a work overflow
                                      // (rows x limit < 2^63: the level's total fits)
  Inst inst0;                       // inst[0] by value: read from the parameter bank when count == 1
  unsigned long long wait_ns;       // bound of the grid barriers' waits (2 s)
  unsigned int bar_extra;           // arrivals added to the barrier target (0; tests raise it)
};

// Instance b's descriptor: the launch's parameter copy for a single instance (no
// memory round trip; kernels take the Launch as a __grid_constant__ parameter), else
// the device table.
__device__ __forceinline__ const Inst *inst_of(const Launch &L, int b) {
  return L.count == 1 ? &L.inst0 : L.inst + b;
}
// first and end rows / scan segments of instance b in the flattened spaces
__device__ __forceinline__ long long row_begin(const Launch &L, int b) { return L.count == 1 ? 0 : L.row_prefix[b]; }
__device__ __forceinline__ long long row_end(const Launch &L, int b) {
  return L.count == 1 ? L.total_rows : L.row_prefix[b + 1];
}
__device__ __forceinline__ long long seg_begin(const Launch &L, int b) { return L.count == 1 ? 0 : L.seg_prefix[b]; }
__device__ __forceinline__ long long seg_end(const Launch &L, int b) {
  return L.count == 1 ? L.total_segs : L.seg_prefix[b + 1];
}
// row offsets a level kernel of levels >= 2 caches in shared memory (one instance)
constexpr int kRowCache = 5120;

__device__ __forceinline__ int find_inst(const long long *prefix, int count, long long t) {
  int lo = 0, hi = count;  // largest b with prefix[b] <= t
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (prefix[mid] <= t) lo = mid; else hi = mid;
  }
  return lo;
}
__device__ __forceinline__ int find_inst_u(const unsigned long long *prefix, int count, unsigned long long t) {
  int lo = 0, hi = count;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (prefix[mid] <= t) lo = mid; else hi = mid;
  }
  return lo;
}

// ---------------------------------------------------------------------------
// host launchers (defined in the .cu files)
struct StdArgs {                    // grouped standardisation
  int count;
  const long long *row_prefix;      // variables (count + 1)
  const long long *x_off;           // element offset of each instance's observations
  const long long *z_off;           // element offset of each instance's Z
  const long long *n;               // samples per instance
  const long long *tc_off;          // element offset of each instance's split operands (or null)
  const long long *n_pad;           // padded samples per instance (tensor-core layout)
  const long long *kdim;            // K' per instance (tensor-core layout)
  int ref_compat;
};
// Outputs: Z (FP64), or with the split-BF16 planes P either Z or (FP32 samples) the
// FP32 pairs ZP (zh plane, then zl at + zp_plane elements).
hpc_status launch_standardise(const void *X, bool f32, const StdArgs &a, long long total_rows, double *Z,
                              float *ZP, long long zp_plane, __nv_bfloat16 *P, cudaStream_t s);
hpc_status launch_pair_to_f64(const float *zh, const float *zl, long long count, double *Z, cudaStream_t s);
struct GramArgs {                   // grouped FP64 Gram
  int count;
  const long long *tile_prefix;     // 64 x 64 upper-triangle tiles (count + 1)
  const long long *z_off, *c_off, *n, *p;
  const double *denom;
};
hpc_status launch_gram_f64(const double *Z, double *C, const GramArgs &a, long long total_tiles, cudaStream_t s);
long long gram_f64_tiles(int64_t p);
hpc_status launch_to_f32(const double *C, int64_t count, float *C32, cudaStream_t s);
int64_t tc_n_pad(int64_t n);
int64_t tc_p_pad(int64_t p);
int64_t tc_k(int64_t n);
long long gram_tc_tiles(int64_t p);
hpc_status tc_make_maps(CUtensorMap *mp, CUtensorMap *mq, const __nv_bfloat16 *P, const __nv_bfloat16 *Q,
                        int64_t p, int64_t n);
struct TcArgs {                     // grouped tensor-core Gram
  int count;
  const long long *tile_prefix;     // 128 x 128 upper-triangle tiles (count + 1)
  const CUtensorMap *maps;          // 2 per instance (P, Q), 64-byte aligned, device
  const long long *c_off, *p, *n;
  int *err;
};
hpc_status launch_gram_tc(float *C, const TcArgs &a, long long total_tiles, cudaStream_t s);
hpc_status tc_make_map(CUtensorMap *m, const __nv_bfloat16 *base, int64_t rows, int64_t K, int box_rows);
// FP64-accurate Gram on the tensor cores (gram_emu.cu): C64 (and C32 when not null) =
// Z^T Z / denom for one instance's standardised data Z (n x p, each variable
// contiguous). D (digits) and E (exponents) are its work buffers of emu_digit_elems /
// emu_p_pad elements.
bool emu_eligible(int64_t p, int64_t n);
int64_t emu_p_pad(int64_t p);
int64_t emu_digit_elems(int64_t p, int64_t n);
hpc_status launch_gram_emu(const double *Z, int64_t p, int64_t n, double denom, __nv_bfloat16 *D, int *E,
                           CUtensorMap *map_host_scratch, double *C64, float *C32, int *err, cudaStream_t s);

hpc_status launch_level0(const Launch &L, long long total_tiles, cudaStream_t s);
hpc_status launch_degrees(const Launch &L, long long total_rows, cudaStream_t s);
hpc_status launch_scan(const Launch &L, cudaStream_t s);
hpc_status launch_expand_adjacency(const uint32_t *adj, int64_t p, int W, uint8_t *out, cudaStream_t s);
// Level l >= 1 in one cooperative launch: snapshot rebuild, test-count scan, CI tests.
// l1_variant: level 1's kernel (kL1Interleaved, kL1Prefetch or kL1Chunked, from the tile policy).
hpc_status launch_level(const Launch &L, int precision, int grid, int l1_variant, cudaStream_t s);
hpc_status launch_retest(const Launch &L, int sms, cudaStream_t s);
void retest_setup();  // once per context creation, before any launch_retest
hpc_status launch_finalize_records(const Inst *inst, int count, cudaStream_t s);
// every instance's records packed back to back: instance b's first record goes to
// record slot prefix[b] of out (stride words each); prefix has count + 1 entries
hpc_status launch_gather_records(const Inst *inst, int count, const long long *prefix, long long total, int stride,
                                 int32_t *out, cudaStream_t s);
// every instance's records in the packed form of hpc_batch_get_records_packed
// one (instance, level) run of records for the packed copy (pack_records_kernel)
struct RecSegment {
  long long src;    // first record, within the instance
  long long count;  // records
  long long dst;    // first output word
  int inst, level;
};
hpc_status launch_pack_records(const Inst *inst, const RecSegment *seg, int nseg, int32_t *out, cudaStream_t s);
int citest_grid(int precision, int level, int device, int l1_variant = kL1Interleaved);

// process-wide tile-policy table (tune.cu)
TuneEntry tune_entry_of(const hpc_tune_params &p);
bool tune_params_valid(const hpc_tune_params *p);
void tune_snapshot(std::vector<TuneEntry> *out, long long *version);
long long tune_version();
void tune_store(int64_t p, int level, int max_degree, const TuneEntry &e);
TuneEntry tune_get(int p_bucket, int level, int deg_bucket);  // by bucket indices

// used by the server's shared launches (serve.cu): a context's neighbour-list and
// record buffers sized from its level-0 counters (ctr_host filled by the caller), and
// the bytes of the re-test queue a context of sum p^2 would hold
hpc_status ctx_size_after_level0(hpc_ctx *c);
long long ctx_retest_queue_bytes(long long sum_p2);
// entries of re-test scratch for a queue of `cap` items: three per item (a level-1
// re-test), at most 32 Mi
long long retest_scratch_entries(long long cap);
// The lowest level whose CI tests run in the set order (citest.cuh; 0: the edge order at
// every level), process-wide: kSetOrderFrom unless hpc_debug_set_order_from changed it.
// uses_set_order: whether a level runs in the set order, given the lowest set-order
// level in effect (0: none). The set order defers every undecided test to the FP64
// re-test queue, so it runs only where the re-tests are queued (no FP64 matrix).
constexpr int kSetOrderFrom = 3;
// ... and only where the level's largest degree fits the set order's 64-bit masks:
// wider rows (hubs) are where the edge order's early exit on removed edges pays most
constexpr int kSetDegMax = 64;
int set_order_from();
bool uses_set_order(int set_from, int level);

// per-instance host bookkeeping
struct InstHost {
  int64_t p = 0, n = 0;
  double alpha = 0.05, zc = 0.0, r_crit = 0.0;
  int W = 0;
  long long cor_off = 0, z_off = 0, x_off = 0, adj_off = 0, row_off = 0, tc_off = 0;
  long long colidx_off = 0, colidx_cap = 0, rec_off = 0, rec_cap = 0;
  int64_t edges = 0;
};

}  // namespace hpc

// ---------------------------------------------------------------------------
// The context (opaque to callers): `count` instances.
struct hpc_ctx {
  int count = 1;
  std::vector<hpc::InstHost> ih;
  int64_t p = 0, n = 0;           // instance 0 (the single-instance API)
  hpc_opts opts{};
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;  // the context's stream; `stream` may be a caller's
  // packed device buffers
  double *cor64 = nullptr;        // sum p^2 (absent in tensor-core mode unless loaded)
  float *cor32 = nullptr;         // sum p^2 (mixed modes)
  double *Z = nullptr;            // sum n * p
  bool z_valid = false;           // Z holds the current data's standardised values
  double *ecache = nullptr;       // FP64 entries formed by the re-tests, sum p^2 (tensor-core mode)
  uint32_t *evalid = nullptr;     // ... validity bits, cleared with every correlation
  long long evalid_words = 0;
  float *zpair = nullptr;         // the same as FP32 pairs (tensor-core mode, FP32 data): zh | zl planes
  bool zpair_valid = false;
  long long ztot = 0;             // sum n * p: the elements of one plane
  __nv_bfloat16 *tcP = nullptr;   // split-BF16 operands, sum p_pad * K'
  __nv_bfloat16 *emuD = nullptr;  // exact digit planes of the FP64-accurate tensor-core Gram
  int *emuE = nullptr;            // ... and the variables' exponents
  CUtensorMap *tc_maps = nullptr;  // device, 2 per instance
  void *X_stage = nullptr;        // device copy of host observations
  int64_t X_stage_bytes = 0;
  uint32_t *adj = nullptr;        // sum p * W
  uint8_t *adj_bytes = nullptr;   // p x p expansion for hpc_get_adjacency (largest p)
  int *deg = nullptr;             // sum p
  int *rowptr = nullptr;          // sum (p + 1)
  unsigned long long *row_work = nullptr;  // sum (p + 1)
  int *colidx = nullptr;          // sum colidx_cap
  long long colidx_total = 0;
  int32_t *recs = nullptr;       // packed records, sum rec_cap x rec_stride words
  long long rec_total = 0;        // words
  int rec_ids = HPC_MAX_LEVEL;    // id slots per record: the highest level the context runs
  hpc::RetestItem *rq = nullptr;
  long long rq_cap = 0;
  double *rq_val = nullptr;       // the re-tests' entries (scratch) and per-item done counters
  unsigned int *rq_done = nullptr;
  long long rq_vcap = 0;
  hpc::DevCounters *ctr = nullptr;       // count x (HPC_MAX_LEVEL + 1)
  hpc::DevCounters *ctr_host = nullptr;  // host mirror
  hpc::DevGlobal *gctr = nullptr;        // count
  hpc::DevGlobal *gctr_host = nullptr;
  hpc::LaunchCounters *lc = nullptr;     // HPC_MAX_LEVEL + 1
  hpc::LaunchCounters lc_host[HPC_MAX_LEVEL + 1] = {};  // host mirror (phase times of timed runs)
  uint8_t *row_dirty = nullptr;          // sum (p + 1): rows whose neighbour list is stale
  unsigned long long snap_epoch = 0;     // of the instance table last written
  hpc::Inst *inst = nullptr;             // device table (count)
  std::vector<hpc::Inst> inst_host;      // the table last written
  long long *prefixes = nullptr;         // device: word, tile, row, segment prefixes (4 x (count + 1))
  hpc::SegAgg *seg = nullptr;            // device: (HPC_MAX_LEVEL + 1) x total_segs
  long long total_segs = 0;
  unsigned long long *work_prefix = nullptr;  // device: (HPC_MAX_LEVEL + 1) x (count + 1)
  long long *meta = nullptr;             // device: correlation metadata arrays
  double *meta_denom = nullptr;
  long long total_words = 0, total_tiles = 0, total_rows = 0;
  long long tiles64 = 0, tiles_tc = 0;
  bool cor64_valid = false;       // cor64 holds the current FP64 matrices
  bool cor32_rounded = true;      // cor32 is the FP32 rounding of cor64 (else the tensor-core Gram)
  long long inst_version = 0;     // bumped whenever the device instance table changes
  // CUDA graph of the whole level sequence 0..graph_top
  cudaGraphExec_t graph = nullptr;
  int graph_top = -1;
  cudaStream_t graph_stream = nullptr;
  long long graph_version = -1;
  int64_t graph_launches = 0;
  bool graphs_enabled = true;
  bool last_run_graph = false;
  int citest_grid[HPC_MAX_LEVEL + 1] = {};
  // tile policy: device copy of the process-wide table, its version, a forced policy
  hpc::TuneEntry *tune_dev = nullptr;
  long long tune_version_dev = -1;
  hpc::TuneEntry tune_force{};
  int p_bucket = 0;
  int citest_grid_l1[3] = {};     // grids of the level-1 kernel variants (kL1*)
  int citest_grid_l1q[2] = {};    // ... and of the queue-only ones (kL1Interleaved, kL1Prefetch | kQueueOnly)
  int citest_grid_set[HPC_MAX_LEVEL + 1] = {};  // grids of the set-order kernels (levels 2-16)
  int l1_max_deg = -1;            // level-1 max degree of the last run (keys level 1's kernel choice)
  int l1v_now = 0;                // the level-1 kernel variant of the runs being queued
  int graph_l1v = 0;              // ... and of the captured graph
  unsigned int graph_set_mask = 0;  // the set-order levels of the captured graph (bit l)
  int deg_seen[HPC_MAX_LEVEL + 1];  // largest degree at each level's start in the last run (-1: unknown)
  bool set_off = false;           // the set order turned off (a re-test queue overflow)
  bool level_by_level = false;    // inside hpc_run_level: the edge order, inline re-tests on overflow
  bool graph_final = false;       // the captured graph ends with the record finalisation
  cudaEvent_t evc[4] = {nullptr, nullptr, nullptr, nullptr};  // correlation phases
  cudaEvent_t evl[HPC_MAX_LEVEL + 1][4] = {};  // per level: start, kernel start, re-tests done, kernel done
  cudaEvent_t evr[2] = {nullptr, nullptr};      // whole skeleton run
  bool cor_timed = false;
  hpc_timings timings{};
  bool have_cor = false;
  int next_level = 0;
  bool records_final = true;     // the records' FP32 p-values have been evaluated in FP64
  bool async_pending = false;    // an hpc_run_skeleton_async run not yet collected by hpc_wait
  unsigned long long wait_ns = 2000000000ull;  // grid-barrier wait bound of the level kernels
  unsigned int bar_extra = 0;    // test hook: arrivals added to the barrier target
  int async_top = -1;
  // runs "until exhausted" (max_level -1): the last level of the previous such run (its
  // first level without tests), so that the next run queues levels 0..exhaust_top as one
  // sequence (one graph replay, one sync) and only continues level by level if the data
  // now reach further; -1 before the first run
  int exhaust_top = -1;
  // whole-batch record retrieval: compacted copy of every instance's records
  int32_t *rec_stage = nullptr;
  long long rec_stage_words = 0;
  long long *rec_prefix_dev = nullptr;  // 2 x (count + 1): record and packed-word prefixes
  hpc::RecSegment *rec_seg = nullptr;  // segments of the packed record copy
  long long rec_seg_cap = 0;
};
