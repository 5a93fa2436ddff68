// Level 0 and the per-level adjacency snapshot, over all instances of a context.
//
// The live adjacency of an instance is a symmetric bitmask, p rows of W = ceil(p/32)
// words (the reference keeps an int32 p x p matrix, src/util/state.cu:21-29).
//
// level0 replaces testRowL0 (src/executor/testing/gpuRowTests.cu:4-27) /
// testRowL0Triangluar (src/executor/testing/cpuRowTests.cpp:5-21): every pair i > j
// is tested once on cor[i][j] (the lower-triangle entry the reference reads), a warp
// per 32 x 32 bit tile, which writes the tile and its transpose.
//
// degrees + scan after level 0: per-row popcounts, then one block per instance scans
// the degrees into the offsets of each row's slot in the neighbour-list buffer. The
// slots keep these sizes for the rest of the skeleton (degrees only fall); the level
// kernels of levels >= 1 refill them and count their CI tests themselves
// (rebuild.cuh).
#include <cuda_runtime.h>

#include <algorithm>

#include "internal.cuh"
#include "stats.cuh"

namespace hpc {
namespace {

// the rare cases of a level-0 decision (FP64 entry inside the guard band, FP32 entry
// inside the tensor-core band): out of line, so that the 32 unrolled decisions of a
// tile stay small
__device__ __noinline__ bool level0_keep_slow(const Launch &L, const Inst &I, int b, int64_t i, int64_t j, double v64) {
  if (I.cor64) return !(calc_pvalue64(v64, I.n_obs) >= I.alpha);
  const unsigned long long slot = atomicAdd(&L.lc->rq_count, 1ull);
  if ((long long)slot < L.rq_cap) {
    RetestItem *it = L.rq + slot;
    it->i = (int32_t)i;
    it->j = (int32_t)j;
    it->level = 0;
    it->inst = b;
    return false;  // the FP64 re-test kernel sets the kept bits
  }
  // queue full: serial FP64 dot product here
  return !(calc_pvalue64(zdot(I, i, j, 0, 1) / I.denom, I.n_obs) >= I.alpha);
}

__device__ __forceinline__ bool level0_keep(const Launch &L, const Inst &I, int b, int64_t i, int64_t j, double v64,
                                            float v32) {
  if (I.cor64) {
    // FP64 entries: the exact formula only inside [r_lo, r_hi]
    const double av = fabs(v64);
    if (isnan(v64) || av < I.r_lo) return false;  // p certainly >= alpha (NaN r is treated as 0)
    if (av > I.r_hi) return true;
    return level0_keep_slow(L, I, b, i, j, v64);
  }
  // FP32 tensor-core entries: pairs inside the band (or NaN) are re-tested in FP64
  const float av = fabsf(v32);
  if (av > I.hi32) return true;
  if (av < I.lo32) return false;
  return level0_keep_slow(L, I, b, i, j, 0.0);
}

// One 4-warp block per 32 x 32 bit tile (TI, w), w <= TI, of the lower triangle: warp
// q decides rows 8q..8q+7 of the tile -- lane c the pairs (i, 32w + c) with j < i, from
// the entries it reads (32 consecutive entries per row: coalesced; the eight rows'
// loads issued together) -- and each row's ballot is its word; warp 0 then transposes
// the tile with 32 more ballots and writes both triangles (the diagonal tile as the
// union of the two).
// A block takes a contiguous run of tiles: the instance is searched once per run (and
// where the run crosses into the next instance), and the tile coordinates step along
// the row-major order instead of being recomputed by a square root per tile.
constexpr int kL0Threads = 128;
__global__ void __launch_bounds__(kL0Threads) level0_kernel(const __grid_constant__ Launch L, long long total) {
  __shared__ uint32_t s_word[32];
  const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
  const long long per = (total + gridDim.x - 1) / gridDim.x;
  const long long t0 = blockIdx.x * per, t1 = min(t0 + per, total);
  int b = -1;
  long long tb1 = 0;     // first tile of the next instance
  int64_t TI = 0, w = 0;  // (TI, w), w <= TI: the tile, row-major over the lower triangle of tiles
  for (long long t = t0; t < t1; ++t) {
    if (b < 0 || t >= tb1) {
      b = L.count == 1 ? 0 : find_inst(L.tile_prefix, L.count, t);
      const long long tb0 = L.count == 1 ? 0 : L.tile_prefix[b];
      tb1 = L.count == 1 ? total : L.tile_prefix[b + 1];
      const long long lt = t - tb0;
      // an FP32 estimate of the triangular root, corrected in integers
      TI = (int64_t)((sqrtf(8.0f * (float)lt + 1.0f) - 1.0f) * 0.5f);
      if (TI < 0) TI = 0;
      while (TI > 0 && TI * (TI + 1) / 2 > lt) --TI;
      while ((TI + 1) * (TI + 2) / 2 <= lt) ++TI;
      w = lt - TI * (TI + 1) / 2;
    } else if (++w > TI) {
      ++TI;
      w = 0;
    }
    const Inst &I = *inst_of(L, b);
    const int64_t j = w * 32 + lane;
    double v64[8];
    float v32[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int64_t i = TI * 32 + wq * 8 + k;
      v64[k] = 0.0;
      v32[k] = 0.f;
      if (i < I.p && j < i) {
        if (I.cor64) v64[k] = I.cor64[i * I.p + j];
        else v32[k] = I.cor32[i * I.p + j];
      }
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int64_t i = TI * 32 + wq * 8 + k;
      const bool keep = i < I.p && j < i && level0_keep(L, I, b, i, j, v64[k], v32[k]);
      const uint32_t bits = __ballot_sync(0xffffffffu, keep);
      if (lane == 0) s_word[wq * 8 + k] = bits;
    }
    __syncthreads();
    if (wq == 0) {
      const uint32_t word = s_word[lane];  // the word of row 32 TI + lane
      uint32_t tr = 0;                     // lane c: the bits of column 32 w + c
      for (int c = 0; c < 32; ++c) {
        const uint32_t bb = __ballot_sync(0xffffffffu, (word >> c) & 1u);
        if (lane == c) tr = bb;
      }
      const int W = I.W;
      const int64_t row = TI * 32 + lane, trow = w * 32 + lane;
      if (TI == w) {
        if (row < I.p) I.adj[row * W + w] = word | tr;
      } else {
        if (row < I.p) I.adj[row * W + w] = word;
        if (trow < I.p) I.adj[trow * W + TI] = tr;
      }
    }
    __syncthreads();
  }
}

__global__ void degrees_kernel(const __grid_constant__ Launch L, long long total) {
  const int lane = threadIdx.x & 31;
  const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long t = warp; t < total; t += nwarps) {
    const int b = find_inst(L.row_prefix, L.count, t);
    const Inst &I = *inst_of(L, b);
    const int64_t i = t - L.row_prefix[b];
    int c = 0;
    for (int w = lane; w < I.W; w += 32) c += __popc(I.adj[i * I.W + w]);
    c = __reduce_add_sync(0xffffffffu, c);
    if (lane == 0) I.deg[i] = c;
  }
}

constexpr int kScanThreads = 1024;

// After level 0, one block per instance: the exclusive prefix of the degrees, i.e. the
// offset of each row's slot in the neighbour-list buffer (kept for the rest of the
// skeleton), and the instance's level-0 summary. Warp-shuffle scan; level 0 has no CI
// tests, so the test counts and their prefix are zero.
__global__ void __launch_bounds__(kScanThreads) scan_kernel(const __grid_constant__ Launch L) {
  __shared__ unsigned long long s_warp[kScanThreads / 32];
  __shared__ int s_max[kScanThreads / 32];
  const int b = blockIdx.x;
  const Inst &I = *inst_of(L, b);
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int64_t p = I.p;
  const int64_t per = (p + kScanThreads - 1) / kScanThreads;
  const int64_t lo = tid * per, hi = (lo + per) < p ? (lo + per) : p;
  unsigned long long sd = 0;
  int mx = 0;
  for (int64_t i = lo; i < hi; ++i) {
    const int d = I.deg[i];
    sd += (unsigned long long)d;
    mx = max(mx, d);
  }
  unsigned long long incl = sd;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long x = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += x;
  }
  mx = __reduce_max_sync(0xffffffffu, mx);
  if (lane == 31) s_warp[wid] = incl;
  if (lane == 0) s_max[wid] = mx;
  __syncthreads();
  if (wid == 0) {  // scan of the warp totals
    unsigned long long v = s_warp[lane], iv = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long x = __shfl_up_sync(0xffffffffu, iv, o);
      if (lane >= o) iv += x;
    }
    s_warp[lane] = iv - v;  // exclusive
    const int m = __reduce_max_sync(0xffffffffu, s_max[lane]);
    if (lane == 31) {
      // level-0 summary of the instance
      DevCounters &C = I.ctr[0];
      const unsigned long long e2 = iv;
      I.rowptr[p] = (int)e2;
      I.row_work[p] = 0;
      C.edges2 = e2;
      C.work_total = 0;
      C.max_deg = m;
      C.rows = 0;
      C.tests = 0;
      C.retests = 0;
      C.deleted = 0;
      C.band_violations = 0;
      C.rec_begin = I.g->rec_count;
      I.g->snap = 0;  // a new CSR layout: every neighbour list is extracted at level 1
      L.work_prefix[b] = 0;
      if (b == L.count - 1) L.work_prefix[L.count] = 0;
    }
  }
  __syncthreads();
  unsigned long long bd = s_warp[wid] + incl - sd;
  for (int64_t i = lo; i < hi; ++i) {
    I.rowptr[i] = (int)bd;
    I.row_work[i] = 0;
    bd += (unsigned long long)I.deg[i];
  }
}

// p x p bytes (1 = edge) from the bitmask, 4 bytes per thread
__global__ void expand_adjacency_kernel(const uint32_t *__restrict__ adj, int64_t p, int W, uint8_t *__restrict__ out) {
  const int64_t total = p * p;
  for (int64_t t = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) * 4; t < total;
       t += (int64_t)gridDim.x * blockDim.x * 4) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int64_t e = t + k;
      if (e < total) {
        const int64_t i = e / p, j = e - i * p;
        out[e] = (uint8_t)((adj[i * W + (j >> 5)] >> (j & 31)) & 1u);
      }
    }
  }
}

int blocks_for(long long items, int per_block) {
  return (int)std::max<long long>(1, std::min<long long>((items + per_block - 1) / per_block, 152LL * 32));
}

}  // namespace

hpc_status launch_level0(const Launch &L, long long total_tiles, cudaStream_t s) {
  const int blocks = (int)std::max<long long>(1, std::min<long long>(total_tiles, 152LL * 16 * 8));
  level0_kernel<<<blocks, kL0Threads, 0, s>>>(L, total_tiles);
  HPC_LAUNCH_CHECK("level0_kernel");
  return HPC_OK;
}

hpc_status launch_degrees(const Launch &L, long long total, cudaStream_t s) {
  degrees_kernel<<<blocks_for(total, 8), 256, 0, s>>>(L, total);
  HPC_LAUNCH_CHECK("degrees_kernel");
  return HPC_OK;
}

hpc_status launch_scan(const Launch &L, cudaStream_t s) {
  scan_kernel<<<L.count, kScanThreads, 0, s>>>(L);
  HPC_LAUNCH_CHECK("scan_kernel");
  return HPC_OK;
}

hpc_status launch_expand_adjacency(const uint32_t *adj, int64_t p, int W, uint8_t *out, cudaStream_t s) {
  const int64_t total = p * p;
  expand_adjacency_kernel<<<blocks_for(total / 4 + 1, 256), 256, 0, s>>>(adj, p, W, out);
  HPC_LAUNCH_CHECK("expand_adjacency_kernel");
  return HPC_OK;
}

}  // namespace hpc
