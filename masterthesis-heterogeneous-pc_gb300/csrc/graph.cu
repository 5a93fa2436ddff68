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

// One warp per 32 x 32 bit tile (I, w), w <= I, of the lower triangle: lane q decides
// the pairs (i, 32w + q) with j < i of the tile's 32 rows from the entries it reads
// (32 consecutive entries per row: coalesced; eight rows' loads in flight), each
// row's ballot is its word, and 32 more ballots transpose the tile, so that both
// triangles are written here (the diagonal tile as the union of the two).
__device__ __forceinline__ bool level0_keep(const Launch &L, const Inst &I, int b, int64_t i, int64_t j, double v64,
                                            float v32) {
  if (I.cor64) {
    // FP64 entries: the exact formula only inside [r_lo, r_hi]
    const double av = fabs(v64);
    if (isnan(v64) || av < I.r_lo) return false;  // p certainly >= alpha (NaN r is treated as 0)
    if (av > I.r_hi) return true;
    return !(calc_pvalue64(v64, I.n_obs) >= I.alpha);
  }
  // FP32 tensor-core entries: pairs inside the band (or NaN) are queued for the FP64
  // re-test kernel, which sets their kept bits
  const float av = fabsf(v32);
  if (av > I.hi32) return true;
  if (av < I.lo32) return false;
  const unsigned long long slot = atomicAdd(&L.lc->rq_count, 1ull);
  if ((long long)slot < L.rq_cap) {
    RetestItem *it = L.rq + slot;
    it->i = (int32_t)i;
    it->j = (int32_t)j;
    it->level = 0;
    it->inst = b;
    return false;
  }
  // queue full: serial FP64 dot product here
  const double *x = I.Z + i * I.n_z, *y = I.Z + j * I.n_z;
  double sum = 0.0;
  for (int64_t k = 0; k < I.n_z; ++k) sum = fma(x[k], y[k], sum);
  return !(calc_pvalue64(sum / I.denom, I.n_obs) >= I.alpha);
}

__global__ void level0_kernel(const __grid_constant__ Launch L, long long total) {
  const int lane = threadIdx.x & 31;
  const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long t = warp; t < total; t += nwarps) {
    const int b = find_inst(L.tile_prefix, L.count, t);
    const Inst &I = *inst_of(L, b);
    const long long lt = t - L.tile_prefix[b];
    // lt -> (TI, w), w <= TI, row-major over the lower triangle of tiles
    int64_t TI = (int64_t)((sqrt(8.0 * (double)lt + 1.0) - 1.0) * 0.5);
    while (TI * (TI + 1) / 2 > lt) --TI;
    while ((TI + 1) * (TI + 2) / 2 <= lt) ++TI;
    const int64_t w = lt - TI * (TI + 1) / 2;
    const int64_t j = w * 32 + lane;
    uint32_t word = 0;  // lane r: the word of row 32 TI + r
#pragma unroll
    for (int r0 = 0; r0 < 32; r0 += 8) {
      double v64[8];
      float v32[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int64_t i = TI * 32 + r0 + k;
        v64[k] = 0.0;
        v32[k] = 0.f;
        if (i < I.p && j < i) {
          if (I.cor64) v64[k] = I.cor64[i * I.p + j];
          else v32[k] = I.cor32[i * I.p + j];
        }
      }
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int64_t i = TI * 32 + r0 + k;
        const bool keep = i < I.p && j < i && level0_keep(L, I, b, i, j, v64[k], v32[k]);
        const uint32_t bits = __ballot_sync(0xffffffffu, keep);
        if (lane == r0 + k) word = bits;
      }
    }
    uint32_t tr = 0;  // lane c: the bits of column 32 w + c over the tile's rows
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

constexpr int kScanThreads = 512;

// One block per instance: exclusive prefixes of degrees (CSR offsets) and of per-row
// test counts, the instance's level summary; the last block to finish forms the
// prefix of test counts over instances (work_prefix) for the CI-test kernel.
__global__ void __launch_bounds__(kScanThreads) scan_kernel(const __grid_constant__ Launch L) {
  __shared__ unsigned long long s_deg[kScanThreads];
  __shared__ unsigned long long s_work[kScanThreads];
  __shared__ int s_max[kScanThreads / 32];
  __shared__ int s_rows[kScanThreads / 32];
  __shared__ int s_over;
  __shared__ bool s_last;
  const int b = blockIdx.x;
  const Inst &I = *inst_of(L, b);
  const int level = L.level;
  const int tid = threadIdx.x;
  const int64_t p = I.p;
  const int64_t per = (p + kScanThreads - 1) / kScanThreads;
  const int64_t lo = tid * per, hi = (lo + per) < p ? (lo + per) : p;
  if (tid == 0) s_over = 0;
  __syncthreads();
  unsigned long long sd = 0, sw = 0;
  int mx = 0, rows = 0;
  bool over = false;
  for (int64_t i = lo; i < hi; ++i) {
    const int d = I.deg[i];
    sd += (unsigned long long)d;
    mx = max(mx, d);
    if (level >= 1 && d - 1 >= level) {
      const unsigned long long c = binom_sat(d - 1, level);
      const unsigned long long w = (unsigned long long)d * c;
      if (c == 0xFFFFFFFFFFFFFFFFull || w / (unsigned long long)d != c || sw + w < sw) over = true;
      sw += w;
      ++rows;
    }
  }
  s_deg[tid] = sd;
  s_work[tid] = sw;
  for (int o = 16; o > 0; o >>= 1) {
    mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    rows += __shfl_xor_sync(0xffffffffu, rows, o);
  }
  if ((tid & 31) == 0) {
    s_max[tid >> 5] = mx;
    s_rows[tid >> 5] = rows;
  }
  if (over) atomicOr(&s_over, 1);
  __syncthreads();
  for (int off = 1; off < kScanThreads; off <<= 1) {  // Hillis-Steele inclusive scan
    const unsigned long long x = tid >= off ? s_deg[tid - off] : 0ull;
    const unsigned long long y = tid >= off ? s_work[tid - off] : 0ull;
    __syncthreads();
    s_deg[tid] += x;
    s_work[tid] += y;
    __syncthreads();
  }
  unsigned long long bd = tid > 0 ? s_deg[tid - 1] : 0ull;
  unsigned long long bw = tid > 0 ? s_work[tid - 1] : 0ull;
  for (int64_t i = lo; i < hi; ++i) {
    I.rowptr[i] = (int)bd;
    I.row_work[i] = bw;
    const int d = I.deg[i];
    bd += (unsigned long long)d;
    if (level >= 1 && d - 1 >= level) bw += (unsigned long long)d * binom_sat(d - 1, level);
  }
  if (tid == 0) {
    DevCounters &C = I.ctr[level];
    const unsigned long long e2 = s_deg[kScanThreads - 1];
    unsigned long long work = s_work[kScanThreads - 1];
    I.rowptr[p] = (int)e2;
    I.row_work[p] = work;
    int m = 0, r = 0;
    for (int w = 0; w < kScanThreads / 32; ++w) {
      m = max(m, s_max[w]);
      r += s_rows[w];
    }
    if (s_over) {
      atomicOr(&I.g->err, kErrWorkOverflow);
      work = 0;  // nothing of this level runs for the instance
    }
    if (level >= 1 && (long long)e2 > I.colidx_cap) {
      atomicOr(&I.g->err, kErrCsrOverflow);  // neighbour lists do not fit: resized by the host
      work = 0;
    }
    C.edges2 = e2;
    C.work_total = work;
    C.max_deg = m;
    C.rows = r;
    C.tests = 0;
    C.retests = 0;
    C.deleted = 0;
    C.band_violations = 0;
    C.rec_begin = I.g->rec_count;
    __threadfence();
    const unsigned int done = atomicAdd(&L.lc->scan_done, 1u);
    s_last = done == (unsigned int)L.count - 1;
  }
  __syncthreads();
  if (s_last && tid == 0) {
    // last block: the prefix of the instances' test counts (the other blocks'
    // counters are visible after their fence and this block's atomic)
    __threadfence();
    unsigned long long acc = 0;
    for (int q = 0; q < L.count; ++q) {
      L.work_prefix[q] = acc;
      acc += *(volatile unsigned long long *)&inst_of(L, q)->ctr[level].work_total;
    }
    L.work_prefix[L.count] = acc;
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
  level0_kernel<<<blocks_for(total_tiles, 8), 256, 0, s>>>(L, total_tiles);
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
