// Level 0 and the per-level adjacency snapshot.
//
// The live adjacency is a symmetric bitmask, p rows of W = ceil(p/32) words
// (the reference keeps an int32 p x p matrix, src/util/state.cu:21-29).
//
// level0_lower + mirror_bits replace testRowL0 (src/executor/testing/gpuRowTests.cu:4-27)
// / testRowL0Triangluar (src/executor/testing/cpuRowTests.cpp:5-21): every pair
// i > j is tested once on cor[i][j] (the lower-triangle entry the reference reads),
// the kept bits are written for the lower triangle and then mirrored by 32 x 32
// bit-tile transposes.
//
// degrees + scan_rows + fill_csr replace compactCUTiled (src/independence/compact.cu:4-89):
// per-row popcounts, one block-wide scan over rows for the CSR offsets and for the
// number of CI tests each row contributes at the level (d_i * C(d_i - 1, l)), and a
// warp-per-row ballot/scan that writes the ascending neighbour ids.
#include <cuda_runtime.h>

#include <algorithm>

#include "internal.cuh"
#include "stats.cuh"

namespace hpc {
namespace {

// one thread per (row, word): 32 decisions on cor64[i][32w .. 32w+31], j < i only
__global__ void level0_lower_kernel(LevelArgs a, double r_lo, double r_hi) {
  const int64_t total = a.p * (int64_t)a.W;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / a.W;
    const int w = (int)(t % a.W);
    const int64_t j0 = (int64_t)w * 32;
    uint32_t bits = 0;
    if (j0 < i) {
      const double *row = a.cor64 + i * a.p;
      const int jend = (i - j0) < 32 ? (int)(i - j0) : 32;
      for (int b = 0; b < jend; ++b) {
        const double v = row[j0 + b];
        const double av = fabs(v);
        bool remove;
        if (isnan(v) || av < r_lo)
          remove = true;          // p certainly >= alpha (NaN r is treated as 0)
        else if (av > r_hi)
          remove = false;         // p certainly < alpha
        else
          remove = calc_pvalue64(v, a.n_obs) >= a.alpha;  // exact reference formula
        if (!remove) bits |= 1u << b;
      }
    }
    a.adj[t] = bits;
  }
}

// Level 0 on the FP32 correlation of the tensor-core mode (no FP64 matrix): pairs
// clear of the band [lo, hi] around r_crit are decided here; pairs inside it, and
// non-finite ones, are queued for the FP64 re-test kernel, which sets the kept bits
// (inline serial dot product only when the queue is full).
__global__ void level0_lower_f32_kernel(LevelArgs a, float lo, float hi) {
  const int64_t total = a.p * (int64_t)a.W;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / a.W;
    const int w = (int)(t % a.W);
    const int64_t j0 = (int64_t)w * 32;
    uint32_t bits = 0;
    if (j0 < i) {
      const float *row = a.cor32 + i * a.p;
      const int jend = (i - j0) < 32 ? (int)(i - j0) : 32;
      for (int b = 0; b < jend; ++b) {
        const float av = fabsf(row[j0 + b]);
        if (av < lo) continue;             // removed
        if (av > hi) {                     // kept
          bits |= 1u << b;
          continue;
        }
        const int64_t j = j0 + b;          // in the band, or NaN
        const unsigned long long slot = atomicAdd(&a.ctr->rq_count, 1ull);
        if ((long long)slot < a.rq_cap) {
          RetestItem *it = a.rq + slot;
          it->i = (int32_t)i;
          it->j = (int32_t)j;
          it->level = 0;
          it->pad = 0;
        } else {
          const double *x = a.Z + i * a.n_z, *y = a.Z + j * a.n_z;
          double s = 0.0;
          for (int64_t k = 0; k < a.n_z; ++k) s = fma(x[k], y[k], s);
          if (!(calc_pvalue64(s / a.denom, a.n_obs) >= a.alpha)) bits |= 1u << b;
        }
      }
    }
    a.adj[t] = bits;
  }
}

// Mirror the lower triangle into the upper: warp per 32x32 bit tile (I, w) with w <= I.
__global__ void mirror_bits_kernel(uint32_t *adj, int64_t p, int W) {
  const int lane = threadIdx.x & 31;
  const int64_t nt = (int64_t)W * (W + 1) / 2;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t t = warp; t < nt; t += nwarps) {
    // t -> (I, w), w <= I, row-major over the lower triangle of tiles
    int64_t I = (int64_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while (I * (I + 1) / 2 > t) --I;
    while ((I + 1) * (I + 2) / 2 <= t) ++I;
    const int64_t w = t - I * (I + 1) / 2;
    const int64_t row = I * 32 + lane;
    uint32_t word = row < p ? adj[row * W + w] : 0u;
    // transposed[c] (held by lane c) = bits of column 32w + c over rows 32I .. 32I+31
    uint32_t tr = 0;
    for (int c = 0; c < 32; ++c) {
      uint32_t b = __ballot_sync(0xffffffffu, (word >> c) & 1u);
      if (lane == c) tr = b;
    }
    const int64_t trow = w * 32 + lane;
    if (I == w) {
      // diagonal tile: symmetric union within the same words
      if (row < p) adj[row * W + w] = word | tr;
    } else if (trow < p) {
      adj[trow * W + I] = tr;
    }
  }
}

__global__ void degrees_kernel(const uint32_t *__restrict__ adj, int64_t p, int W, int *__restrict__ deg) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = warp; i < p; i += nwarps) {
    int c = 0;
    for (int w = lane; w < W; w += 32) c += __popc(adj[i * W + w]);
    c = __reduce_add_sync(0xffffffffu, c);
    if (lane == 0) deg[i] = c;
  }
}

constexpr int kScanThreads = 1024;

// Single block: exclusive prefixes of degrees (CSR offsets) and of per-row test
// counts, plus the level summary in ctr.
__global__ void __launch_bounds__(kScanThreads) scan_rows_kernel(int64_t p, int level, const int *__restrict__ deg,
                                                                 int *__restrict__ rowptr,
                                                                 unsigned long long *__restrict__ row_work,
                                                                 DevCounters *ctr, DevGlobal *g) {
  __shared__ unsigned long long s_deg[kScanThreads];
  __shared__ unsigned long long s_work[kScanThreads];
  __shared__ int s_max[kScanThreads / 32];
  __shared__ int s_rows[kScanThreads / 32];
  __shared__ int s_over;
  const int tid = threadIdx.x;
  const int64_t per = (p + kScanThreads - 1) / kScanThreads;
  const int64_t lo = tid * per, hi = (lo + per) < p ? (lo + per) : p;
  if (tid == 0) s_over = 0;
  unsigned long long sd = 0, sw = 0;
  int mx = 0, rows = 0;
  bool over = false;
  for (int64_t i = lo; i < hi; ++i) {
    int d = deg[i];
    sd += (unsigned long long)d;
    mx = max(mx, d);
    if (level >= 1 && d - 1 >= level) {
      unsigned long long c = binom_sat(d - 1, level);
      unsigned long long w = (unsigned long long)d * c;
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
  if ((tid & 31) == 0) { s_max[tid >> 5] = mx; s_rows[tid >> 5] = rows; }
  if (over) atomicOr(&s_over, 1);
  __syncthreads();
  // Hillis-Steele inclusive scan over the 1024 partial sums
  for (int off = 1; off < kScanThreads; off <<= 1) {
    unsigned long long a = tid >= off ? s_deg[tid - off] : 0ull;
    unsigned long long b = tid >= off ? s_work[tid - off] : 0ull;
    __syncthreads();
    s_deg[tid] += a;
    s_work[tid] += b;
    __syncthreads();
  }
  unsigned long long bd = tid > 0 ? s_deg[tid - 1] : 0ull;
  unsigned long long bw = tid > 0 ? s_work[tid - 1] : 0ull;
  for (int64_t i = lo; i < hi; ++i) {
    rowptr[i] = (int)bd;
    row_work[i] = bw;
    int d = deg[i];
    bd += (unsigned long long)d;
    if (level >= 1 && d - 1 >= level) bw += (unsigned long long)d * binom_sat(d - 1, level);
  }
  if (tid == kScanThreads - 1) {
    rowptr[p] = (int)s_deg[kScanThreads - 1];
    row_work[p] = s_work[kScanThreads - 1];
  }
  if (tid == 0) {
    ctr->edges2 = s_deg[kScanThreads - 1];
    ctr->work_total = s_work[kScanThreads - 1];
    int m = 0, r = 0;
    for (int w = 0; w < kScanThreads / 32; ++w) { m = max(m, s_max[w]); r += s_rows[w]; }
    ctr->max_deg = m;
    ctr->rows = r;
    if (s_over) {
      atomicOr(&g->err, kErrWorkOverflow);
      ctr->work_total = 0;  // nothing of this level runs
    }
    ctr->tile_next = 0;
    ctr->tests = 0;
    ctr->retests = 0;
    ctr->deleted = 0;
    ctr->band_violations = 0;
    ctr->rec_begin = g->rec_count;
  }
}

__global__ void fill_csr_kernel(const uint32_t *__restrict__ adj, int64_t p, int W, const int *__restrict__ rowptr,
                                int *__restrict__ colidx, long long cap, DevCounters *ctr, DevGlobal *g) {
  const int lane = threadIdx.x & 31;
  if ((long long)ctr->edges2 > cap) {
    // the neighbour-list buffer is too small for this level: flag it, test nothing
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      atomicOr(&g->err, kErrCsrOverflow);
      ctr->work_total = 0;
    }
    return;
  }
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = warp; i < p; i += nwarps) {
    int base = rowptr[i];
    for (int w0 = 0; w0 < W; w0 += 32) {
      const int w = w0 + lane;
      uint32_t word = w < W ? adj[i * W + w] : 0u;
      int c = __popc(word);
      int incl = c;
      for (int o = 1; o < 32; o <<= 1) {
        int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
      }
      int pos = base + incl - c;
      while (word) {
        int b = __ffs(word) - 1;
        colidx[pos++] = w * 32 + b;
        word &= word - 1;
      }
      base += __shfl_sync(0xffffffffu, incl, 31);
    }
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

}  // namespace

hpc_status launch_expand_adjacency(const uint32_t *adj, int64_t p, int W, uint8_t *out, cudaStream_t s) {
  const int64_t total = p * p;
  int blocks = (int)std::min<int64_t>((total / 4 + 255) / 256 + 1, 152 * 32);
  expand_adjacency_kernel<<<blocks, 256, 0, s>>>(adj, p, W, out);
  HPC_LAUNCH_CHECK("expand_adjacency_kernel");
  return HPC_OK;
}

hpc_status launch_level0(const LevelArgs &a, double r_lo, double r_hi, cudaStream_t s) {
  const int64_t total = a.p * (int64_t)a.W;
  int blocks = (int)std::min<int64_t>((total + 255) / 256, 152 * 32);
  level0_lower_kernel<<<blocks, 256, 0, s>>>(a, r_lo, r_hi);
  HPC_LAUNCH_CHECK("level0_lower_kernel");
  const int64_t tiles = (int64_t)a.W * (a.W + 1) / 2;
  int mblocks = (int)std::min<int64_t>((tiles + 7) / 8, 152 * 32);
  mirror_bits_kernel<<<mblocks, 256, 0, s>>>(a.adj, a.p, a.W);
  HPC_LAUNCH_CHECK("mirror_bits_kernel");
  return HPC_OK;
}

hpc_status launch_level0_f32(const LevelArgs &a, float lo, float hi, cudaStream_t s) {
  const int64_t total = a.p * (int64_t)a.W;
  int blocks = (int)std::min<int64_t>((total + 255) / 256, 152 * 32);
  level0_lower_f32_kernel<<<blocks, 256, 0, s>>>(a, lo, hi);
  HPC_LAUNCH_CHECK("level0_lower_f32_kernel");
  return HPC_OK;
}

hpc_status launch_mirror(const LevelArgs &a, cudaStream_t s) {
  const int64_t tiles = (int64_t)a.W * (a.W + 1) / 2;
  int mblocks = (int)std::min<int64_t>((tiles + 7) / 8, 152 * 32);
  mirror_bits_kernel<<<mblocks, 256, 0, s>>>(a.adj, a.p, a.W);
  HPC_LAUNCH_CHECK("mirror_bits_kernel");
  return HPC_OK;
}

hpc_status launch_degrees(const LevelArgs &a, int *deg, cudaStream_t s) {
  int blocks = (int)std::min<int64_t>((a.p + 7) / 8, 152 * 16);
  degrees_kernel<<<blocks, 256, 0, s>>>(a.adj, a.p, a.W, deg);
  HPC_LAUNCH_CHECK("degrees_kernel");
  return HPC_OK;
}

hpc_status launch_scan(int64_t p, int level, const int *deg, int *rowptr, unsigned long long *row_work,
                       DevCounters *ctr, DevGlobal *g, cudaStream_t s) {
  scan_rows_kernel<<<1, kScanThreads, 0, s>>>(p, level, deg, rowptr, row_work, ctr, g);
  HPC_LAUNCH_CHECK("scan_rows_kernel");
  return HPC_OK;
}

hpc_status launch_fill_csr(const LevelArgs &a, int *colidx, cudaStream_t s) {
  int blocks = (int)std::min<int64_t>((a.p + 7) / 8, 152 * 16);
  fill_csr_kernel<<<blocks, 256, 0, s>>>(a.adj, a.p, a.W, a.rowptr, colidx, a.colidx_cap, a.ctr, a.gctr);
  HPC_LAUNCH_CHECK("fill_csr_kernel");
  return HPC_OK;
}

}  // namespace hpc
