// Level-l CI tests (l >= 1): the re-test and record kernels, the level-kernel
// instantiations of levels 1-8 and the launchers (the level kernels' device code is in
// citest.cuh).
#include <algorithm>

#include "citest.cuh"

namespace hpc {
namespace {

// p-values of the removals decided in FP32 (negative pmax), for every instance's
// records: FP64 re-evaluation where the instance has an FP64 matrix -- a result below
// alpha flags kErrBandViolation (the FP32 error bound did not hold) -- else the formula
// in FP32 on the stored FP32 |r|. Run at the end of every skeleton run. The instances
// run side by side, a group of gridDim / count blocks (at least one) each: taking them
// one after another over the whole grid cost a chain of dependent loads per instance
// (0.8 ms for a batch of 512 instances of p 20-800).
__global__ void finalize_records_kernel(const Inst *__restrict__ inst, int count) {
  if (count <= 0) return;
  const unsigned per = max(1u, gridDim.x / (unsigned)count);  // blocks per instance
  const unsigned groups = gridDim.x / per;
  const unsigned long long tid = (blockIdx.x % per) * (unsigned long long)blockDim.x + threadIdx.x;
  const unsigned long long nthreads = (unsigned long long)per * blockDim.x;
  for (int b = (int)(blockIdx.x / per); b < count; b += (int)groups) {
    const Inst &I = inst[b];
    unsigned long long end = I.g->rec_count;
    if (end > (unsigned long long)I.rec_cap) end = (unsigned long long)I.rec_cap;
    for (unsigned long long r = tid; r < end; r += nthreads) {
      int32_t *rec = I.recs + r * (unsigned long long)I.rec_stride;
      RecHead *h = reinterpret_cast<RecHead *>(rec);
      if (!(h->pmax < 0.0)) continue;
      if (!I.cor64) {
        h->pmax = (double)calc_pvalue32((float)(-1.0 - h->pmax), I.n_obs);
        continue;
      }
      // level 1: the closed form from the three entries (what exact_pvalue evaluates
      // there, without its matrix in local memory); else the general path, its arrays
      // sized by the level
      double pv;
      const int l = h->level;
      if (l == 1) {
        const int64_t k = rec[kRecHeadWords];
        pv = pval_l1_64(I.cor64[h->i * I.p + h->j], I.cor64[h->i * I.p + k], I.cor64[h->j * I.p + k], I.n_obs);
      } else {
        pv = l <= 16 ? exact_pvalue<16>(I, h->i, h->j, rec + kRecHeadWords, l)
                     : exact_pvalue<HPC_MAX_LEVEL>(I, h->i, h->j, rec + kRecHeadWords, l);
      }
      h->pmax = pv;
      if (!(pv >= I.alpha)) atomicOr(&I.g->err, kErrBandViolation);
    }
  }
}

// Records of all instances compacted into one buffer: one warp per record, its
// words copied by the lanes (record r of the output belongs to the instance b with
// prefix[b] <= r < prefix[b + 1]).
__global__ void gather_records_kernel(const Inst *__restrict__ inst, int count, const long long *__restrict__ prefix,
                                      long long total, int stride, int32_t *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long r = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; r < total; r += nw) {
    const int b = find_inst(prefix, count, r);
    const int32_t *src = inst[b].recs + (r - prefix[b]) * (long long)stride;
    for (int w = lane; w < stride; w += 32) out[r * (long long)stride + w] = src[w];
  }
}

// Records of all instances in the packed form of hpc_batch_get_records_packed. The host
// cuts them into segments, one per (instance, level) with removals: an instance's
// records are appended level by level, so a segment is a contiguous run of `count`
// records from record `src` of instance `inst` (rec_stride words each), and it goes to
// the contiguous words from `dst`, w = 6 + 2 ceil(l / 2) words per record (head, l ids,
// -1 padding). One block per segment, its threads over the segment's output words
// (coalesced writes, no per-record search).
__global__ void pack_records_kernel(const Inst *__restrict__ inst, const RecSegment *__restrict__ seg, int nseg,
                                    int32_t *__restrict__ out) {
  for (int g = blockIdx.x; g < nseg; g += gridDim.x) {
    const RecSegment S = seg[g];
    const Inst &I = inst[S.inst];
    const int l = S.level;
    const int w = 6 + ((l + 1) & ~1);
    const long long words = S.count * (long long)w;
    const int32_t *src = I.recs + S.src * (long long)I.rec_stride;
    int32_t *dst = out + S.dst;
    for (long long t = threadIdx.x; t < words; t += blockDim.x) {
      const long long r = t / w;
      const int q = (int)(t - r * w);
      dst[t] = q < 6 + l ? src[r * I.rec_stride + q] : -1;
    }
  }
}

__device__ __forceinline__ double warp_dot(const Inst &I, int64_t a, int64_t b) {
  const int lane = threadIdx.x & 31;
  double s = zdot(I, a, b, lane, 32);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  return s;
}

// FP64 re-tests deferred by the level kernels (instances without an FP64 matrix). A
// re-test of level l needs the E = (l + 2)(l + 1) / 2 FP64 correlation entries among
// i, j and S, each a dot product of two FP64-standardised columns (n samples). One warp
// per dot product: the launch's first W items (W = min(queued, rq_vcap / E)) are cut
// into W * E (item, entry) units over the grid, each warp writes its entry to the item's
// scratch row and counts it done; the warp completing an item's last entry gathers the
// row into its (l + 2)^2 matrix in shared memory and lane 0 evaluates the reference
// formula. So a level with a few re-tests of many entries (the high levels) runs them
// side by side instead of one warp stepping through 100+ dot products; items beyond the
// scratch take a warp each. Level-0 items (one entry) set the kept bits of both
// triangles; level >= 1 items remove the edge. The done counters return to zero when
// their item is evaluated, ready for the next launch.
// KM: the highest level of the launch's items (16 for levels up to 16, HPC_MAX_LEVEL
// above), which sizes the FP64 fallback's local arrays.
constexpr int kRetestWarps = 8;

// the variable at position r of a re-test's matrix order (i, j, S)
__device__ __forceinline__ int64_t retest_var(const RetestItem *it, int r) {
  return r == 0 ? (int64_t)it->i : r == 1 ? (int64_t)it->j : (int64_t)it->ids[r - 2];
}

// entry e of the upper triangle of a k x k matrix, row by row: (r, c), r < c
__device__ __forceinline__ void entry_rc(int e, int k, int &r, int &c) {
  r = 0;
  while (e >= k - 1 - r) {
    e -= k - 1 - r;
    ++r;
  }
  c = r + 1 + e;
}

// lane 0: the FP64 decision of item it from its matrix M (k x k, warp-filled)
template <int KM>
__device__ __forceinline__ void retest_decide(const Launch &L, const Inst &I, const RetestItem *it, int l, double *M) {
  bool nan_p;
  const double r = partial_r_of_matrix<KM>(M, l, &nan_p);
  double pv;
  const int64_t i = it->i, j = it->j;
  if (decide_of_r(I, r, nan_p, &pv) && claim_edge(I, i, j)) write_record(I, L.level, i, j, it->ids, l, pv);
}

// Levels 1-4 (K = l + 2 <= 6 variables): one warp per item, every lane accumulating the
// E = K(K - 1) / 2 products over its samples (k = lane, lane + 32, ...) in passes of
// kRetestPass entries (the accumulators of a pass stay in registers), so that each of
// the K columns is read once per item instead of once per entry it takes part in (2E
// column reads in the entry-parallel form). Above level 4 the entry-parallel form is
// faster (measured on a batch of 512 instances of p 20-800: a re-test's 28-45 entries
// spread over as many warps beat one warp stepping through the columns, and the column
// form's registers halve occupancy). The products are
// summed as in zdot: the FP32 pairs' products with their exact rounding errors and cross
// terms, compensated in FP32 and carried into FP64 every 16 samples of a lane.
constexpr int kRetestPass = 16;
constexpr int kColumnTop = 4;  // the highest level re-tested by columns

// (r, c) of entry e of the upper triangle of a K x K matrix, row by row
__host__ __device__ constexpr int entry_row(int e, int K) {
  int r = 0;
  while (e >= K - 1 - r) {
    e -= K - 1 - r;
    ++r;
  }
  return r;
}
__host__ __device__ constexpr int entry_col(int e, int K) {
  int r = 0;
  while (e >= K - 1 - r) {
    e -= K - 1 - r;
    ++r;
  }
  return r + 1 + e;
}

// one pass: entries E0 .. E0 + EN - 1, written to the warp's matrix M (K x K) by lane 0
template <int K, int E0, int EN>
__device__ __forceinline__ void retest_columns_pass(const Inst &I, const float *const *ch, int64_t lo_off,
                                                    double *M) {
  const int lane = threadIdx.x & 31;
  const int64_t n = I.n_z;
  double acc[EN];
#pragma unroll
  for (int e = 0; e < EN; ++e) acc[e] = 0.0;
  for (int64_t k0 = lane; k0 < n; k0 += 32 * 16) {
    float sh[EN], sl[EN];
#pragma unroll
    for (int e = 0; e < EN; ++e) sh[e] = sl[e] = 0.f;
    // the products of one sample's loaded values
    auto add = [&](const float *ah, const float *al) {
      int e = 0;
#pragma unroll
      for (int r = 0; r < K; ++r)
#pragma unroll
        for (int c = r + 1; c < K; ++c, ++e) {
          if (e < E0 || e >= E0 + EN) continue;
          const int x = e - E0;
          const float p = ah[r] * ah[c];
          float er = fmaf(ah[r], ah[c], -p);
          er = fmaf(ah[r], al[c], fmaf(al[r], ah[c], er));
          const float t = sh[x] + p;
          const float bb = t - sh[x];
          sl[x] += ((sh[x] - (t - bb)) + (p - bb)) + er;
          sh[x] = t;
        }
    };
    // S samples at a time, all loaded before the arithmetic (no bounds test between):
    // the loop is bound by its round trips to memory, so a round trip carries as many
    // samples as the registers allow
    constexpr int S = K <= 4 ? 8 : K == 5 ? 4 : 2;
#pragma unroll 1
    for (int u = 0; u < 16; u += S) {
      const int64_t k = k0 + 32 * u;
      if (k + 32 * (S - 1) < n) {
        float ah[S][K], al[S][K];
#pragma unroll
        for (int v = 0; v < S; ++v)
#pragma unroll
          for (int r = 0; r < K; ++r) {
            ah[v][r] = ch[r][k + 32 * v];
            al[v][r] = ch[r][k + 32 * v + lo_off];
          }
#pragma unroll
        for (int v = 0; v < S; ++v) add(ah[v], al[v]);
      } else {
#pragma unroll 1
        for (int v = 0; v < S && k + 32 * v < n; ++v) {  // the ragged end, a sample at a time
          float ah[K], al[K];
#pragma unroll
          for (int r = 0; r < K; ++r) {
            ah[r] = ch[r][k + 32 * v];
            al[r] = ch[r][k + 32 * v + lo_off];
          }
          add(ah, al);
        }
      }
    }
#pragma unroll
    for (int e = 0; e < EN; ++e) acc[e] += (double)sh[e] + (double)sl[e];
  }
#pragma unroll
  for (int e = 0; e < EN; ++e) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc[e] += __shfl_xor_sync(0xffffffffu, acc[e], o);
    if (lane == 0) {
      const int r = entry_row(E0 + e, K), c = entry_col(E0 + e, K);
      M[r * K + c] = M[c * K + r] = acc[e] / I.denom;
    }
  }
}

template <int K, int E0>
__device__ __forceinline__ void retest_columns_passes(const Inst &I, const float *const *ch, int64_t lo_off,
                                                      double *M) {
  constexpr int E = K * (K - 1) / 2;
  if constexpr (E0 < E) {
    constexpr int EN = E - E0 < kRetestPass ? E - E0 : kRetestPass;
    retest_columns_pass<K, E0, EN>(I, ch, lo_off, M);
    retest_columns_passes<K, E0 + kRetestPass>(I, ch, lo_off, M);
  }
}

// the item's matrix M (K x K, the warp's shared memory) from its columns
template <int K>
__device__ __forceinline__ void retest_item_columns(const Inst &I, const RetestItem *it, double *M) {
  constexpr int E = K * (K - 1) / 2;
  static_assert(E <= 32, "one lane per entry");
  const int lane = threadIdx.x & 31;
  const int64_t n = I.n_z;
  if (lane < K) M[lane * K + lane] = 1.0;
  // lane e: entry e -- formed by an earlier re-test? then no column is read
  int er = 0, ec = 0;
  int64_t va = 0, vb = 0;
  double v = 0.0;
  bool have = true;
  if (lane < E) {
    entry_rc(lane, K, er, ec);
    va = retest_var(it, er);
    vb = retest_var(it, ec);
    have = ecache_get(I, va, vb, &v);
  }
  if (__all_sync(0xffffffffu, have)) {
    if (lane < E) M[er * K + ec] = M[ec * K + er] = v;
    return;
  }
  const float *ch[K];
  const int64_t lo_off = I.zl - I.zh;  // the zl plane, at a fixed distance from zh
#pragma unroll
  for (int r = 0; r < K; ++r) ch[r] = I.zh + retest_var(it, r) * n;
  retest_columns_passes<K, 0>(I, ch, lo_off, M);
  __syncwarp();
  if (lane < E && !have) ecache_put(I, va, vb, M[er * K + ec]);
}

template <int KM>
__global__ void __launch_bounds__(kRetestWarps * 32, 2) retest_kernel(const __grid_constant__ Launch L) {
  extern __shared__ double retest_smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int l = L.level;
  const int k = l + 2;
  double *M = retest_smem + (size_t)wib * k * k;
  unsigned long long count = L.lc->rq_count;
  if (count > (unsigned long long)L.rq_cap) count = (unsigned long long)L.rq_cap;
  const unsigned long long warp = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) >> 5;
  const unsigned long long nwarps = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
  if (l == 0) {
    for (unsigned long long q = warp; q < count; q += nwarps) {
      const RetestItem *it = L.rq + q;
      const Inst &I = *inst_of(L, it->inst);
      const int64_t i = it->i, j = it->j;
      double r;
      if (!ecache_get(I, i, j, &r)) {
        r = warp_dot(I, i, j) / I.denom;
        if (lane == 0) ecache_put(I, i, j, r);
      }
      double pv;
      if (lane == 0 && !decide_of_r(I, r, false, &pv)) {  // kept: both triangles' bits
        atomicOr(I.adj + i * I.W + (j >> 5), 1u << (j & 31));
        atomicOr(I.adj + j * I.W + (i >> 5), 1u << (i & 31));
      }
    }
    return;
  }
  if (l <= kColumnTop) {
    // an item per warp from its columns (instances with FP32-pair data; FP64 Z takes
    // the general path below)
    for (unsigned long long q = warp; q < count; q += nwarps) {
      const RetestItem *it = L.rq + q;
      const Inst &I = *inst_of(L, it->inst);
      if (!I.zh || !live_bit(I.adj, I.W, it->i, it->j)) continue;
      switch (l) {
        case 1: retest_item_columns<3>(I, it, M); break;
        case 2: retest_item_columns<4>(I, it, M); break;
        case 3: retest_item_columns<5>(I, it, M); break;
        default: retest_item_columns<6>(I, it, M); break;
      }
      __syncwarp();
      if (lane == 0) retest_decide<KM>(L, I, it, l, M);
      __syncwarp();
    }
  }
  const int E = k * (k - 1) / 2;
  // the items not taken above run entry by entry (the first W of them) or a warp each
  const bool by_columns = l <= kColumnTop;
  const unsigned long long W =
      L.rq_val ? min(count, (unsigned long long)(L.rq_vcap / E)) : 0ull;
  const unsigned long long units = W * (unsigned long long)E;
  for (unsigned long long u = warp; u < units; u += nwarps) {
    const unsigned long long q = u / (unsigned long long)E;
    const int e = (int)(u - q * (unsigned long long)E);
    const RetestItem *it = L.rq + q;
    const Inst &I = *inst_of(L, it->inst);
    if (by_columns && I.zh) continue;  // decided above
    const int64_t i = it->i, j = it->j;
    if (live_bit(I.adj, I.W, i, j)) {  // else removed meanwhile: nothing to compute
      int r, c;
      entry_rc(e, k, r, c);
      const int64_t va = retest_var(it, r), vb = retest_var(it, c);
      double v;
      if (!ecache_get(I, va, vb, &v)) {
        v = warp_dot(I, va, vb) / I.denom;
        if (lane == 0) ecache_put(I, va, vb, v);
      }
      if (lane == 0) L.rq_val[q * (unsigned long long)E + e] = v;
    }
    unsigned last = 0;
    if (lane == 0) {
      __threadfence();
      last = atomicAdd(L.rq_done + q, 1u) == (unsigned)(E - 1);
    }
    if (!__shfl_sync(0xffffffffu, last, 0)) continue;
    // the item's last entry: gather its matrix and decide
    __threadfence();
    if (lane == 0) L.rq_done[q] = 0u;
    if (!live_bit(I.adj, I.W, i, j)) continue;
    for (int t = lane; t < k * k; t += 32) {
      const int r = t / k, c = t - r * k;
      double v = 1.0;
      if (r != c) {
        const int a = r < c ? r : c, b2 = r < c ? c : r;
        const int eidx = a * k - a * (a + 1) / 2 + (b2 - a - 1);  // entry_rc's numbering
        v = __ldcg(L.rq_val + q * (unsigned long long)E + eidx);
      }
      M[t] = v;
    }
    __syncwarp();
    if (lane == 0) retest_decide<KM>(L, I, it, l, M);
    __syncwarp();
  }
  // items beyond the scratch: a warp each
  for (unsigned long long q = W + warp; q < count; q += nwarps) {
    const RetestItem *it = L.rq + q;
    const Inst &I = *inst_of(L, it->inst);
    if (by_columns && I.zh) continue;                    // decided above
    if (!live_bit(I.adj, I.W, it->i, it->j)) continue;  // removed by another test meanwhile
    for (int r = 0; r < k; ++r) {
      if (lane == 0) M[r * k + r] = 1.0;
      for (int c2 = r + 1; c2 < k; ++c2) {
        const int64_t va = retest_var(it, r), vb = retest_var(it, c2);
        double v;
        if (!ecache_get(I, va, vb, &v)) {
          v = warp_dot(I, va, vb) / I.denom;
          if (lane == 0) ecache_put(I, va, vb, v);
        }
        if (lane == 0) M[r * k + c2] = M[c2 * k + r] = v;
      }
    }
    __syncwarp();
    if (lane == 0) retest_decide<KM>(L, I, it, l, M);
    __syncwarp();
  }
}

template <bool MIXED>
void *kernel_for(int level, int l1_variant) {
  if (MIXED && l1_variant == kSetOrder && level >= 2 && level <= kSetTop) {
    switch (level) {
      case 2: return (void *)level_kernel<2, true, kSetOrder>;
      case 3: return (void *)level_kernel<3, true, kSetOrder>;
      case 4: return (void *)level_kernel<4, true, kSetOrder>;
      case 5: return (void *)level_kernel<5, true, kSetOrder>;
      case 6: return (void *)level_kernel<6, true, kSetOrder>;
      case 7: return (void *)level_kernel<7, true, kSetOrder>;
      case 8: return (void *)level_kernel<8, true, kSetOrder>;
      default:
        return level <= 12 ? level_kernel_9_12(level, true, true)
               : level <= 16 ? level_kernel_13_16(level, true, true)
                             : level_kernel_17_24_set(level);
    }
  }
  switch (level) {
    case 1:
      if (MIXED && l1_variant == (kL1Interleaved | kQueueOnly)) return (void *)level_kernel<1, true, kL1Interleaved | kQueueOnly>;
      if (MIXED && l1_variant == (kL1Prefetch | kQueueOnly)) return (void *)level_kernel<1, true, kL1Prefetch | kQueueOnly>;
      return l1_variant == kL1Chunked    ? (void *)level_kernel<1, MIXED, kL1Chunked>
             : l1_variant == kL1Prefetch ? (void *)level_kernel<1, MIXED, kL1Prefetch>
                                         : (void *)level_kernel<1, MIXED>;
    case 2: return (void *)level_kernel<2, MIXED>;
    case 3: return (void *)level_kernel<3, MIXED>;
    case 4: return (void *)level_kernel<4, MIXED>;
    case 5: return (void *)level_kernel<5, MIXED>;
    case 6: return (void *)level_kernel<6, MIXED>;
    case 7: return (void *)level_kernel<7, MIXED>;
    case 8: return (void *)level_kernel<8, MIXED>;
    default:
      return level <= 12 ? level_kernel_9_12(level, MIXED, false)
                         : level <= 16 ? level_kernel_13_16(level, MIXED, false) : level_kernel_17_up(level, MIXED);
  }
}

}  // namespace

int citest_grid(int precision, int level, int device, int l1_variant) {
  void *k = precision == HPC_PREC_FP64 ? kernel_for<false>(level, l1_variant) : kernel_for<true>(level, l1_variant);
  const int smem = level == 1 ? 0 : kRowCache * (int)sizeof(unsigned long long);
  // the row-offset cache is beyond the default 48 KB of dynamic shared memory
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) cudaGetLastError();
  int per_sm = 0, sms = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kThreads, smem) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms < 1) sms = 1;
  return per_sm * sms;
}

// The re-test kernel of levels 17-32 needs up to 74 KB of dynamic shared memory, above
// the default 48 KB: allowed once per creation of a context that can reach those levels
// (not at launch, which may be under capture; levels up to 16 stay below 48 KB).
void retest_setup() {
  const int most = (int)(sizeof(double) * kRetestWarps * (HPC_MAX_LEVEL + 2) * (HPC_MAX_LEVEL + 2));
  if (cudaFuncSetAttribute((const void *)retest_kernel<HPC_MAX_LEVEL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           most) != cudaSuccess)
    cudaGetLastError();
}

hpc_status launch_retest(const Launch &L, int sms, cudaStream_t s) {
  const int kmax = L.level + 2;
  const size_t smem = sizeof(double) * (size_t)kRetestWarps * kmax * kmax;  // 20.7 KB at level 16
  if (L.level <= 16)
    retest_kernel<16><<<sms * 4, kRetestWarps * 32, smem, s>>>(L);
  else
    retest_kernel<HPC_MAX_LEVEL><<<sms * 4, kRetestWarps * 32, smem, s>>>(L);
  HPC_LAUNCH_CHECK("retest_kernel");
  return HPC_OK;
}

hpc_status launch_finalize_records(const Inst *inst, int count, cudaStream_t s) {
  finalize_records_kernel<<<152 * 4, 128, 0, s>>>(inst, count);
  HPC_LAUNCH_CHECK("finalize_records_kernel");
  return HPC_OK;
}

hpc_status launch_gather_records(const Inst *inst, int count, const long long *prefix, long long total, int stride,
                                 int32_t *out, cudaStream_t s) {
  if (total <= 0) return HPC_OK;
  const long long blocks = std::min<long long>((total + 7) / 8, 152 * 8);
  gather_records_kernel<<<(unsigned)blocks, 256, 0, s>>>(inst, count, prefix, total, stride, out);
  HPC_LAUNCH_CHECK("gather_records_kernel");
  return HPC_OK;
}

hpc_status launch_pack_records(const Inst *inst, const RecSegment *seg, int nseg, int32_t *out, cudaStream_t s) {
  if (nseg <= 0) return HPC_OK;
  pack_records_kernel<<<(unsigned)std::min(nseg, 152 * 16), 256, 0, s>>>(inst, seg, nseg, out);
  HPC_LAUNCH_CHECK("pack_records_kernel");
  return HPC_OK;
}

hpc_status launch_level(const Launch &L, int precision, int grid, int l1_variant, cudaStream_t s) {
  void *k = precision == HPC_PREC_FP64 ? kernel_for<false>(L.level, l1_variant)
                                       : kernel_for<true>(L.level, l1_variant);
  Launch args = L;
  void *params[] = {&args};
  // cooperative: every block co-resident, as the grid barriers require
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = L.level == 1 || !L.row_cache ? 0 : kRowCache * sizeof(unsigned long long);
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  HPC_CUDA(cudaLaunchKernelExC(&cfg, k, params));
  return HPC_OK;
}

}  // namespace hpc
