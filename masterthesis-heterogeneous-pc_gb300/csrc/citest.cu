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
// in FP32 on the stored FP32 |r|. Run at the end of every skeleton run.
__global__ void finalize_records_kernel(const Inst *__restrict__ inst, int count) {
  const unsigned long long tid = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
  const unsigned long long nthreads = (unsigned long long)gridDim.x * blockDim.x;
  for (int b = 0; b < count; ++b) {
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
      const double pv = exact_pvalue<HPC_MAX_LEVEL>(I, h->i, h->j, rec + kRecHeadWords, h->level);
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

// Records of all instances in the packed form of hpc_batch_get_records_packed: record
// r (instance b with pre[b] <= r < pre[b + 1]) has level l, found from the instance's
// removals per level (records are appended level by level, so an instance's records of
// level l follow those of lower levels), and goes to word
//   inst_words[b] + sum_{l' < l} deleted(l') * w(l') + (rank within level l) * w(l),
// w(l) = 6 + 2 ceil(l / 2). One warp per record.
__global__ void pack_records_kernel(const Inst *__restrict__ inst, int count, const long long *__restrict__ pre,
                                    const long long *__restrict__ inst_words, long long total,
                                    int32_t *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long r = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; r < total; r += nw) {
    const int b = find_inst(pre, count, r);
    const Inst &I = inst[b];
    const long long rr = r - pre[b];
    long long cum = 0, words = inst_words[b];
    int l = 1;
    for (; l <= HPC_MAX_LEVEL; ++l) {
      const long long d = (long long)I.ctr[l].deleted;
      if (rr < cum + d) break;
      cum += d;
      words += d * (long long)(6 + ((l + 1) & ~1));
    }
    const int w = 6 + ((l + 1) & ~1);
    const int32_t *src = I.recs + rr * (long long)I.rec_stride;
    int32_t *dst = out + words + (rr - cum) * (long long)w;
    for (int q = lane; q < w; q += 32) dst[q] = q < 6 + l ? src[q] : -1;
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

template <int KM>
__global__ void __launch_bounds__(kRetestWarps * 32) retest_kernel(const __grid_constant__ Launch L) {
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
      const double r = warp_dot(I, i, j) / I.denom;
      double pv;
      if (lane == 0 && !decide_of_r(I, r, false, &pv)) {  // kept: both triangles' bits
        atomicOr(I.adj + i * I.W + (j >> 5), 1u << (j & 31));
        atomicOr(I.adj + j * I.W + (i >> 5), 1u << (i & 31));
      }
    }
    return;
  }
  const int E = k * (k - 1) / 2;
  const unsigned long long W =
      L.rq_val ? min(count, (unsigned long long)(L.rq_vcap / E)) : 0ull;  // items run entry by entry
  const unsigned long long units = W * (unsigned long long)E;
  for (unsigned long long u = warp; u < units; u += nwarps) {
    const unsigned long long q = u / (unsigned long long)E;
    const int e = (int)(u - q * (unsigned long long)E);
    const RetestItem *it = L.rq + q;
    const Inst &I = *inst_of(L, it->inst);
    const int64_t i = it->i, j = it->j;
    if (live_bit(I.adj, I.W, i, j)) {  // else removed meanwhile: nothing to compute
      int r, c;
      entry_rc(e, k, r, c);
      const double v = warp_dot(I, retest_var(it, r), retest_var(it, c)) / I.denom;
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
    if (!live_bit(I.adj, I.W, it->i, it->j)) continue;  // removed by another test meanwhile
    for (int r = 0; r < k; ++r) {
      if (lane == 0) M[r * k + r] = 1.0;
      for (int c2 = r + 1; c2 < k; ++c2) {
        const double v = warp_dot(I, retest_var(it, r), retest_var(it, c2)) / I.denom;
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
  if (MIXED && l1_variant == kSetOrder && level >= 2 && level <= 16) {
    switch (level) {
      case 2: return (void *)level_kernel<2, true, kSetOrder>;
      case 3: return (void *)level_kernel<3, true, kSetOrder>;
      case 4: return (void *)level_kernel<4, true, kSetOrder>;
      case 5: return (void *)level_kernel<5, true, kSetOrder>;
      case 6: return (void *)level_kernel<6, true, kSetOrder>;
      case 7: return (void *)level_kernel<7, true, kSetOrder>;
      case 8: return (void *)level_kernel<8, true, kSetOrder>;
      default: return level <= 12 ? level_kernel_9_12(level, true, true) : level_kernel_13_16(level, true, true);
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
  finalize_records_kernel<<<152 * 2, 128, 0, s>>>(inst, count);
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

hpc_status launch_pack_records(const Inst *inst, int count, const long long *prefix, const long long *inst_words,
                               long long total, int32_t *out, cudaStream_t s) {
  if (total <= 0) return HPC_OK;
  const long long blocks = std::min<long long>((total + 7) / 8, 152 * 8);
  pack_records_kernel<<<(unsigned)blocks, 256, 0, s>>>(inst, count, prefix, inst_words, total, out);
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
