// The first two phases of a level kernel (levels >= 1), separated by grid barriers of
// a cooperative launch:
//
//   rebuild  every warp takes a contiguous run of rows (flattened over the instances),
//            counts each row's live bits (the snapshot degree d_i) and writes its
//            neighbour ids, ascending, into the row's fixed slot of the neighbour-list
//            buffer -- slots are sized by the degrees after level 0 (degrees only
//            fall), so no per-level offsets are needed for the lists; the per-segment
//            sums of d_i, of the row test counts d_i * C(d_i - 1, l) and of the row
//            conditioning-set counts C(d_i, l) go to SegAgg.
//   scan     one block per segment of kSegRows rows: the exclusive prefix of the row
//            work units -- tests in the edge order, conditioning sets in the set order
//            (citest.cuh) -- which is the CI-test phase's flattened index, each
//            instance's level summary, and (one block) the prefix of the instances'
//            unit counts.
//
// Together they replace compactCUTiled (src/independence/compact.cu:4-89), which
// rebuilds the reference's dense adj_compact rows with one thread block per row.
#pragma once
#include "internal.cuh"
#include "stats.cuh"

namespace hpc {

constexpr int kLevelThreads = 256;
static_assert(kLevelThreads == kSegRows, "one scan thread per segment row");

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int *p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid-wide barrier of a cooperative launch (all blocks co-resident). `epoch` counts
// the barriers this block has passed. The wait is bounded (L.wait_ns of %globaltimer,
// 2 s by default): on expiry the kernel's error flag is set and false is returned; the
// caller returns. L.bar_extra (0 outside tests) raises the arrival target, so that a
// test can make the wait run out without anything faulting.
__device__ __forceinline__ bool grid_barrier(const Launch &L, unsigned int &epoch) {
  __shared__ int s_ok;
  __syncthreads();
  ++epoch;
  if (threadIdx.x == 0) {
    const unsigned int target = epoch * gridDim.x + L.bar_extra;
    __threadfence();
    atomicAdd(&L.lc->bar, 1u);
    int ok = 1;
    const unsigned long long t0 = globaltimer_ns();
    while (ld_acquire_u32(&L.lc->bar) < target) {
      if (globaltimer_ns() - t0 > L.wait_ns) {
        ok = 0;
        atomicOr(&inst_of(L, 0)->g->err, kErrTimeout);
        break;
      }
      __nanosleep(20);
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// tests a row of degree d contributes at level l; sets *over when beyond the limit
// (limit: the launch's row_work_limit, so that the level's total fits 63 bits)
__device__ __forceinline__ unsigned long long row_tests(int d, int level, unsigned long long limit, int *over) {
  if (d - 1 < level) return 0ull;
  const unsigned long long c = binom_fast(d - 1, level);
  if (c >= limit || (unsigned long long)d * c >= limit || umul64hi((unsigned long long)d, c) != 0ull) {
    *over = 1;
    return 0ull;
  }
  return (unsigned long long)d * c;
}

// conditioning sets of a row of degree d at level l (the set order's units): C(d, l)
// when the row has tests (d - 1 >= l), else 0. Never above row_tests.
__device__ __forceinline__ unsigned long long row_sets(int d, int level) {
  return d - 1 < level ? 0ull : binom_fast(d, level);
}

__device__ __forceinline__ bool csr_overflow(const Inst &I) { return (long long)I.rowptr[I.p] > I.colidx_cap; }

// Row i's neighbour list from its adjacency row (whole warp, converged), written
// ascending at its CSR slot; returns the degree (warp-uniform).
__device__ __forceinline__ int extract_row(const Inst &I, int64_t i) {
  const int lane = threadIdx.x & 31;
  // the row's first 128 words and its slot offset in one round trip
  const uint32_t *words = I.adj + i * I.W;
  const int W = I.W;
  uint32_t pre[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) pre[q] = q * 32 + lane < W ? words[q * 32 + lane] : 0u;
  int *out = I.colidx + I.rowptr[i];
  int cnt = 0;
  auto emit = [&](uint32_t word, int w) {
    const int c = __popc(word);
    int incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    int pos = cnt + incl - c;
    while (word) {
      const int bit = __ffs(word) - 1;
      out[pos++] = w * 32 + bit;
      word &= word - 1;
    }
    cnt += __shfl_sync(0xffffffffu, incl, 31);
  };
#pragma unroll
  for (int q = 0; q < 4; ++q)
    if (q * 32 < W) emit(pre[q], q * 32 + lane);
  for (int w0 = 128; w0 < W; w0 += 32) emit(w0 + lane < W ? words[w0 + lane] : 0u, w0 + lane);
  return cnt;
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// The level's neighbour-list snapshot and its per-segment sums (degrees, tests,
// conditioning sets, rows with tests). A warp takes a contiguous range of rows, 32 at a
// time (a lane each, within one instance and segment). A row's list is extracted again
// (whole warp) only when it may have changed: every row of an instance whose snapshot is
// not current (after level 0, a reset or a new instance table), else the rows that lost
// an edge since their last extraction (marked by claim_edge); the other rows keep their
// lists and degrees. Rows of an instance whose lists overflow their capacity are left
// alone (the scan phase flags it; the host resizes and reruns).
__device__ __forceinline__ void rebuild_phase(const Launch &L) {
  const int lane = threadIdx.x & 31;
  const long long gw = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  const long long R = L.total_rows;
  const long long per = (R + nw - 1) / nw;
  long long t = gw * per;
  const long long tend = t + per < R ? t + per : R;
  const int level = L.level;
  long long cur = -1;
  unsigned long long a_deg = 0, a_work = 0, a_sets = 0;
  int a_max = 0, a_rows = 0, a_over = 0;
  auto flush = [&]() {
    if (cur >= 0 && lane == 0) {
      SegAgg &S = L.seg[cur];
      if (a_deg) atomicAdd(&S.deg, a_deg);
      if (a_work) atomicAdd(&S.work, a_work);
      if (a_sets) atomicAdd(&S.sets, a_sets);
      if (a_max) atomicMax(&S.max_deg, a_max);
      if (a_rows) atomicAdd(&S.rows, a_rows);
      if (a_over) atomicOr(&S.over, 1);
    }
    a_deg = a_work = a_sets = 0;
    a_max = a_rows = a_over = 0;
  };
  int b = -1;
  const Inst *I = nullptr;
  long long r0 = 0, r1 = 0, g0 = 0;
  bool skip = false, current = false;
  while (t < tend) {
    if (b < 0 || t >= r1) {
      b = L.count == 1 ? 0 : find_inst(L.row_prefix, L.count, t);
      I = inst_of(L, b);
      r0 = row_begin(L, b);
      r1 = row_end(L, b);
      g0 = seg_begin(L, b);
      skip = csr_overflow(*I);  // flagged by the scan phase; the host resizes and reruns
      current = !skip && I->dirty && __ldcg(&I->g->snap) == I->snap_epoch;
    }
    const int64_t i0 = t - r0;
    const long long g = g0 + i0 / kSegRows;
    if (g != cur) {
      flush();
      cur = g;
    }
    const long long seg_end_row = r0 + (i0 / kSegRows + 1) * kSegRows;
    const int n = (int)min(32ll, min(tend, min(r1, seg_end_row)) - t);
    const int64_t i = i0 + lane;
    const bool mine = lane < n && !skip;
    const bool stale = mine && (!current || I->dirty[i] != 0);
    int cnt = mine && !stale ? I->deg[i] : 0;
    unsigned todo = __ballot_sync(0xffffffffu, stale);
    while (todo) {
      const int q = __ffs(todo) - 1;
      todo &= todo - 1;
      const int c = extract_row(*I, i0 + q);
      if (lane == q) cnt = c;
    }
    if (stale) {
      I->deg[i] = cnt;
      if (I->dirty) I->dirty[i] = 0;
    }
    int over = 0;
    const unsigned long long w = mine ? row_tests(cnt, level, L.row_work_limit, &over) : 0ull;
    a_deg += warp_sum_u64(mine ? (unsigned long long)cnt : 0ull);
    a_work += warp_sum_u64(w);
    a_sets += warp_sum_u64(w ? row_sets(cnt, level) : 0ull);
    a_max = max(a_max, __reduce_max_sync(0xffffffffu, mine ? cnt : 0));
    a_rows += (int)__reduce_add_sync(0xffffffffu, w ? 1u : 0u);
    a_over |= (int)__reduce_or_sync(0xffffffffu, (unsigned)over);
    t += n;
  }
  // the warps' last segment sums are merged per block first (the warps of a block
  // take neighbouring rows): one set of global atomics per block and segment
  __shared__ long long s_seg[kLevelThreads / 32];
  __shared__ unsigned long long s_v[kLevelThreads / 32][3];
  __shared__ int s_i[kLevelThreads / 32][3];
  const int wid = threadIdx.x >> 5;
  if (lane == 0) {
    s_seg[wid] = cur;
    s_v[wid][0] = a_deg;
    s_v[wid][1] = a_work;
    s_v[wid][2] = a_sets;
    s_i[wid][0] = a_max;
    s_i[wid][1] = a_rows;
    s_i[wid][2] = a_over;
  }
  __syncthreads();
  if (threadIdx.x < kLevelThreads / 32) {
    const int q = threadIdx.x;
    const long long g = s_seg[q];
    bool leader = g >= 0;
    for (int r = 0; r < q && leader; ++r) leader = s_seg[r] != g;
    if (leader) {
      unsigned long long v0 = 0, v1 = 0, v2 = 0;
      int i0 = 0, i1 = 0, i2 = 0;
      for (int r = q; r < kLevelThreads / 32; ++r)
        if (s_seg[r] == g) {
          v0 += s_v[r][0];
          v1 += s_v[r][1];
          v2 += s_v[r][2];
          i0 = max(i0, s_i[r][0]);
          i1 += s_i[r][1];
          i2 |= s_i[r][2];
        }
      SegAgg &S = L.seg[g];
      if (v0) atomicAdd(&S.deg, v0);
      if (v1) atomicAdd(&S.work, v1);
      if (v2) atomicAdd(&S.sets, v2);
      if (i0) atomicMax(&S.max_deg, i0);
      if (i1) atomicAdd(&S.rows, i1);
      if (i2) atomicOr(&S.over, 1);
    }
  }
}

// block-wide exclusive scan of one value per thread; *total receives the sum
__device__ __forceinline__ unsigned long long block_exclusive_scan(unsigned long long v, unsigned long long *total) {
  __shared__ unsigned long long s_warp[kLevelThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned long long incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long x = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += x;
  }
  if (lane == 31) s_warp[wid] = incl;
  __syncthreads();
  unsigned long long before = 0, all = 0;
#pragma unroll
  for (int q = 0; q < kLevelThreads / 32; ++q) {
    const unsigned long long x = s_warp[q];
    if (q < wid) before += x;
    all += x;
  }
  __syncthreads();
  *total = all;
  return before + incl - v;
}

struct InstSums {
  unsigned long long deg, work, units, base;
  int max_deg, rows, over;
};

// sums over the segments of instance b (one warp); base = units of segments before g
// (units: tests, or conditioning sets with `set`)
__device__ __forceinline__ InstSums warp_inst_sums(const Launch &L, int b, long long g, bool set) {
  const int lane = threadIdx.x & 31;
  InstSums r{0, 0, 0, 0, 0, 0, 0};
  for (long long q = seg_begin(L, b) + lane; q < seg_end(L, b); q += 32) {
    const SegAgg *S = L.seg + q;
    const unsigned long long wk = __ldcg(&S->work);
    const unsigned long long un = set ? __ldcg(&S->sets) : wk;
    r.deg += __ldcg(&S->deg);
    r.work += wk;
    r.units += un;
    if (q < g) r.base += un;
    r.max_deg = max(r.max_deg, __ldcg(&S->max_deg));
    r.rows += __ldcg(&S->rows);
    r.over |= __ldcg(&S->over);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    r.deg += __shfl_xor_sync(0xffffffffu, r.deg, o);
    r.work += __shfl_xor_sync(0xffffffffu, r.work, o);
    r.units += __shfl_xor_sync(0xffffffffu, r.units, o);
    r.base += __shfl_xor_sync(0xffffffffu, r.base, o);
    r.max_deg = max(r.max_deg, __shfl_xor_sync(0xffffffffu, r.max_deg, o));
    r.rows += __shfl_xor_sync(0xffffffffu, r.rows, o);
    r.over |= __shfl_xor_sync(0xffffffffu, r.over, o);
  }
  return r;
}

__device__ __forceinline__ void scan_phase(const Launch &L, bool set) {
  __shared__ InstSums s_sum;
  __shared__ int s_bad;
  const int level = L.level;
  const long long G = L.total_segs;
  // the prefix of the instances' test counts, by the last block (the first blocks
  // take the segments)
  if (blockIdx.x == gridDim.x - 1) {
    __shared__ unsigned long long s_carry;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (int c0 = 0; c0 < L.count; c0 += kLevelThreads) {
      const int b = c0 + (int)threadIdx.x;
      unsigned long long tot = 0;
      if (b < L.count) {
        int over = 0, md = 0;
        for (long long q = seg_begin(L, b); q < seg_end(L, b); ++q) {
          tot += set ? __ldcg(&L.seg[q].sets) : __ldcg(&L.seg[q].work);
          over |= __ldcg(&L.seg[q].over);
          md = max(md, __ldcg(&L.seg[q].max_deg));
        }
        if (over || csr_overflow(*inst_of(L, b))) tot = 0;
        if (md > 0) atomicMax(&L.lc->max_deg, md);  // the key of the level's tile policy
      }
      unsigned long long all;
      const unsigned long long ex = block_exclusive_scan(tot, &all);
      if (b < L.count) L.work_prefix[b] = s_carry + ex;
      __syncthreads();
      if (threadIdx.x == 0) s_carry += all;
      __syncthreads();
    }
    if (threadIdx.x == 0) L.work_prefix[L.count] = s_carry;
  }
  for (long long g = blockIdx.x; g < G; g += gridDim.x) {
    const int b = L.count == 1 ? 0 : find_inst(L.seg_prefix, L.count, g);
    const Inst &I = *inst_of(L, b);
    // the row's degree is read before the segment sums (one round trip for both)
    const int64_t r = (g - seg_begin(L, b)) * kSegRows + threadIdx.x;
    const bool valid = r < I.p;
    const int d_row = valid ? __ldcg(I.deg + r) : 0;
    if (threadIdx.x < 32) {
      const InstSums rs = warp_inst_sums(L, b, g, set);
      if (threadIdx.x == 0) {
        s_sum = rs;
        s_bad = (rs.over || csr_overflow(I)) ? 1 : 0;
      }
    }
    __syncthreads();
    const bool bad = s_bad != 0;
    int over = 0;
    const int d = bad ? 0 : d_row;
    unsigned long long w = row_tests(d, level, L.row_work_limit, &over);
    if (set && w) w = row_sets(d, level);
    unsigned long long all;
    const unsigned long long ex = block_exclusive_scan(w, &all);
    if (valid && !bad) I.row_work[r] = s_sum.base + ex;
    if (threadIdx.x == 0 && g == seg_end(L, b) - 1) {
      // last segment of the instance: its level summary
      DevCounters &C = I.ctr[level];
      if (!bad) I.row_work[I.p] = s_sum.units;
      // the lists just rebuilt are the instance's snapshot (unless they overflowed, or the
      // level is 1, whose removals do not mark their rows)
      I.g->snap = bad || s_sum.over || level == 1 ? 0ull : I.snap_epoch;
      if (s_sum.over) atomicOr(&I.g->err, kErrWorkOverflow);
      if (csr_overflow(I)) atomicOr(&I.g->err, kErrCsrOverflow);
      C.edges2 = s_sum.deg;
      C.work_total = bad ? 0ull : s_sum.work;
      C.max_deg = s_sum.max_deg;
      C.rows = s_sum.rows;
      C.tests = 0;
      C.retests = 0;
      C.deleted = 0;
      C.band_violations = 0;
      C.rec_begin = *(volatile unsigned long long *)&I.g->rec_count;
    }
    __syncthreads();
  }
}

}  // namespace hpc
