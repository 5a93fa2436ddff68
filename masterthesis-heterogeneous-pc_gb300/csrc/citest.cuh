// Device code of the level kernels (levels >= 1), shared by the translation units
// that instantiate them: citest.cu (levels 1-8, the re-test and record kernels and the
// launchers) and citest_l9.cu / citest_l13.cu / citest_l17.cu (levels 9-12, 13-16 and
// the runtime-level kernel of levels 17-32, compiled in parallel).
//
// Level-l conditional-independence tests (l >= 1) on a persistent grid, over all
// instances of a context in one launch.
//
// Replaces testRowL1 / testRowLN<l+2,l> (src/executor/testing/gpuRowTests.cu:29-205),
// their workstealing twins (src/executor/testing/gpuWorkstealingTests.cu) and the
// CPU/GPU balancer (src/loadbalance/balancer.cpp): the reference launches one
// 64-thread block per (row, neighbour slot) with grid y = the maximum degree and has
// each thread unrank a subset and run a 30-iteration FP64 SVD in local memory.
//
// Here every test of the level is one index of a flattened space
//   t in [0, sum_b T_l(b)),  T_l(b) = sum_i d_i * C(d_i - 1, l)
// ordered by (instance b, row i, neighbour slot s, lexicographic subset rank). Warps
// take tiles of 32 * m consecutive tests (the first by their index, later ones with
// one atomicAdd on a device-wide counter); the warp finds the row of its tile start by
// a 32-ary search, each lane its own row from the next 32 row offsets. At level 1 the
// lanes are interleaved over the tile (tests_l1); at levels >= 2 each lane takes m
// consecutive tests, unranks its first subset once (the order of ithCombination,
// src/util/cuda_util.cu:34-50) and then steps to the lexicographic successor. Lanes
// stop testing an edge as soon as its live bit is cleared (the reference's
// `adj == 0` early exit, gpuRowTests.cu:166-168).
//
// The partial correlation of (i, j) given S comes from a Cholesky factorisation of
// the S block and forward solves for r_iS and r_jS:
//   r = (r_ij - w_i . w_j) / sqrt((1 - |w_i|^2)(1 - |w_j|^2)),  w = L_S^-1 r_S.
// In mixed precision this runs in FP32 on cor32; a test is decided in FP32 only when
// |r| is outside the re-test band around r_crit (the configured relative |z| margin
// plus an error bound from the smallest pivot); every other test is re-evaluated in
// FP64 with the reference's formula (closed form at l = 1 as cpuInd.cpp:16-27; pinv
// semantics at l >= 2 as cpuInd.cpp:29-38: Cholesky when well conditioned, Jacobi
// pseudoinverse with arma::pinv's tolerance otherwise). The decision is p >= alpha in
// FP64. With an FP64 matrix the re-test runs inline; without one (tensor-core mode)
// it is queued for retest_kernel, which forms the FP64 entries as warp-cooperative
// dot products of the standardised data.
//
// Removal (src/executor/testing/cpuUtil.cpp:23-48, gpuRowTests.cu:172-201): the lane
// clearing the (min, max) bit with atomicAnd owns the edge and clears the mirror bit;
// its separation-set record is appended when the warp's tile is done.
//
// A level is one cooperative launch (level_kernel): snapshot rebuild and test-count
// scan (rebuild.cuh), each followed by a grid barrier, then the CI tests.
#pragma once
#include <cuda_runtime.h>

#include <type_traits>

#include "internal.cuh"
#include "rebuild.cuh"
#include "stats.cuh"

namespace hpc {
namespace {

constexpr int kThreads = kLevelThreads;

// Loops over a level's conditioning-set members are unrolled in the kernels of levels
// 1-16 (LA = the level); the runtime-level kernel of levels 17-32 (LA = HPC_MAX_LEVEL)
// keeps them rolled, which bounds its code size and compile time.
template <int LA>
constexpr int kUnr = LA <= kSetTop ? (LA > 0 ? LA : 1) : 1;

__device__ __forceinline__ bool live_bit(const uint32_t *adj, int W, int64_t i, int64_t j) {
  const volatile uint32_t *w = adj + i * W + (j >> 5);
  return (*w >> (j & 31)) & 1u;
}

// FP64 correlation entries of one instance: read from its FP64 matrix when there is
// one, else the dot product of its FP64-standardised columns (zdot). Index order as the
// reference reads cor[row * p + col].
__device__ __forceinline__ double exact_entry(const Inst &I, int64_t x, int64_t y) {
  if (I.cor64) return I.cor64[x * I.p + y];
  double v;
  if (ecache_get(I, x, y, &v)) return v;
  v = zdot(I, x, y, 0, 1) / I.denom;
  ecache_put(I, x, y, v);
  return v;
}

// FP64 partial correlation of a k x k submatrix M (row-major, ordered i, j, S;
// overwritten): the value the reference's p-value formula is applied to. *nan_p is
// set where the reference's p-value is NaN (a NaN entry, cpuInd.cpp:31-33 and the
// closed form at l = 1): the edge is kept.
template <int LA>
__device__ __noinline__ double partial_r_of_matrix(double *M, int l, bool *nan_p) {
  const int k = l + 2;
  *nan_p = false;
  if (l == 1) {  // closed form (cpuInd.cpp:16-27), as pval_l1_64
    const double x1 = M[1], x2 = M[2], x3 = M[k + 2];
    if (isnan(x1) || isnan(x2) || isnan(x3)) {
      *nan_p = true;
      return 0.0;
    }
    return (x1 - x2 * x3) / sqrt((1.0 - x3 * x3) * (1.0 - x2 * x2));
  }
  for (int q = 0; q < k * k; ++q)
    if (isnan(M[q])) {
      *nan_p = true;
      return 0.0;
    }
  double Lm[LA * (LA + 1) / 2], wx[LA], wy[LA];
  double dmin = 1.0;
  for (int r = 0; r < l; ++r) {
    for (int c = 0; c < r; ++c) {
      double v = M[(c + 2) * k + (r + 2)];
      for (int q = 0; q < c; ++q) v -= Lm[r * (r + 1) / 2 + q] * Lm[c * (c + 1) / 2 + q];
      Lm[r * (r + 1) / 2 + c] = v / Lm[c * (c + 1) / 2 + c];
    }
    double d = 1.0;
    for (int q = 0; q < r; ++q) d -= Lm[r * (r + 1) / 2 + q] * Lm[r * (r + 1) / 2 + q];
    dmin = fmin(dmin, d);
    if (!(d > 1e-10)) break;
    const double lrr = sqrt(d);
    Lm[r * (r + 1) / 2 + r] = lrr;
    double vx = M[r + 2], vy = M[k + r + 2];
    for (int q = 0; q < r; ++q) {
      vx -= Lm[r * (r + 1) / 2 + q] * wx[q];
      vy -= Lm[r * (r + 1) / 2 + q] * wy[q];
    }
    wx[r] = vx / lrr;
    wy[r] = vy / lrr;
  }
  if (dmin > 1e-10) {
    double ax = 1.0, ay = 1.0, b = M[1];
    for (int q = 0; q < l; ++q) {
      ax -= wx[q] * wx[q];
      ay -= wy[q] * wy[q];
      b -= wx[q] * wy[q];
    }
    if (ax > 1e-10 && ay > 1e-10) return b / sqrt(ax * ay);
  }
  double V[(LA + 2) * (LA + 2)];
  double p00, p01, p11;
  pinv_sym64_corner(M, k, V, &p00, &p01, &p11);
  return -p01 / sqrt(p00 * p11);
}

// FP64 p-value of a k x k submatrix M with the reference's semantics.
template <int LA>
__device__ __forceinline__ double pvalue_of_matrix(double *M, int l, int n_obs) {
  bool nan_p;
  const double r = partial_r_of_matrix<LA>(M, l, &nan_p);
  return nan_p ? nan("") : calc_pvalue64(r, n_obs);
}

// The reference's decision p >= alpha from the FP64 partial correlation r: the
// p-value is monotone in |r|, so outside [r_lo, r_hi] (|r_crit| -+ 1e-7 relative,
// far beyond the formula's rounding) |r| decides; inside, the formula itself. *pv
// receives the p-value where it was evaluated, else -1 - |r| (evaluated later, when
// the records are read; calc_pvalue64 clamps |r| the same way).
__device__ __forceinline__ bool decide_of_r(const Inst &I, double r, bool nan_p, double *pv) {
  if (nan_p) {
    *pv = nan("");
    return false;
  }
  const double ar = isnan(r) ? 0.0 : fmin(kCutThr, fabs(r));
  if (ar < I.r_lo) {
    *pv = isnan(r) ? 1.0 : -1.0 - ar;
    return true;
  }
  if (ar > I.r_hi) {
    *pv = -1.0 - ar;
    return false;
  }
  *pv = calc_pvalue64(r, I.n_obs);
  return *pv >= I.alpha;
}

// FP64 p-value of the test (i, j | ids) of instance I.
template <int LA>
__device__ __noinline__ double exact_pvalue(const Inst &I, int64_t i, int64_t j, const int *ids, int l) {
  const int k = l + 2;
  double M[(LA + 2) * (LA + 2)];
  for (int q = 0; q < k * k; ++q) M[q] = 0.0;
  for (int q = 0; q < k; ++q) M[q * k + q] = 1.0;
  M[1] = M[k] = exact_entry(I, i, j);
  for (int q = 2; q < k; ++q) {
    M[q] = M[q * k] = exact_entry(I, i, ids[q - 2]);
    M[k + q] = M[q * k + 1] = exact_entry(I, j, ids[q - 2]);
  }
  for (int r = 2; r < k; ++r)
    for (int c = r + 1; c < k; ++c) M[r * k + c] = M[c * k + r] = exact_entry(I, ids[r - 2], ids[c - 2]);
  return pvalue_of_matrix<LA>(M, l, I.n_obs);
}

// The reference's decision for the test (i, j | ids) in FP64 (see decide_of_r).
template <int LA>
__device__ __noinline__ bool exact_remove(const Inst &I, int64_t i, int64_t j, const int *ids, int l, double *pv) {
  const int k = l + 2;
  double M[(LA + 2) * (LA + 2)];
  for (int q = 0; q < k * k; ++q) M[q] = 0.0;
  for (int q = 0; q < k; ++q) M[q * k + q] = 1.0;
  M[1] = M[k] = exact_entry(I, i, j);
  for (int q = 2; q < k; ++q) {
    M[q] = M[q * k] = exact_entry(I, i, ids[q - 2]);
    M[k + q] = M[q * k + 1] = exact_entry(I, j, ids[q - 2]);
  }
  for (int r = 2; r < k; ++r)
    for (int c = r + 1; c < k; ++c) M[r * k + c] = M[c * k + r] = exact_entry(I, ids[r - 2], ids[c - 2]);
  bool nan_p;
  const double r = partial_r_of_matrix<LA>(M, l, &nan_p);
  return decide_of_r(I, r, nan_p, pv);
}

// exact_remove from the FP64 matrix with the factorisation in registers: every entry
// gathered in one round of loads, rsqrt in place of divisions and square roots (a
// few ulps, far inside decide_of_r's guard band). Tests the Cholesky path does not
// accept (an ill-conditioned block) and instances without an FP64 matrix go to
// exact_remove.
template <int LA>
__device__ __noinline__ bool exact_remove_fast(const Inst &I, int64_t i, int64_t j, const int *ids, int l, double *pv) {
  const double *C = I.cor64;
  if (!C) return exact_remove<LA>(I, i, j, ids, l, pv);
  const int64_t p = I.p;
  const double rij = C[i * p + j];
  double gx[LA], gy[LA], gs[LA * (LA - 1) / 2 > 0 ? LA * (LA - 1) / 2 : 1];
#pragma unroll (kUnr<LA>)
  for (int r = 0; r < LA; ++r)
    if (r < l) {
      const int64_t idr = ids[r];
      gx[r] = C[i * p + idr];
      gy[r] = C[j * p + idr];
#pragma unroll (kUnr<LA>)
      for (int c = 0; c < LA; ++c)
        if (c < r) gs[r * (r - 1) / 2 + c] = C[(int64_t)ids[c] * p + idr];
    }
  if (l == 1) {  // the closed form, as pval_l1_64
    const double x1 = rij, x2 = gx[0], x3 = gy[0];
    if (isnan(x1) || isnan(x2) || isnan(x3)) return decide_of_r(I, 0.0, true, pv);
    return decide_of_r(I, (x1 - x2 * x3) / sqrt((1.0 - x3 * x3) * (1.0 - x2 * x2)), false, pv);
  }
  bool nan_in = isnan(rij);
#pragma unroll (kUnr<LA>)
  for (int r = 0; r < LA; ++r)
    if (r < l) {
      nan_in |= isnan(gx[r]) || isnan(gy[r]);
#pragma unroll (kUnr<LA>)
      for (int c = 0; c < LA; ++c)
        if (c < r) nan_in |= isnan(gs[r * (r - 1) / 2 + c]);
    }
  if (nan_in) return decide_of_r(I, 0.0, true, pv);
  double Lm[LA * (LA + 1) / 2 > 0 ? LA * (LA + 1) / 2 : 1], inv[LA], wx[LA], wy[LA];
  bool ok = true;
#pragma unroll (kUnr<LA>)
  for (int r = 0; r < LA; ++r)
    if (r < l) {
      double vx = gx[r], vy = gy[r], d = 1.0;
#pragma unroll (kUnr<LA>)
      for (int c = 0; c < LA; ++c)
        if (c < r) {
          double v = gs[r * (r - 1) / 2 + c];
#pragma unroll (kUnr<LA>)
          for (int q = 0; q < LA; ++q)
            if (q < c) v -= Lm[r * (r + 1) / 2 + q] * Lm[c * (c + 1) / 2 + q];
          v *= inv[c];
          Lm[r * (r + 1) / 2 + c] = v;
          d -= v * v;
          vx -= v * wx[c];
          vy -= v * wy[c];
        }
      ok = ok && d > 1e-10;
      inv[r] = rsqrt(fmax(d, 1e-300));
      wx[r] = vx * inv[r];
      wy[r] = vy * inv[r];
    }
  if (ok) {
    double ax = 1.0, ay = 1.0, b = rij;
#pragma unroll (kUnr<LA>)
    for (int q = 0; q < LA; ++q)
      if (q < l) {
        ax -= wx[q] * wx[q];
        ay -= wy[q] * wy[q];
        b -= wx[q] * wy[q];
      }
    if (ax > 1e-10 && ay > 1e-10) return decide_of_r(I, b * rsqrt(ax * ay), false, pv);
  }
  return exact_remove<LA>(I, i, j, ids, l, pv);  // pinv semantics
}

// Running FP32 factorisation of the conditioning block of one lane's current test,
// kept across the lexicographic walk: the Cholesky factor of S (rows, inverse
// diagonal, pivots) and the forward solves w_i, w_j.
template <int LA>
struct Fact {
  float Lm[LA * (LA + 1) / 2 > 0 ? LA * (LA + 1) / 2 : 1];
  float invd[LA], piv[LA], wx[LA], wy[LA];
};

// FP32 test of (i, j | ids). The partial correlation comes from a Cholesky
// factorisation of the S block and forward solves for r_iS and r_jS:
//   r = (r_ij - w_i . w_j) / sqrt((1 - |w_i|^2)(1 - |w_j|^2)),  w = L_S^-1 r_S;
// only rows ci..l-1 are refactored (rows below ci are still valid for the current
// i, j and the unchanged first ci members of S). Returns 1 = remove, 0 = keep,
// 2 = undecided (re-test in FP64): |r| is compared with r_c outside a band of
// margin_r + 8 * ke(l) / smallest pivot. *rr_out receives |r|.
// The entries are read from C at [x * stride + y]: the instance's FP32 matrix with
// variable ids (C = cor32, stride = p, xi = i, xj = j, xs = ids), or a row's block
// staged in shared memory with block-local indices (a generic pointer; the same FP32
// values, so the same decisions).
template <int LA>
__device__ __forceinline__ int test_f32_inc(const Inst &I, const float *__restrict__ C, int64_t stride, int64_t xi,
                                            int64_t xj, const int *xs, int l, int ci, Fact<LA> &F, float *rr_out) {
  // unrolled levels (LA <= 8): all entries the changed rows need are gathered before
  // any arithmetic (one round of independent loads instead of one per factor row); the
  // generic level kernel loads row by row (its 16-wide arrays would live in local
  // memory)
  constexpr bool kGather = LA <= 8;
  constexpr int kG = kGather ? LA : 1;
  float gx[kG], gy[kG], gs[kG * (kG - 1) / 2 > 0 ? kG * (kG - 1) / 2 : 1];
  if constexpr (kGather) {
#pragma unroll (kUnr<LA>)
    for (int r = 0; r < LA; ++r) {
      if (r >= ci && r < l) {
        const int64_t xr = xs[r];
        gx[r] = C[xi * stride + xr];
        gy[r] = C[xj * stride + xr];
#pragma unroll (kUnr<LA>)
        for (int c = 0; c < LA; ++c)
          if (c < r) gs[r * (r - 1) / 2 + c] = C[(int64_t)xs[c] * stride + xr];
      }
    }
  }
  const float rij = C[xi * stride + xj];
#pragma unroll (kUnr<LA>)
  for (int r = 0; r < LA; ++r) {
    if (r >= ci && r < l) {
      const int64_t xr = xs[r];
      float vx, vy;
      if constexpr (kGather) {
        vx = gx[r];
        vy = gy[r];
      } else {
        vx = C[xi * stride + xr];
        vy = C[xj * stride + xr];
      }
      float d = 1.0f;
#pragma unroll (kUnr<LA>)
      for (int c = 0; c < LA; ++c) {
        if (c < r) {
          float v;
          if constexpr (kGather)
            v = gs[r * (r - 1) / 2 + c];
          else
            v = C[(int64_t)xs[c] * stride + xr];
#pragma unroll (kUnr<LA>)
          for (int q = 0; q < LA; ++q)
            if (q < c) v -= F.Lm[r * (r + 1) / 2 + q] * F.Lm[c * (c + 1) / 2 + q];
          v *= F.invd[c];
          F.Lm[r * (r + 1) / 2 + c] = v;
          d -= v * v;
          vx -= v * F.wx[c];
          vy -= v * F.wy[c];
        }
      }
      const float id = rsqrtf(fmaxf(d, 1e-30f));
      F.piv[r] = d;
      F.invd[r] = id;
      F.wx[r] = vx * id;
      F.wy[r] = vy * id;
    }
  }
  // the sums in row order, whatever ci was, so that the decision does not depend on
  // the walk
  float sx = 0.f, sy = 0.f, sxy = 0.f, dmin = 1.f;
#pragma unroll (kUnr<LA>)
  for (int r = 0; r < LA; ++r)
    if (r < l) {
      dmin = fminf(dmin, F.piv[r]);
      sx += F.wx[r] * F.wx[r];
      sy += F.wy[r] * F.wy[r];
      sxy += F.wx[r] * F.wy[r];
    }
  const float ax = 1.0f - sx, ay = 1.0f - sy;
  const float cond = fminf(dmin, fminf(ax, ay));
  if (!(cond > 1e-3f)) return 2;
  const float rr = fabsf(rij - sxy) * rsqrtf(ax * ay);
  *rr_out = rr;
  const float dist = rr - I.r_c;
  const float ke = I.ke_a + (float)(l + 2) * I.ke_b;
  const float band = I.margin_r + 8.0f * __fdividef(ke, cond);
  if (!(fabsf(dist) > band)) return 2;
  return dist < 0.0f ? 1 : 0;
}

// Rows of degree up to kBlkD have their correlation block -- the row variable and its
// neighbours, (d + 1)^2 FP32 entries -- staged in shared memory by the warp whose tile
// starts in the row (levels 2-16 of the mixed-precision kernels): every test of the row
// reads only that block (the row, the edge's other end and the conditioning set are all
// among them), so the gathers of a test come from shared memory instead of L2/HBM.
// Block-local index 0 is the row itself, k + 1 its k-th neighbour in the snapshot.
constexpr int kBlkD = 31, kBlkS = kBlkD + 1;

// Stage the block of row i of instance I (whole warp, converged; d + 1 <= 32 lanes hold
// the block's variable ids): row a of the block is one gather of d + 1 entries.
__device__ __forceinline__ void stage_block(const Inst &I, int64_t i, int d, float *__restrict__ B) {
  const int lane = threadIdx.x & 31;
  const int base = I.rowptr[i];
  const int gid = lane == 0 ? (int)i : (lane <= d ? I.colidx[base + lane - 1] : 0);
  const float *__restrict__ C = I.cor32;
  __syncwarp();
#pragma unroll 4
  for (int a = 0; a <= d; ++a) {
    const int ga = __shfl_sync(0xffffffffu, gid, a);
    if (lane <= d) B[a * kBlkS + lane] = __ldg(C + (int64_t)ga * I.p + gid);
  }
  __syncwarp();
}

__device__ __forceinline__ int64_t find_row(const unsigned long long *row_work, int64_t p, unsigned long long t) {
  // largest i with row_work[i] <= t (row_work is non-decreasing, row_work[p] > t)
  int64_t lo = 0, hi = p;
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) >> 1;
    if (row_work[mid] <= t) lo = mid; else hi = mid;
  }
  return lo;
}

// find_row for a position at or after the start of row i0 (t >= row_work[i0]): the
// lanes walk forward through the flattened space, so the row is usually i0 + 1 or a
// few rows on; a galloping probe finds it in O(log distance) loads instead of the
// log2(p) of a search over all rows.
__device__ __forceinline__ int64_t find_row_from(const unsigned long long *row_work, int64_t p, int64_t i0,
                                                 unsigned long long t) {
  int64_t lo = i0, step = 1;  // row_work[lo] <= t
  while (lo + step < p && row_work[lo + step] <= t) {
    lo += step;
    step <<= 1;
  }
  int64_t hi = min(lo + step, p);  // row_work[hi] > t (row_work[p] > t)
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) >> 1;
    if (row_work[mid] <= t) lo = mid; else hi = mid;
  }
  return lo;
}

// The row offsets of a single-instance level copied into shared memory by the whole
// block (one round of coalesced loads), so that every row search of the CI tests
// stays on the SM; null when the launch has no cache (several instances, or more than
// kRowCache - 1 rows: the shared memory is then left to the L1 cache).
__device__ __forceinline__ const unsigned long long *cache_row_work(const Launch &L, unsigned long long *smem) {
  if (!smem || !L.row_cache) return nullptr;
  const Inst &I = *inst_of(L, 0);
  for (int64_t r = threadIdx.x; r <= I.p; r += blockDim.x) smem[r] = __ldcg(I.row_work + r);
  __syncthreads();
  return smem;
}

// Row of a warp-uniform position t: a 32-ary search (coalesced probes, two or three
// rounds for thousands of rows) instead of log2(p) dependent loads. Whole warp.
__device__ __forceinline__ int64_t warp_find_row(const unsigned long long *rw, int64_t p, unsigned long long t) {
  const int lane = threadIdx.x & 31;
  int64_t lo = 0, hi = p;  // rw[lo] <= t < rw[hi]
  while (hi - lo > 32) {
    const int64_t step = (hi - lo + 31) >> 5;
    const int64_t probe = lo + (int64_t)(lane + 1) * step;
    const bool le = probe < hi && rw[probe] <= t;
    lo += (int64_t)__popc(__ballot_sync(0xffffffffu, le)) * step;
    hi = min(hi, lo + step);
  }
  const int64_t probe = lo + 1 + lane;
  const bool le = probe < hi && rw[probe] <= t;
  return lo + __popc(__ballot_sync(0xffffffffu, le));
}

// Row of each lane's position t >= t0, given i0 = the row of t0 (same instance): the
// next 32 row offsets in one coalesced load and a shuffle search; a lane further on
// (rows without tests in between) searches alone. Whole warp; `valid` lanes only use
// the result.
__device__ __forceinline__ int64_t lane_find_row(const unsigned long long *rw, int64_t p, int64_t i0,
                                                 unsigned long long t, bool valid) {
  const int lane = threadIdx.x & 31;
  const int64_t r = i0 + 1 + lane;
  const unsigned long long v = r <= p ? rw[r] : ~0ull;
  int pos = 0;  // number of the 32 offsets <= t (up to 31 here)
#pragma unroll
  for (int sh = 16; sh >= 1; sh >>= 1) {
    const unsigned long long vv = __shfl_sync(0xffffffffu, v, pos + sh - 1);
    if (vv <= t) pos += sh;
  }
  const unsigned long long v31 = __shfl_sync(0xffffffffu, v, 31);
  if (valid && v31 <= t) return find_row(rw, p, t);
  return i0 + pos;
}

// Removals: the lane whose atomicAnd clears the (min, max) bit owns the edge and clears
// the mirror bit at once (other tests see the edge gone); its separation-set record
// waits in the warp's shared-memory list until the tile is done, so that one
// record-counter atomic per instance and flush replaces one per removal.
constexpr int kPend = 32;
template <int LA>
struct PendRem {
  int32_t lo, hi, b, pad;
  double pv;
  int32_t ids[LA > 0 ? LA : 1];
};

// MARK: the removal marks both rows' neighbour lists stale (every removal outside level
// 1, whose launch leaves the snapshot invalid instead: its 4 M removals on a batch of 512
// instances of p 20-800 made the marks cost a third of the level-1 kernel)
template <bool MARK = true>
__device__ __forceinline__ bool claim_edge(const Inst &I, int64_t i, int64_t j) {
  const int64_t lo = i < j ? i : j, hi = i < j ? j : i;
  const uint32_t bit = 1u << (hi & 31);
  const uint32_t old = atomicAnd(I.adj + lo * I.W + (hi >> 5), ~bit);
  if (!(old & bit)) return false;  // another test removed it first
  atomicAnd(I.adj + hi * I.W + (lo >> 5), ~(1u << (lo & 31)));
  if (MARK && I.dirty) {  // both rows' neighbour lists are stale from here on
    I.dirty[lo] = 1;
    I.dirty[hi] = 1;
  }
  return true;
}

// the record of a removal this lane owns (claim_edge returned true)
__device__ __forceinline__ void write_record(const Inst &I, int level, int64_t i, int64_t j, const int *ids, int l,
                                             double pv) {
  atomicAdd(&I.ctr[level].deleted, 1ull);
  const unsigned long long slot = atomicAdd(&I.g->rec_count, 1ull);
  if ((long long)slot >= I.rec_cap) {
    atomicOr(&I.g->err, kErrRecOverflow);
    return;
  }
  int32_t *rec = I.recs + slot * (unsigned long long)I.rec_stride;
  RecHead *h = reinterpret_cast<RecHead *>(rec);
  h->i = (int32_t)(i < j ? i : j);
  h->j = (int32_t)(i < j ? j : i);
  h->level = l;
  h->pad = 0;
  h->pmax = pv;
  for (int q = 0; q < I.rec_ids; ++q) rec[kRecHeadWords + q] = q < l ? ids[q] : -1;
}

template <int LA>
__device__ __forceinline__ void push_pending(PendRem<LA> *list, int *np, const Inst &I, int b, int level, int64_t i,
                                             int64_t j, const int *ids, int l, double pv) {
  const int slot = atomicAdd(np, 1);
  if (slot >= kPend) {  // list full: record at once
    write_record(I, level, i, j, ids, l, pv);
    return;
  }
  PendRem<LA> &e = list[slot];
  e.lo = (int32_t)(i < j ? i : j);
  e.hi = (int32_t)(i < j ? j : i);
  e.b = b;
  e.pad = 0;
  e.pv = pv;
#pragma unroll (kUnr<LA>)
  for (int q = 0; q < (LA > 0 ? LA : 1); ++q) e.ids[q] = q < l ? ids[q] : -1;
}

// Apply a warp's pending removals (whole warp, converged).
template <int LA>
__device__ __forceinline__ void flush_pending(const Launch &L, int level, PendRem<LA> *list, int *np) {
  const int lane = threadIdx.x & 31;
  __syncwarp();
  const int n = min(*np, kPend);
  for (int q0 = 0; q0 < n; q0 += 32) {
    const int q = q0 + lane;
    const bool won = q < n;
    const Inst *I = nullptr;
    int b = -1;
    if (won) {
      b = list[q].b;
      I = inst_of(L, b);
    }
    const unsigned wm = __ballot_sync(0xffffffffu, won);
    if (won) {
      const unsigned g = __match_any_sync(wm, b);
      const int leader = __ffs(g) - 1;
      unsigned long long base = 0;
      if (lane == leader) {
        base = atomicAdd(&I->g->rec_count, (unsigned long long)__popc(g));
        atomicAdd(&I->ctr[level].deleted, (unsigned long long)__popc(g));
      }
      base = __shfl_sync(g, base, leader);
      const unsigned long long slot = base + (unsigned long long)__popc(g & ((1u << lane) - 1u));
      if ((long long)slot >= I->rec_cap) {
        atomicOr(&I->g->err, kErrRecOverflow);
      } else {
        const PendRem<LA> &e = list[q];
        int32_t *rec = I->recs + slot * (unsigned long long)I->rec_stride;
        RecHead *h = reinterpret_cast<RecHead *>(rec);
        h->i = e.lo;
        h->j = e.hi;
        h->level = level;
        h->pad = 0;
        h->pmax = e.pv;
        const int nid = I->rec_ids;
#pragma unroll (kUnr<LA>)
        for (int t = 0; t < (LA > 0 ? LA : 1); ++t)
          if (t < nid) rec[kRecHeadWords + t] = e.ids[t];
        for (int t = (LA > 0 ? LA : 1); t < nid; ++t) rec[kRecHeadWords + t] = -1;
      }
    }
  }
  __syncwarp();
  if (lane == 0) *np = 0;
  __syncwarp();
}

// Defer an undecided test to the FP64 re-test kernel; false when the queue is full.
__device__ __forceinline__ bool push_retest(const Launch &L, int b, int64_t i, int64_t j, const int *ids, int l) {
  const unsigned long long slot = atomicAdd(&L.lc->rq_count, 1ull);
  if ((long long)slot >= L.rq_cap) return false;
  RetestItem *it = L.rq + slot;
  it->i = (int32_t)i;
  it->j = (int32_t)j;
  it->level = l;
  it->inst = b;
  for (int q = 0; q < HPC_MAX_LEVEL; ++q) it->ids[q] = q < l ? ids[q] : -1;
  return true;
}

// The level's tile policy: the forced one, else the context's table entry for (largest
// p, level, largest degree at the level start), else the defaults. Read after the
// scan phase's grid barrier (the degree is formed there).
__device__ __forceinline__ TuneEntry tile_policy(const Launch &L) {
  TuneEntry te = L.force;
  if (te.tile_cap <= 0 && L.tune) {
    const int md = *(volatile const int *)&L.lc->max_deg;
    te = L.tune[((size_t)L.p_bucket * (HPC_MAX_LEVEL + 1) + L.level) * kTuneDB + tune_bucket(md, kTuneDB)];
  }
  if (te.tile_cap <= 0) te = TuneEntry{kTuneDefaultCap, kTuneDefaultTpl, kTuneDefaultEdgeLanes, 0};
  te.tiles_per_lane = max(1, te.tiles_per_lane);
  return te;
}

// tests per lane per tile: about te.tiles_per_lane tiles per lane of the grid, at most
// te.tile_cap; a level with at most tiles_per_lane tests per lane runs in one round of
// tiles (one set-up per warp; the lane's further tests are successor steps)
__device__ __forceinline__ int tile_tests_per_lane(unsigned long long total, unsigned long long lanes,
                                                   const TuneEntry &te, bool one_round) {
  const unsigned long long tpl = (unsigned long long)te.tiles_per_lane;
  if (one_round && total <= lanes * tpl) return (int)((total + lanes - 1) / lanes);
  return (int)max(1ull, min((unsigned long long)te.tile_cap, total / (lanes * tpl)));
}

// Tiles are claimed in increasing order (tile = nwarps + counter), so once an edge is
// removed, every tile lying wholly inside its remaining tests holds nothing to do:
// raising the counter to the tile that holds the edge's end (which may hold tests of
// the next edge, so it is still claimed) skips them all. edge_end and tile_end are
// positions in the level's flattened test space; only tiles after the caller's own
// are affected.
__device__ __forceinline__ void skip_tiles_of_edge(const Launch &L, unsigned long long edge_end,
                                                   unsigned long long tile_end, unsigned long long per_tile,
                                                   unsigned long long nwarps) {
  if (edge_end <= tile_end) return;
  const unsigned long long target = edge_end / per_tile;
  if (target > nwarps) atomicMax(&L.lc->tile_next, target - nwarps);
}

// Shared memory of a level kernel's CI-test phase: per warp, the pending removals and
// (mixed precision: levels 2-16 of the edge order, every set-order level) the staged
// correlation block.
template <int LT, bool MIXED>
struct TestSmem {
  static constexpr int LA = LT > 0 ? LT : HPC_MAX_LEVEL;
  static constexpr bool kBlk = MIXED && LT >= 2 && LT <= kSetTop;
  PendRem<LA> pend[kThreads / 32][kPend];
  int np[kThreads / 32];
  float blk[kBlk ? kThreads / 32 : 1][kBlk ? kBlkS * kBlkS : 1];
};

template <int LT, bool MIXED>
__device__ __forceinline__ void tests_generic(const Launch &L, unsigned long long *rw_smem, const TuneEntry &te,
                                              TestSmem<LT, MIXED> &sm) {
  constexpr int LA = LT > 0 ? LT : HPC_MAX_LEVEL;
  const int l = LT > 0 ? LT : L.level;
  const int level = L.level;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  // the staged correlation block of the warp (levels 2-16, mixed precision)
  constexpr bool kBlk = TestSmem<LT, MIXED>::kBlk;
  float *blk = sm.blk[kBlk ? wib : 0];
  int64_t blk_i = -1;  // row and instance of the staged block
  int blk_b = -1;
  PendRem<LA> *pend = sm.pend[wib];
  int *np = sm.np + wib;
  if (lane == 0) *np = 0;
  __syncwarp();
  const unsigned long long total = L.work_prefix[L.count];
  if (total == 0) return;
  const unsigned long long *rw_c = cache_row_work(L, rw_smem);
  const unsigned long long lanes = (unsigned long long)gridDim.x * blockDim.x;
  const int m = tile_tests_per_lane(total, lanes, te, true);
  const unsigned long long per_tile = 32ull * (unsigned long long)m;
  int pos[LA], ids[LA];
  // the first tile of every warp is its global index, later tiles come from the
  // device-wide counter (one atomic round trip fewer per warp)
  const unsigned long long nwarps = lanes >> 5;
  bool first_tile = true;
  for (;;) {
    unsigned long long tile = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) >> 5;
    if (!first_tile) {
      if (lane == 0) tile = nwarps + atomicAdd(&L.lc->tile_next, 1ull);
      tile = __shfl_sync(0xffffffffu, tile, 0);
    }
    first_tile = false;
    const unsigned long long t0 = tile * per_tile;
    if (t0 >= total) break;
    unsigned long long t = t0 + (unsigned long long)lane * m;
    const unsigned long long tend = min(t + (unsigned long long)m, total);
    unsigned executed = 0, retests = 0;
    int b_last = -1;
    // instance and row of the tile start (whole warp), then each lane's row
    int b = find_inst_u(L.work_prefix, L.count, t0);
    const Inst *I = inst_of(L, b);
    unsigned long long base_t = L.work_prefix[b];
    const int64_t i0 = warp_find_row(rw_c ? rw_c : I->row_work, I->p, t0 - base_t);
    if (kBlk && (i0 != blk_i || b != blk_b)) {  // the block of the tile's first row
      const int d0 = I->deg[i0];
      if (d0 <= kBlkD) {
        stage_block(*I, i0, d0, blk);
        blk_i = i0;
        blk_b = b;
      }
    }
    const bool active = t < tend;
    const bool same = t < L.work_prefix[b + 1];
    int64_t i = lane_find_row(rw_c ? rw_c : I->row_work, I->p, i0, (active && same ? t : t0) - base_t, active && same);
    if (active && !same) {  // the tile runs into the next instance
      b = find_inst_u(L.work_prefix, L.count, t);
      I = inst_of(L, b);
      base_t = L.work_prefix[b];
      i = find_row(rw_c ? rw_c : I->row_work, I->p, t - base_t);
    }
    if (active) {
      int d = I->deg[i];
      unsigned long long c = binom_fast(d - 1, l);
      const unsigned long long off = t - base_t - (rw_c ? rw_c : I->row_work)[i];
      int s = (int)(off / c);
      unsigned long long rank = off - (unsigned long long)s * c;
      int base = I->rowptr[i];
      int64_t j = I->colidx[base + s];
      bool alive = live_bit(I->adj, I->W, i, j);
      // a removed edge needs no subset: its rest is skipped below, and when the whole
      // tile lies inside it, so are the edge's further tiles
      if (alive) unrank_lex_fast(rank, l, d - 1, pos);
      else if (lane == 0) skip_tiles_of_edge(L, t - rank + c, t0 + per_tile, per_tile, nwarps);
      unsigned tested_edge = 0;
      int ci = 0;  // lowest position changed since the last test (rows below are valid)
      Fact<LA> F;
      for (;;) {
        if (alive) {
#pragma unroll (kUnr<LA>)
          for (int q = 0; q < LA; ++q)
            if (q < l && q >= ci) ids[q] = I->colidx[base + pos[q] + (pos[q] >= s ? 1 : 0)];
          int res = 2;
          float rr = 0.f;
          if (MIXED) {
            if (kBlk && i == blk_i && b == blk_b) {  // from the staged block, block-local indices
              int lids[LA];
#pragma unroll (kUnr<LA>)
              for (int q = 0; q < LA; ++q)
                if (q < l) lids[q] = pos[q] + (pos[q] >= s ? 1 : 0) + 1;
              res = test_f32_inc<LA>(*I, blk, kBlkS, 0, s + 1, lids, l, ci, F, &rr);
            } else {
              res = test_f32_inc<LA>(*I, I->cor32, I->p, i, j, ids, l, ci, F, &rr);
            }
          }
          ci = l;
          ++executed;
          ++tested_edge;
          bool rm = false;
          double pv = 0.0;
          if (res == 1) {
            // decided in FP32; the p-value is evaluated when the records are read
            // (the negative value carries |r| for instances without an FP64 matrix)
            rm = true;
            pv = -1.0 - (double)rr;
          } else if (res == 2) {
            if (MIXED) ++retests;
            if (!(MIXED && !I->cor64 && push_retest(L, b, i, j, ids, l))) rm = exact_remove_fast<LA>(*I, i, j, ids, l, &pv);
          }
          if (rm) {
            if (claim_edge<LT != 1>(*I, i, j)) {
              push_pending<LA>(pend, np, *I, b, level, i, j, ids, l, pv);
              skip_tiles_of_edge(L, t - rank + c, t0 + per_tile, per_tile, nwarps);
            }
            alive = false;
          }
        }
        if (!alive) {  // the rest of a removed edge
          t += c - 1ull - rank;
          rank = c - 1ull;
        }
        if (++t >= tend) break;
        if (++rank == c) {
          rank = 0;
          if (++s == d) {
            // next row with tests, possibly of the next instance
            if (t >= L.work_prefix[b + 1]) {
              b = find_inst_u(L.work_prefix, L.count, t);
              I = inst_of(L, b);
              base_t = L.work_prefix[b];
              i = find_row(rw_c ? rw_c : I->row_work, I->p, t - base_t);
            } else {
              i = find_row_from(rw_c ? rw_c : I->row_work, I->p, i, t - base_t);
            }
            d = I->deg[i];
            c = binom_fast(d - 1, l);
            base = I->rowptr[i];
            s = 0;
          }
#pragma unroll (kUnr<LA>)
          for (int q = 0; q < LA; ++q)
            if (q < l) pos[q] = q;
          j = I->colidx[base + s];
          alive = live_bit(I->adj, I->W, i, j);
          tested_edge = 0;
          ci = 0;
        } else {
          const int changed = next_lex(l, d - 1, pos);
          ci = min(ci, changed);
          if (alive && (tested_edge & 3u) == 0) alive = live_bit(I->adj, I->W, i, j);
        }
      }
      b_last = b;
    }
    __syncwarp();
    flush_pending<LA>(L, level, pend, np);
    // per-instance test counts, one atomic per instance present in the warp (a
    // lane's range rarely crosses instances: its counts go to its last instance)
    const unsigned grp = __match_any_sync(0xffffffffu, b_last);
    const unsigned ex = __reduce_add_sync(grp, executed);
    const unsigned rt = __reduce_add_sync(grp, retests);
    if (b_last >= 0 && lane == __ffs(grp) - 1) {
      atomicAdd(&inst_of(L, b_last)->ctr[level].tests, (unsigned long long)ex);
      if (rt) atomicAdd(&inst_of(L, b_last)->ctr[level].retests, (unsigned long long)rt);
    }
  }
}

// Level 1, lane-interleaved: lane q of a warp takes tests t0 + q, t0 + q + 32, ... of
// its tile, so the 32 lanes work on consecutive conditioning variables of the same
// edge (i, j): their reads of the neighbour list and of row i of cor32 fall into few
// cache lines and stay in L1 across the edges of row i, and only the reads of row j
// are scattered. Decisions as test_f32_inc with l = 1 (the closed form of cpuInd.cpp:16-27
// in FP32), FP64 re-tests as in citest_kernel. QO (queue only, mixed precision without
// an FP64 matrix): an undecided test is only queued, and a full queue is flagged for a
// rerun as in the set order -- the kernel then holds no inline FP64 re-test, whose
// registers the interleaved body would otherwise spill for.
template <bool MIXED, bool PF, bool QO = false>
__device__ __forceinline__ void tests_l1(const Launch &L, unsigned long long *rw_smem, const TuneEntry &te) {
  const int level = 1;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  __shared__ PendRem<1> s_pend[kThreads / 32][kPend];
  __shared__ int s_np[kThreads / 32];
  PendRem<1> *pend = s_pend[wib];
  int *np = s_np + wib;
  if (lane == 0) *np = 0;
  __syncwarp();
  const unsigned long long total = L.work_prefix[L.count];
  if (total == 0) return;
  const unsigned long long *rw_c = cache_row_work(L, rw_smem);
  const unsigned long long lanes = (unsigned long long)gridDim.x * blockDim.x;
  const int m = tile_tests_per_lane(total, lanes, te, false);
  const unsigned long long per_tile = 32ull * (unsigned long long)m;
  // the first tile of every warp is its global index, later tiles come from the
  // device-wide counter (one atomic round trip fewer per warp)
  const unsigned long long nwarps = lanes >> 5;
  bool first_tile = true;
  for (;;) {
    unsigned long long tile = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) >> 5;
    if (!first_tile) {
      if (lane == 0) tile = nwarps + atomicAdd(&L.lc->tile_next, 1ull);
      tile = __shfl_sync(0xffffffffu, tile, 0);
    }
    first_tile = false;
    const unsigned long long t0 = tile * per_tile;
    if (t0 >= total) break;
    const unsigned long long tend = min(t0 + per_tile, total);
    unsigned long long t = t0 + lane;
    unsigned executed = 0, retests = 0;
    int b_last = -1;
    // instance and row of the tile start (whole warp), then each lane's row
    int b = find_inst_u(L.work_prefix, L.count, t0);
    const Inst *I = inst_of(L, b);
    unsigned long long base_t = L.work_prefix[b];
    const int64_t i0 = warp_find_row(rw_c ? rw_c : I->row_work, I->p, t0 - base_t);
    const bool active = t < tend;
    const bool same = t < L.work_prefix[b + 1];
    int64_t i = lane_find_row(rw_c ? rw_c : I->row_work, I->p, i0, (active && same ? t : t0) - base_t, active && same);
    if (active && !same) {  // the tile runs into the next instance
      b = find_inst_u(L.work_prefix, L.count, t);
      I = inst_of(L, b);
      base_t = L.work_prefix[b];
      i = find_row(rw_c ? rw_c : I->row_work, I->p, t - base_t);
    }
    if (active) {
      int d = I->deg[i];
      int c = d - 1;  // tests per edge at level 1
      unsigned long long off = t - base_t - (rw_c ? rw_c : I->row_work)[i];
      int s = (int)(off / (unsigned long long)c);
      int rank = (int)(off - (unsigned long long)s * c);
      int base = I->rowptr[i];
      int64_t j = I->colidx[base + s];
      float rij = MIXED ? __ldg(I->cor32 + i * I->p + j) : 0.f;
      // the live bit is read when the lane enters an edge and every fourth step on it
      // (removals by this warp reach its lanes through the step's ballot)
      bool live = live_bit(I->adj, I->W, i, j);
      if (!live && lane == 0) skip_tiles_of_edge(L, t - rank + c, tend, per_tile, nwarps);
      unsigned steps_on_edge = 0;
      // The entries are loaded before the live bit is known (in bounds either way): the
      // two round trips overlap instead of following each other. With PF (the prefetch
      // variant, for long edges) the entries of the next position on the same edge are
      // also loaded one step ahead -- its neighbour id before the test, its entries
      // before the step's ballots -- so that their round trip overlaps this step.
      int k = 0;
      float x2 = 0.f, x3 = 0.f;
      if (PF) {
        k = I->colidx[base + rank + (rank >= s ? 1 : 0)];
        if (MIXED) {
          x2 = __ldg(I->cor32 + i * I->p + k);
          x3 = __ldg(I->cor32 + j * I->p + k);
        }
      }
      for (;;) {
        int kn = 0;
        bool ahead = false;
        if (PF) {
          const int rn = rank + 32;
          ahead = rn < c;
          if (ahead) kn = I->colidx[base + rn + (rn >= s ? 1 : 0)];
        } else {
          k = I->colidx[base + rank + (rank >= s ? 1 : 0)];
          if (MIXED) {
            x2 = __ldg(I->cor32 + i * I->p + k);
            x3 = __ldg(I->cor32 + j * I->p + k);
          }
        }
        bool rm = false;
        double pv_rm = 0.0;
        if (live) {
          int res = 2;
          float rr = 0.f;
          if (MIXED) {
            const float ax = 1.0f - x2 * x2, ay = 1.0f - x3 * x3;
            const float cond = fminf(ax, ay);
            if (cond > 1e-3f) {
              rr = fabsf(rij - x2 * x3) * rsqrtf(ax * ay);
              const float dist = rr - I->r_c;
              const float band = I->margin_r + 8.0f * __fdividef(I->ke_a + 3.0f * I->ke_b, cond);
              if (fabsf(dist) > band) res = dist < 0.0f ? 1 : 0;
            }
          }
          ++executed;
          if (res == 1) {
            // decided in FP32; the p-value is evaluated when the records are read
            rm = true;
            pv_rm = -1.0 - (double)rr;
          } else if (res == 2) {
            if (MIXED) ++retests;
            if constexpr (QO) {
              if (!push_retest(L, b, i, j, &k, 1)) atomicOr(&I->g->err, kErrRetestOverflow);
            } else {
              if (!(MIXED && !I->cor64 && push_retest(L, b, i, j, &k, 1)))
                rm = exact_remove_fast<1>(*I, i, j, &k, 1, &pv_rm);
            }
          }
        }
        float x2n = 0.f, x3n = 0.f;
        if (PF && MIXED && ahead) {
          x2n = __ldg(I->cor32 + i * I->p + kn);
          x3n = __ldg(I->cor32 + j * I->p + kn);
        }
        {
          // lanes on the same edge learn of its removal in this step; one of them
          // claims the edge and keeps its record for the flush (the lanes' edges are
          // grouped only in the steps where some lane removes)
          const unsigned act = __activemask();
          const unsigned rall = __ballot_sync(act, rm);
          if (rall) {
            const unsigned grp = __match_any_sync(act, (unsigned)(t - (unsigned long long)rank));
            const unsigned rmask = rall & grp;
            if (rmask) {
              if (lane == __ffs(rmask) - 1 && claim_edge<false>(*I, i, j)) {
                push_pending<1>(pend, np, *I, b, level, i, j, &k, 1, pv_rm);
                skip_tiles_of_edge(L, t - rank + c, t0 + per_tile, per_tile, nwarps);
              }
              live = false;
            }
          }
        }
        // a removed edge is left at once: the lane moves to its first position of
        // the next edge (its positions are 32 apart)
        const int steps = live ? 1 : (c - rank + 31) >> 5;
        t += 32ull * (unsigned long long)steps;
        if (t >= tend) break;
        rank += 32 * steps;
        bool moved = false;
        while (rank >= c) {  // next edge (and row, and instance) along the flattened order
          rank -= c;
          moved = true;
          if (++s == d) {
            if (t >= L.work_prefix[b + 1]) {
              b = find_inst_u(L.work_prefix, L.count, t);
              I = inst_of(L, b);
              base_t = L.work_prefix[b];
              i = find_row(rw_c ? rw_c : I->row_work, I->p, t - base_t);
            } else {
              i = find_row_from(rw_c ? rw_c : I->row_work, I->p, i, t - base_t);
            }
            d = I->deg[i];
            c = d - 1;
            base = I->rowptr[i];
            off = t - base_t - (rw_c ? rw_c : I->row_work)[i];
            s = (int)(off / (unsigned long long)c);
            rank = (int)(off - (unsigned long long)s * c);
            break;
          }
        }
        if (moved) {
          j = I->colidx[base + s];
          if (MIXED) rij = __ldg(I->cor32 + i * I->p + j);
          live = live_bit(I->adj, I->W, i, j);
          steps_on_edge = 0;
          if (PF) {
            k = I->colidx[base + rank + (rank >= s ? 1 : 0)];
            if (MIXED) {
              x2 = __ldg(I->cor32 + i * I->p + k);
              x3 = __ldg(I->cor32 + j * I->p + k);
            }
          }
        } else {
          if (PF) {  // one step on the same edge: the position loaded ahead
            k = kn;
            x2 = x2n;
            x3 = x3n;
          }
          if (live && (++steps_on_edge & 3u) == 0) live = live_bit(I->adj, I->W, i, j);
        }
      }
      b_last = b;
    }
    __syncwarp();
    flush_pending<1>(L, level, pend, np);
    const unsigned grp = __match_any_sync(0xffffffffu, b_last);
    const unsigned ex = __reduce_add_sync(grp, executed);
    const unsigned rt = __reduce_add_sync(grp, retests);
    if (b_last >= 0 && lane == __ffs(grp) - 1) {
      atomicAdd(&inst_of(L, b_last)->ctr[level].tests, (unsigned long long)ex);
      if (rt) atomicAdd(&inst_of(L, b_last)->ctr[level].retests, (unsigned long long)rt);
    }
  }
}

// ---------------------------------------------------------------------------
// The set order of a level's CI tests (levels 2-24, mixed precision; the kSetOrder
// kernels, launched from the level set_order_from() on). The flattened index runs over (instance, row i, l-subset S of the row's snapshot neighbours in
// lexicographic order), and one unit runs the tests (i, j | S) for every live
// neighbour j outside S, in ascending order. A row of degree d > l has C(d, l) units
// holding C(d, l) (d - l) = d C(d - 1, l) tests: every test of the edge order once,
// each in the same FP32 arithmetic -- the Cholesky factor of S and w_i formed as
// test_f32_inc forms them (along the lexicographic walk, from the lowest changed
// member on), w_j by the same forward solve -- so the same decisions and the same
// re-test band. The factor and w_i are formed once per unit instead of once per test:
// a test costs the forward solve for r_jS (about l^2 / 2 FMAs) instead of the
// refactored rows (about l^2 / 2 per changed row, and a warp pays for its lane with
// the most changed rows). Removed edges are skipped when the lane knows of the
// removal: its own at once, the others' when it enters a row or a tile; unlike the
// edge order, a unit cannot skip the rest of one edge's tests, so the host picks the
// order from a level on where removals are rare. Rows of degree up to 64 keep the
// membership of S and the live neighbours as bit masks; wider rows test membership
// against the positions and read the live bit per test.
constexpr int kSetMaskD = 64;
template <int LT>
constexpr int kSetBlocks = LT <= 11 ? 2 : 1;  // resident blocks per SM the set-order kernels are compiled for

// Rows ci..l-1 of the Cholesky factor of the S block and of w_i = L_S^-1 r_iS: the
// operations of test_f32_inc without w_j.
// IdxT: int for the staged block in shared memory, int64_t for the instance's matrix.
template <int LA, typename IdxT>
__device__ __forceinline__ void factor_set(const float *__restrict__ C, IdxT stride, IdxT xi, const int *xs, int l,
                                           int ci, Fact<LA> &F) {
#pragma unroll (kUnr<LA>)
  for (int r = 0; r < LA; ++r) {
    if (r >= ci && r < l) {
      const IdxT xr = xs[r];
      float vx = C[xi * stride + xr];
      float d = 1.0f;
#pragma unroll (kUnr<LA>)
      for (int c = 0; c < LA; ++c) {
        if (c < r) {
          float v = C[(IdxT)xs[c] * stride + xr];
#pragma unroll (kUnr<LA>)
          for (int q = 0; q < LA; ++q)
            if (q < c) v -= F.Lm[r * (r + 1) / 2 + q] * F.Lm[c * (c + 1) / 2 + q];
          v *= F.invd[c];
          F.Lm[r * (r + 1) / 2 + c] = v;
          d -= v * v;
          vx -= v * F.wx[c];
        }
      }
      const float id = rsqrtf(fmaxf(d, 1e-30f));
      F.piv[r] = d;
      F.invd[r] = id;
      F.wx[r] = vx * id;
    }
  }
}

// The tail of test_f32_inc on a test's sums: sx = |w_i|^2, sy = |w_j|^2, sxy = w_i.w_j
// and dmin = the smallest pivot of S. 0: keep, 1: remove (FP32-decided, |r| in *rr_out),
// 2: inside the re-test band.
__device__ __forceinline__ int set_decide(const Inst &I, int l, float sx, float dmin, float rij, float sy, float sxy,
                                          float *rr_out) {
  const float ax = 1.0f - sx, ay = 1.0f - sy;
  const float cond = fminf(dmin, fminf(ax, ay));
  if (!(cond > 1e-3f)) return 2;
  const float rr = fabsf(rij - sxy) * rsqrtf(ax * ay);
  *rr_out = rr;
  const float dist = rr - I.r_c;
  const float ke = I.ke_a + (float)(l + 2) * I.ke_b;
  const float band = I.margin_r + 8.0f * __fdividef(ke, cond);
  if (!(fabsf(dist) > band)) return 2;
  return dist < 0.0f ? 1 : 0;
}

// FP32 test of (i, j | S) on the unit's factor: w_j by forward solve, then the tail of
// test_f32_inc (sx = |w_i|^2 and dmin = the smallest pivot, both in row order, come
// with the factor). Same return values.
template <int LA, typename IdxT>
__device__ __forceinline__ int test_set_j(const Inst &I, const float *__restrict__ C, IdxT stride, IdxT xi, IdxT xj,
                                          const int *xs, int l, const Fact<LA> &F, float sx, float dmin,
                                          float *rr_out) {
  float gy[LA], wy[LA];
#pragma unroll (kUnr<LA>)
  for (int r = 0; r < LA; ++r)
    if (r < l) gy[r] = C[xj * stride + xs[r]];
  const float rij = C[xi * stride + xj];
  float sy = 0.f, sxy = 0.f;
#pragma unroll (kUnr<LA>)
  for (int r = 0; r < LA; ++r)
    if (r < l) {
      float vy = gy[r];
#pragma unroll (kUnr<LA>)
      for (int c = 0; c < LA; ++c)
        if (c < r) vy -= F.Lm[r * (r + 1) / 2 + c] * wy[c];
      wy[r] = vy * F.invd[r];
      sy += wy[r] * wy[r];
      sxy += F.wx[r] * wy[r];
    }
  return set_decide(I, l, sx, dmin, rij, sy, sxy, rr_out);
}

// Two tests (i, j1 | S) and (i, j2 | S) of one unit side by side: each in exactly the
// operations of test_set_j, the two dependency chains of the forward solves interleaved
// (the single solve leaves the issue slots waiting on its own results).
template <int LA, typename IdxT>
__device__ __forceinline__ void test_set_j2(const Inst &I, const float *__restrict__ C, IdxT stride, IdxT xi,
                                            IdxT xj1, IdxT xj2, const int *xs, int l, const Fact<LA> &F, float sx,
                                            float dmin, int *res1, int *res2, float *rr1, float *rr2) {
  float g1[LA], g2[LA], w1[LA], w2[LA];
#pragma unroll (kUnr<LA>)
  for (int r = 0; r < LA; ++r)
    if (r < l) {
      g1[r] = C[xj1 * stride + xs[r]];
      g2[r] = C[xj2 * stride + xs[r]];
    }
  const float rij1 = C[xi * stride + xj1], rij2 = C[xi * stride + xj2];
  float sy1 = 0.f, sxy1 = 0.f, sy2 = 0.f, sxy2 = 0.f;
#pragma unroll (kUnr<LA>)
  for (int r = 0; r < LA; ++r)
    if (r < l) {
      float v1 = g1[r], v2 = g2[r];
#pragma unroll (kUnr<LA>)
      for (int c = 0; c < LA; ++c)
        if (c < r) {
          const float lrc = F.Lm[r * (r + 1) / 2 + c];
          v1 -= lrc * w1[c];
          v2 -= lrc * w2[c];
        }
      w1[r] = v1 * F.invd[r];
      w2[r] = v2 * F.invd[r];
      sy1 += w1[r] * w1[r];
      sxy1 += F.wx[r] * w1[r];
      sy2 += w2[r] * w2[r];
      sxy2 += F.wx[r] * w2[r];
    }
  *res1 = set_decide(I, l, sx, dmin, rij1, sy1, sxy1, rr1);
  *res2 = set_decide(I, l, sx, dmin, rij2, sy2, sxy2, rr2);
}

// Levels whose set-order tests run in pairs: 3-5 (measured on a batch of 512 instances of
// p 20-800 against the single loop, level by level: 10 % faster at level 3, 3 % at 5,
// even at 4; 7-9 % slower at 6-7 and 3-7 % at 12-14, where the second solve's registers
// crowd the schedule; 9-11 spill).
template <int LA>
constexpr bool kSetPairs = LA <= 5;

// live bits of row i's snapshot neighbours (bit q: the q-th; d <= kSetMaskD), read by
// one lane
__device__ __forceinline__ uint64_t row_live_mask(const Inst &I, int64_t i, int base, int d) {
  uint64_t m = 0;
  if (d > kSetMaskD) return m;
  for (int q = 0; q < d; ++q)
    if (live_bit(I.adj, I.W, i, I.colidx[base + q])) m |= 1ull << q;
  return m;
}

template <int LT>
__device__ __forceinline__ void tests_set(const Launch &L, unsigned long long *rw_smem, const TuneEntry &te,
                                          TestSmem<LT, true> &sm) {
  constexpr int LA = LT;
  constexpr int l = LT;
  const int level = L.level;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  float *blk = sm.blk[wib];
  int64_t blk_i = -1;  // row and instance of the staged block
  int blk_b = -1;
  uint64_t blk_live = 0;  // live bits of the staged row's neighbours, read when the tile starts
  PendRem<LA> *pend = sm.pend[wib];
  int *np = sm.np + wib;
  if (lane == 0) *np = 0;
  __syncwarp();
  const unsigned long long total = L.work_prefix[L.count];
  if (total == 0) return;
  const unsigned long long *rw_c = cache_row_work(L, rw_smem);
  const unsigned long long lanes = (unsigned long long)gridDim.x * blockDim.x;
  const int m = tile_tests_per_lane(total, lanes, te, true);
  const unsigned long long per_tile = 32ull * (unsigned long long)m;
  const unsigned long long nwarps = lanes >> 5;
  int pos[LA], xs[LA];
  bool first_tile = true;
  for (;;) {
    unsigned long long tile = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) >> 5;
    if (!first_tile) {
      if (lane == 0) tile = nwarps + atomicAdd(&L.lc->tile_next, 1ull);
      tile = __shfl_sync(0xffffffffu, tile, 0);
    }
    first_tile = false;
    const unsigned long long t0 = tile * per_tile;
    if (t0 >= total) break;
    unsigned long long t = t0 + (unsigned long long)lane * m;
    const unsigned long long tend = min(t + (unsigned long long)m, total);
    unsigned executed = 0, retests = 0;
    int b_last = -1;
    int b = find_inst_u(L.work_prefix, L.count, t0);
    const Inst *I = inst_of(L, b);
    unsigned long long base_t = L.work_prefix[b];
    const int64_t i0 = warp_find_row(rw_c ? rw_c : I->row_work, I->p, t0 - base_t);
    {  // the block of the tile's first row and its neighbours' live bits (whole warp)
      const int d0 = I->deg[i0];
      if (d0 <= kBlkD) {
        if (i0 != blk_i || b != blk_b) {
          stage_block(*I, i0, d0, blk);
          blk_i = i0;
          blk_b = b;
        }
        const int base0 = I->rowptr[i0];
        const bool lv = lane < d0 && live_bit(I->adj, I->W, i0, I->colidx[base0 + lane]);
        blk_live = __ballot_sync(0xffffffffu, lv);
      } else {
        blk_i = -1;
        blk_b = -1;
      }
    }
    const bool active = t < tend;
    const bool same = t < L.work_prefix[b + 1];
    int64_t i = lane_find_row(rw_c ? rw_c : I->row_work, I->p, i0, (active && same ? t : t0) - base_t, active && same);
    if (active && !same) {  // the tile runs into the next instance
      b = find_inst_u(L.work_prefix, L.count, t);
      I = inst_of(L, b);
      base_t = L.work_prefix[b];
      i = find_row(rw_c ? rw_c : I->row_work, I->p, t - base_t);
    }
    if (active) {
      int d = I->deg[i];
      int base = I->rowptr[i];
      unrank_lex_fast(t - base_t - (rw_c ? rw_c : I->row_work)[i], l, d, pos);
      bool staged = i == blk_i && b == blk_b;
      uint64_t live = staged ? blk_live : row_live_mask(*I, i, base, d);
      int ci = 0;  // lowest member changed since the last unit (factor rows below are valid)
      Fact<LA> F;
      // one unit: the factor of S (rows from ci on), then the tests. ST: the row's block
      // is staged (entries from shared memory by block-local index, 32-bit index
      // arithmetic), else the instance's matrix by variable id
      auto unit = [&](auto staged_c) {
        constexpr bool ST = decltype(staged_c)::value;
        using IdxT = typename std::conditional<ST, int, int64_t>::type;
        const float *C = ST ? blk : I->cor32;
        const IdxT stride = ST ? (IdxT)kBlkS : (IdxT)I->p;
        const IdxT xi = ST ? (IdxT)0 : (IdxT)i;
#pragma unroll (kUnr<LA>)
        for (int q = 0; q < LA; ++q)
          if (q >= ci) xs[q] = ST ? pos[q] + 1 : I->colidx[base + pos[q]];
        factor_set<LA, IdxT>(C, stride, xi, xs, l, ci, F);
        float sx = 0.f, dmin = 1.f;
#pragma unroll (kUnr<LA>)
        for (int r = 0; r < LA; ++r) {
          dmin = fminf(dmin, F.piv[r]);
          sx += F.wx[r] * F.wx[r];
        }
        // the unit's tests: neighbours q outside S, live as far as the lane knows
        // a test's outcome: a removal claims the edge (and the lane forgets j for its
        // later units), an undecided test goes to the re-test queue
        auto finish_q = [&](int q, IdxT xj, int res, float rr) {
          ++executed;
          if (res == 0) return;
          // removal or re-test: the variable ids of j and S
          const int64_t j = ST ? (int64_t)I->colidx[base + q] : (int64_t)xj;
          int ids[LA];
#pragma unroll (kUnr<LA>)
          for (int r = 0; r < LA; ++r) ids[r] = ST ? I->colidx[base + pos[r]] : xs[r];
          bool rm = false;
          double pv = 0.0;
          if (res == 1) {
            // decided in FP32; the p-value is evaluated when the records are read
            rm = true;
            pv = -1.0 - (double)rr;
          } else {
            // deferred to the FP64 re-test kernel (the set order runs only without an FP64
            // matrix); a full queue is flagged and the host reruns the skeleton in the edge
            // order, so the test is never decided here
            ++retests;
            if (!push_retest(L, b, i, j, ids, l)) atomicOr(&I->g->err, kErrRetestOverflow);
          }
          if (rm) {
            if (claim_edge(*I, i, j)) push_pending<LA>(pend, np, *I, b, level, i, j, ids, l, pv);
            if (q < kSetMaskD) live &= ~(1ull << q);
          }
        };
        auto xj_of = [&](int q) -> IdxT { return ST ? (IdxT)(q + 1) : (IdxT)I->colidx[base + q]; };
        auto test_q = [&](int q) {
          const IdxT xj = xj_of(q);
          float rr = 0.f;
          const int res = test_set_j<LA, IdxT>(*I, C, stride, xi, xj, xs, l, F, sx, dmin, &rr);
          finish_q(q, xj, res, rr);
        };
        if (ST || d <= kSetMaskD) {
          uint64_t in_s = 0;
#pragma unroll (kUnr<LA>)
          for (int r = 0; r < LA; ++r) in_s |= 1ull << pos[r];
          uint64_t todo = live & ~in_s;
          if constexpr (kSetPairs<LA>) {
            // in pairs, the outcomes taken in the order of the single loop
            while (todo) {
              const int q1 = __ffsll((long long)todo) - 1;
              todo &= todo - 1;
              if (!todo) {
                test_q(q1);
                break;
              }
              const int q2 = __ffsll((long long)todo) - 1;
              todo &= todo - 1;
              const IdxT x1 = xj_of(q1), x2 = xj_of(q2);
              int res1, res2;
              float rr1 = 0.f, rr2 = 0.f;
              test_set_j2<LA, IdxT>(*I, C, stride, xi, x1, x2, xs, l, F, sx, dmin, &res1, &res2, &rr1, &rr2);
              finish_q(q1, x1, res1, rr1);
              finish_q(q2, x2, res2, rr2);
            }
          } else {
            while (todo) {
              const int q = __ffsll((long long)todo) - 1;
              todo &= todo - 1;
              test_q(q);
            }
          }
        } else {
          for (int q = 0; q < d; ++q) {
            bool member = false;
#pragma unroll (kUnr<LA>)
            for (int r = 0; r < LA; ++r) member |= pos[r] == q;
            if (member || !live_bit(I->adj, I->W, i, I->colidx[base + q])) continue;
            test_q(q);
          }
        }
      };
      for (;;) {
        if (staged)
          unit(std::true_type{});
        else
          unit(std::false_type{});
        if (++t >= tend) break;
        ci = next_lex(l, d, pos);
        if (ci < 0) {  // the row's last set: the next row with tests, possibly of the next instance
          if (t >= L.work_prefix[b + 1]) {
            b = find_inst_u(L.work_prefix, L.count, t);
            I = inst_of(L, b);
            base_t = L.work_prefix[b];
            i = find_row(rw_c ? rw_c : I->row_work, I->p, t - base_t);
          } else {
            i = find_row_from(rw_c ? rw_c : I->row_work, I->p, i, t - base_t);
          }
          d = I->deg[i];
          base = I->rowptr[i];
#pragma unroll (kUnr<LA>)
          for (int q = 0; q < LA; ++q) pos[q] = q;
          ci = 0;
          staged = i == blk_i && b == blk_b;
          live = staged ? blk_live : row_live_mask(*I, i, base, d);
        }
      }
      b_last = b;
    }
    __syncwarp();
    flush_pending<LA>(L, level, pend, np);
    const unsigned grp = __match_any_sync(0xffffffffu, b_last);
    const unsigned ex = __reduce_add_sync(grp, executed);
    const unsigned rt = __reduce_add_sync(grp, retests);
    if (b_last >= 0 && lane == __ffs(grp) - 1) {
      atomicAdd(&inst_of(L, b_last)->ctr[level].tests, (unsigned long long)ex);
      if (rt) atomicAdd(&inst_of(L, b_last)->ctr[level].retests, (unsigned long long)rt);
    }
  }
}

// One level l >= 1: rebuild | grid barrier | scan | grid barrier | CI tests. LT = 1
// is the lane-interleaved level-1 body (V: kL1Prefetch loads one step ahead,
// kL1Chunked runs the chunked body of the higher levels; picked by the tile policy),
// LT = 2..16 the bodies unrolled for l = LT (V = kSetOrder: in the set order, LT up to
// kSetTop), LT = 0 the runtime-level body.
template <int LT, bool MIXED, int V = kL1Interleaved>
__global__ void __launch_bounds__(kThreads, V == kSetOrder ? kSetBlocks<LT> : (LT == 1 && (V & 3) != kL1Chunked ? 4 : 2))
    level_kernel(const __grid_constant__ Launch L) {
  extern __shared__ unsigned long long rw_smem[];  // kRowCache entries
  unsigned int epoch = 0;
  const bool stamp = blockIdx.x == 0 && threadIdx.x == 0;  // the phase times
  if (stamp) L.lc->t_entry = globaltimer_ns();
  rebuild_phase(L);
  if (!grid_barrier(L, epoch)) return;
  if (stamp) L.lc->t_rebuilt = globaltimer_ns();
  scan_phase(L, V == kSetOrder);
  if (!grid_barrier(L, epoch)) return;
  if (stamp) L.lc->t_scanned = globaltimer_ns();
  const TuneEntry te = tile_policy(L);
  if constexpr (V == kSetOrder) {
    static_assert(MIXED && LT >= 2 && LT <= kSetTop, "the set order runs levels 2-24 in mixed precision");
    __shared__ TestSmem<LT, true> sm;
    tests_set<LT>(L, rw_smem, te, sm);
  } else if constexpr (LT == 1 && (V & 3) != kL1Chunked) {  // level 1 keeps the SM's on-chip memory for L1 cache
    tests_l1<MIXED, (V & 3) == kL1Prefetch, (V & kQueueOnly) != 0>(L, nullptr, te);
  } else {
    __shared__ TestSmem<LT, MIXED> sm;
    tests_generic<LT, MIXED>(L, LT == 1 ? nullptr : rw_smem, te, sm);
  }
  __syncthreads();
  if (threadIdx.x == 0) atomicMax(&L.lc->t_end, globaltimer_ns());
}

}  // namespace

// level kernels of levels 9-32 (citest_l9.cu, citest_l13.cu, citest_l17.cu)
void *level_kernel_9_12(int level, bool mixed, bool set);
void *level_kernel_13_16(int level, bool mixed, bool set);
void *level_kernel_17_24_set(int level);
void *level_kernel_17_up(int level, bool mixed);

}  // namespace hpc
