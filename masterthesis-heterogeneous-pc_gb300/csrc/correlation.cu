// Correlation: column standardisation and the FP64 Gram, grouped over the instances
// of a context.
//
// Replaces gpuMeans / gpuSD / gpuPMCC (src/correlation/corHelper.cu:8-116), which
// launch one 64-thread block per (i, j) pair and re-read both columns for every pair.
// Here one block per variable standardises its column once (NaN-skipping mean, SD with
// the n-1 denominator, z = (x - mean) / sd, missing samples as 0 so that a product with
// a missing sample contributes nothing -- the reference's pairwise NaN skip,
// corHelper.cu:101) into the FP64 copy Z or, for the tensor-core Gram, into the
// split-BF16 operands (and z as an FP32 pair for the FP64 re-tests); the FP64
// correlation is the register- and shared-memory-tiled Gram C = Z^T Z / (n - 1) over
// upper-triangle 64 x 64 tiles, mirrored on write.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <type_traits>

#include "internal.cuh"

namespace hpc {
namespace {

constexpr int kStdThreads = 256;

// Error-free FP32 sum (Knuth's TwoSum): a + b == s + e exactly.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// x - mean as an unevaluated FP32 pair (dh + de), mean = mh + ml; the pair is exact up
// to the representation error of ml (2^-48 |mean|).
__device__ __forceinline__ void centre_f32(float xv, float mh, float ml, float &dh, float &de) {
  float h, e;
  two_sum(xv, -mh, h, e);
  two_sum(h, e - ml, dh, de);
}

// Warp sum of FP32 pairs (h + l), compensated: every lane ends with the total.
__device__ __forceinline__ void warp_sum_pair(float &h, float &l) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, h, o), ol = __shfl_xor_sync(0xffffffffu, l, o);
    float s, e;
    two_sum(h, oh, s, e);
    h = s;
    l = l + ol + e;
  }
}

// The scalars of one variable that the sample loops use, formed once per block by thread
// 0 (an FP64 division or square root is a long instruction sequence on this GPU's
// 1/64-rate FP64 pipe: in every thread of every block they would cost more than the
// sample loops). mean and inv_sd = 1 / sd in FP64; scale = 1 / sqrt(n - 1); FP32 pairs
// (h + l) of mean, inv_sd * scale (i*) and inv_sd (j*).
struct ColScalars {
  double mean, inv_sd, scale;
  float mh, ml, ih, il, jh, jl;
};

// Block-wide total of the warps' FP32 pairs (lane 0 of warp w stored them in rh[w],
// rl[w]), compensated in FP32, converted to FP64 once: thread 0 only. (Every FP64 warp
// instruction occupies the SM's FP64 unit for 16 cycles, whether one lane or 32 use it.)
__device__ __forceinline__ double warp_totals(const float *rh, const float *rl) {
  float h = 0.f, l = 0.f;
#pragma unroll
  for (int w = 0; w < kStdThreads / 32; ++w) {
    float s, e;
    two_sum(h, rh[w], s, e);
    h = s;
    l += rl[w] + e;
  }
  return (double)h + (double)l;
}
__device__ __forceinline__ double warp_totals(const double *red) {
  double t = 0.0;
#pragma unroll
  for (int w = 0; w < kStdThreads / 32; ++w) t += red[w];
  return t;
}

__device__ __forceinline__ void finish_scalars(double ss, long long n, int ref_compat, ColScalars &S) {
  // z = (x - mean) * (1 / sd): one multiply per sample instead of a division; 1 / sd by
  // rsqrt of the variance (within an ulp of 1 / sqrt, fewer FP64 instructions than a
  // square root and a division)
  if (ref_compat)  // corHelper.cu:75: sqrtf of (sum / (dim - 1.f))
    S.inv_sd = 1.0 / (double)sqrtf((float)(ss / (double)((float)n - 1.f)));
  else
    S.inv_sd = rsqrt(ss / (double)(n - 1));
  const double denom = ref_compat ? (double)((float)n - 1.f) : (double)(n - 1);
  S.scale = rsqrt(denom);
  const double inv = S.inv_sd * S.scale;
  S.ih = (float)inv;
  S.il = (float)(inv - (double)S.ih);
  S.jh = (float)S.inv_sd;
  S.jl = (float)(S.inv_sd - (double)S.jh);
}

// Column moments of FP32 samples with FP64-grade accuracy but FP32 arithmetic per sample
// (these loops touch every sample): compensated FP32 sums per thread and warp (TwoSum),
// the warps' pairs added in FP64. NaN samples are skipped, as cpuMeans / the reference's
// SD loop skip them.
__device__ __forceinline__ void column_scalars(const float *__restrict__ x, long long n, int ref_compat,
                                               ColScalars &S) {
  __shared__ float rh[kStdThreads / 32], rl[kStdThreads / 32];
  __shared__ long long redc[kStdThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float sh = 0.f, sl = 0.f;
  int cnt = 0;
  for (long long k = threadIdx.x; k < n; k += kStdThreads) {
    const float xv = x[k];
    if (xv == xv) {
      float s, e;
      two_sum(sh, xv, s, e);
      sh = s;
      sl += e;
      ++cnt;
    }
  }
  warp_sum_pair(sh, sl);
  cnt = __reduce_add_sync(0xffffffffu, cnt);
  if (lane == 0) {
    rh[wid] = sh;
    rl[wid] = sl;
    redc[wid] = cnt;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    long long c = 0;
    for (int w = 0; w < kStdThreads / 32; ++w) c += redc[w];
    S.mean = warp_totals(rh, rl) / (double)c;
    S.mh = (float)S.mean;
    S.ml = (float)(S.mean - (double)S.mh);
  }
  __syncthreads();
  const float mh = S.mh, ml = S.ml;
  float qh = 0.f, ql = 0.f;
  for (long long k = threadIdx.x; k < n; k += kStdThreads) {
    const float xv = x[k];
    if (xv == xv) {
      float dh, de;
      centre_f32(xv, mh, ml, dh, de);
      const float p = dh * dh;
      float pe = fmaf(dh, dh, -p);  // exact error of the square
      pe = fmaf(2.f * dh, de, pe);
      pe = fmaf(de, de, pe);
      float s, e;
      two_sum(qh, p, s, e);
      qh = s;
      ql += e + pe;
    }
  }
  warp_sum_pair(qh, ql);
  __syncthreads();  // rh, rl are reused
  if (lane == 0) {
    rh[wid] = qh;
    rl[wid] = ql;
  }
  __syncthreads();
  if (threadIdx.x == 0) finish_scalars(warp_totals(rh, rl), n, ref_compat, S);
  __syncthreads();
}

// FP64 samples: FP64 sums (two passes, as the reference's mean-then-SD loops)
__device__ __forceinline__ void column_scalars(const double *__restrict__ x, long long n, int ref_compat,
                                               ColScalars &S) {
  __shared__ double red[kStdThreads / 32];
  __shared__ long long redc[kStdThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  double s = 0.0;
  int cnt = 0;
  for (long long k = threadIdx.x; k < n; k += kStdThreads) {
    const double xv = x[k];
    if (!isnan(xv)) {
      s += xv;
      ++cnt;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  cnt = __reduce_add_sync(0xffffffffu, cnt);
  if (lane == 0) {
    red[wid] = s;
    redc[wid] = cnt;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    long long c = 0;
    for (int w = 0; w < kStdThreads / 32; ++w) c += redc[w];
    S.mean = warp_totals(red) / (double)c;
    S.mh = (float)S.mean;
    S.ml = (float)(S.mean - (double)S.mh);
  }
  __syncthreads();
  const double mean = S.mean;
  double q = 0.0;
  for (long long k = threadIdx.x; k < n; k += kStdThreads) {
    const double xv = x[k];
    if (!isnan(xv)) {
      const double d = xv - mean;
      q = fma(d, d, q);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
  __syncthreads();
  if (lane == 0) red[wid] = q;
  __syncthreads();
  if (threadIdx.x == 0) finish_scalars(warp_totals(red), n, ref_compat, S);
  __syncthreads();
}

// Outputs of the standardisation (compile-time, so that no sample loop carries a
// branch or an idle computation for an absent output):
//   kStdZ        Z: FP64 standardised samples
//   kStdSplitZ   Z and the split-BF16 planes of the tensor-core Gram (FP64 samples)
//   kStdSplitPair the split-BF16 planes and z as an unevaluated FP32 pair (zh + zl,
//                FP64-grade), formed with no FP64 instruction per sample (FP32 samples)
constexpr int kStdZ = 0, kStdSplitZ = 1, kStdSplitPair = 2;

// z = (x - mean) * inv as an FP32 pair from the centred pair (dh + de) and inv = ih + il:
// the product's rounding error is recovered exactly (fmaf), the cross terms are 2^-24
// of the result
__device__ __forceinline__ void scale_pair(float dh, float de, float ih, float il, float &zh, float &zl) {
  const float p = dh * ih;
  float e = fmaf(dh, ih, -p);
  e = fmaf(dh, il, fmaf(de, ih, e));
  zh = p + e;
  zl = e - (zh - p);
}

// grid: one block per variable of every instance (flattened over row_prefix).
template <typename TIn, int OUT>
__global__ void __launch_bounds__(kStdThreads) standardise_kernel(const TIn *__restrict__ X, StdArgs a,
                                                                  double *__restrict__ Z, float *__restrict__ ZP,
                                                                  long long zp_plane, __nv_bfloat16 *__restrict__ P) {
  constexpr bool kF32 = std::is_same<TIn, float>::value;
  static_assert(OUT != kStdSplitPair || kF32, "the FP32 pair output is formed from FP32 samples");
  const long long t = blockIdx.x;
  const int b = find_inst(a.row_prefix, a.count, t);
  const long long v = t - a.row_prefix[b];
  const long long n = a.n[b];
  const TIn *x = X + a.x_off[b] + v * n;
  __shared__ ColScalars S;
  column_scalars(x, n, a.ref_compat, S);
  const double mean = S.mean, inv_sd = S.inv_sd;
  if constexpr (OUT == kStdZ) {
    double *z = Z + a.z_off[b] + v * n;
    for (long long k = threadIdx.x; k < n; k += kStdThreads) {
      const double xv = (double)x[k];
      z[k] = isnan(xv) ? 0.0 : (xv - mean) * inv_sd;
    }
    return;
  }
  // split-BF16 operand of the tensor-core Gram: two planes T = [hi | lo] of
  // zs = z / sqrt(n - 1) (the Gram's producer pairs the planes: hi.hi + hi.lo + lo.hi +
  // lo.lo is the correlation). hi = bf16(zs), lo = bf16(zs - hi), the subtraction exact in
  // FP32. FP32 samples form zs in FP32 pairs (x - mean as dh + de, times 1 / sqrt(n - 1)
  // / sd as ih + il): within an ulp of the FP64 value. Two consecutive samples per
  // thread, so that the planes are written as 4-byte pairs.
  const double scale = S.scale;
  const float mh = S.mh, ml = S.ml, ih = S.ih, il = S.il, jh = S.jh, jl = S.jl;
  const long long n_pad = a.n_pad[b], K = a.kdim[b];
  __nv_bfloat16 *pr = P + a.tc_off[b] + v * K;
  double *z = OUT == kStdSplitZ ? Z + a.z_off[b] + v * n : nullptr;
  float *zh = OUT == kStdSplitPair ? ZP + a.z_off[b] + v * n : nullptr;
  float *zl = OUT == kStdSplitPair ? zh + zp_plane : nullptr;
  for (long long k = 2 * (long long)threadIdx.x; k < n_pad; k += 2 * kStdThreads) {
    float s2[2] = {0.f, 0.f};
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const long long kk = k + u;
      if (kk >= n) break;
      if constexpr (kF32) {
        const float xv = x[kk];
        float dh = 0.f, de = 0.f;
        if (xv == xv) centre_f32(xv, mh, ml, dh, de);
        s2[u] = fmaf(dh, ih, fmaf(dh, il, de * ih));
        if constexpr (OUT == kStdSplitPair) {
          float h, l;
          scale_pair(dh, de, jh, jl, h, l);
          zh[kk] = h;
          zl[kk] = l;
        } else {
          z[kk] = xv != xv ? 0.0 : ((double)xv - mean) * inv_sd;
        }
      } else {
        const double xv = x[kk];
        const double zv = isnan(xv) ? 0.0 : (xv - mean) * inv_sd;
        z[kk] = zv;
        s2[u] = (float)(zv * scale);
      }
    }
    const __nv_bfloat162 hi = __floats2bfloat162_rn(s2[0], s2[1]);
    const float2 hf = __bfloat1622float2(hi);
    const __nv_bfloat162 lo = __floats2bfloat162_rn(s2[0] - hf.x, s2[1] - hf.y);
    *reinterpret_cast<__nv_bfloat162 *>(pr + k) = hi;
    *reinterpret_cast<__nv_bfloat162 *>(pr + n_pad + k) = lo;
  }
}

// FP64 standardised samples from the FP32 pairs (zh + zl, exact in FP64)
__global__ void pair_to_f64_kernel(const float *__restrict__ zh, const float *__restrict__ zl, long long count,
                                   double *__restrict__ Z) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x)
    Z[i] = (double)zh[i] + (double)zl[i];
}

// FP64 Gram, 64 x 64 output tile per block, K staged 16 at a time through shared
// memory, 4 x 4 outputs per thread; blocks flattened over all instances' tiles.
constexpr int BM = 64, BK = 16, GT = 256;

__global__ void __launch_bounds__(GT) gram_f64_kernel(const double *__restrict__ Zall, double *__restrict__ Call,
                                                      GramArgs g) {
  const long long tt = blockIdx.x;
  const int b = find_inst(g.tile_prefix, g.count, tt);
  long long t = tt - g.tile_prefix[b];
  const long long p = g.p[b], n = g.n[b];
  const int nb = (int)((p + BM - 1) / BM);
  const double *Z = Zall + g.z_off[b];
  double *C = Call + g.c_off[b];
  const double denom = g.denom[b];
  int bi = 0;
  while (t >= nb - bi) {  // (bi, bj), bi <= bj, row-major over the upper triangle of tiles
    t -= nb - bi;
    ++bi;
  }
  const int bj = bi + (int)t;
  const long long a0 = (long long)bi * BM, b0 = (long long)bj * BM;
  __shared__ double As[BK][BM + 1];
  __shared__ double Bs[BK][BM + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
  for (long long k0 = 0; k0 < n; k0 += BK) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int idx = threadIdx.x + r * GT;  // 0..1023: 64 columns x 16 k per operand
      const int col = idx >> 4, kk = idx & 15;
      const long long k = k0 + kk;
      const long long va = a0 + col, vb = b0 + col;
      As[kk][col] = (va < p && k < n) ? Z[va * n + k] : 0.0;
      Bs[kk][col] = (vb < p && k < n) ? Z[vb * n + k] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      double av[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) av[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const long long ra = a0 + ty + 16 * i;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const long long cb = b0 + tx + 16 * j;
      if (ra < p && cb < p && ra <= cb) {
        const double v = acc[i][j] / denom;
        C[ra * p + cb] = v;
        C[cb * p + ra] = v;
      }
    }
  }
}

__global__ void to_f32_kernel(const double *__restrict__ C, int64_t count, float *__restrict__ C32) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    C32[i] = (float)C[i];
}

}  // namespace

long long gram_f64_tiles(int64_t p) {
  const long long nb = (p + BM - 1) / BM;
  return nb * (nb + 1) / 2;
}

hpc_status launch_standardise(const void *X, bool f32, const StdArgs &a, long long total_rows, double *Z,
                              float *ZP, long long zp_plane, __nv_bfloat16 *P, cudaStream_t s) {
  const unsigned grid = (unsigned)total_rows;
  if (!P) {
    if (!Z) return HPC_ERR_INVALID_ARG;
    if (f32)
      standardise_kernel<float, kStdZ><<<grid, kStdThreads, 0, s>>>((const float *)X, a, Z, nullptr, 0, nullptr);
    else
      standardise_kernel<double, kStdZ><<<grid, kStdThreads, 0, s>>>((const double *)X, a, Z, nullptr, 0, nullptr);
  } else if (ZP) {
    if (!f32) return HPC_ERR_INVALID_ARG;
    standardise_kernel<float, kStdSplitPair><<<grid, kStdThreads, 0, s>>>((const float *)X, a, nullptr, ZP, zp_plane, P);
  } else {
    if (!Z) return HPC_ERR_INVALID_ARG;
    if (f32)
      standardise_kernel<float, kStdSplitZ><<<grid, kStdThreads, 0, s>>>((const float *)X, a, Z, nullptr, 0, P);
    else
      standardise_kernel<double, kStdSplitZ><<<grid, kStdThreads, 0, s>>>((const double *)X, a, Z, nullptr, 0, P);
  }
  HPC_LAUNCH_CHECK("standardise_kernel");
  return HPC_OK;
}

hpc_status launch_pair_to_f64(const float *zh, const float *zl, long long count, double *Z, cudaStream_t s) {
  pair_to_f64_kernel<<<1024, 256, 0, s>>>(zh, zl, count, Z);
  HPC_LAUNCH_CHECK("pair_to_f64_kernel");
  return HPC_OK;
}

hpc_status launch_gram_f64(const double *Z, double *C, const GramArgs &a, long long total_tiles, cudaStream_t s) {
  gram_f64_kernel<<<(unsigned)total_tiles, GT, 0, s>>>(Z, C, a);
  HPC_LAUNCH_CHECK("gram_f64_kernel");
  return HPC_OK;
}

hpc_status launch_to_f32(const double *C, int64_t count, float *C32, cudaStream_t s) {
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((count + 255) / 256, 152 * 16));
  to_f32_kernel<<<blocks, 256, 0, s>>>(C, count, C32);
  HPC_LAUNCH_CHECK("to_f32_kernel");
  return HPC_OK;
}

}  // namespace hpc
