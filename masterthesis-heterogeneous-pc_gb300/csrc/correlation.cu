// Correlation: column standardisation and the FP64 Gram, grouped over the instances
// of a context.
//
// Replaces gpuMeans / gpuSD / gpuPMCC (src/correlation/corHelper.cu:8-116), which
// launch one 64-thread block per (i, j) pair and re-read both columns for every pair.
// Here one block per variable standardises its column once (NaN-skipping mean, SD with
// the n-1 denominator, z = (x - mean) / sd, missing samples as 0 so that a product with
// a missing sample contributes nothing -- the reference's pairwise NaN skip,
// corHelper.cu:101) into the FP64 copy Z and, for the tensor-core Gram, into the
// split-BF16 operands; the FP64 correlation is the register- and shared-memory-tiled
// Gram C = Z^T Z / (n - 1) over upper-triangle 64 x 64 tiles, mirrored on write.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>

#include "internal.cuh"

namespace hpc {
namespace {

constexpr int kStdThreads = 256;

// grid: one block per variable of every instance (flattened over row_prefix)
template <typename TIn, bool SPLIT>
__global__ void __launch_bounds__(kStdThreads) standardise_kernel(const TIn *__restrict__ X, StdArgs a,
                                                                  double *__restrict__ Z,
                                                                  __nv_bfloat16 *__restrict__ P,
                                                                  __nv_bfloat16 *__restrict__ Q) {
  const long long t = blockIdx.x;
  const int b = find_inst(a.row_prefix, a.count, t);
  const long long v = t - a.row_prefix[b];
  const long long n = a.n[b];
  const TIn *x = X + a.x_off[b] + v * n;
  double *z = Z + a.z_off[b] + v * n;
  __shared__ double red[kStdThreads / 32];
  __shared__ long long redc[kStdThreads / 32];
  __shared__ double mean_s, sd_s;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;

  double s = 0.0;
  long long c = 0;
  for (long long k = threadIdx.x; k < n; k += kStdThreads) {
    const double xv = (double)x[k];
    if (!isnan(xv)) {
      s += xv;
      ++c;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  if (lane == 0) {
    red[wid] = s;
    redc[wid] = c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double tt = 0.0;
    long long tc = 0;
    for (int w = 0; w < kStdThreads / 32; ++w) {
      tt += red[w];
      tc += redc[w];
    }
    mean_s = tt / (double)tc;
  }
  __syncthreads();
  const double mean = mean_s;
  double ss = 0.0;
  for (long long k = threadIdx.x; k < n; k += kStdThreads) {
    const double xv = (double)x[k];
    if (!isnan(xv)) {
      const double d = xv - mean;
      ss += d * d;
    }
  }
  for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
  __syncthreads();
  if (lane == 0) red[wid] = ss;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tt = 0.0;
    for (int w = 0; w < kStdThreads / 32; ++w) tt += red[w];
    if (a.ref_compat)  // corHelper.cu:75: sqrtf of (sum / (dim - 1.f))
      sd_s = (double)sqrtf((float)(tt / (double)((float)n - 1.f)));
    else
      sd_s = sqrt(tt / (double)(n - 1));
  }
  __syncthreads();
  // z = (x - mean) * (1 / sd): one FP64 multiply per sample instead of a division (FP64
  // division is a long instruction sequence on this GPU, and this loop touches every
  // sample of every variable); the values differ from (x - mean) / sd by at most an ulp
  const double inv_sd = 1.0 / sd_s;
  if (!SPLIT) {
    for (long long k = threadIdx.x; k < n; k += kStdThreads) {
      const double xv = (double)x[k];
      z[k] = isnan(xv) ? 0.0 : (xv - mean) * inv_sd;
    }
    return;
  }
  // split-BF16 operand of the tensor-core Gram: two planes T = [hi | lo] of z / sqrt(n - 1)
  // (the Gram's producer pairs the planes: hi.hi + hi.lo + lo.hi + lo.lo is the
  // correlation). The split runs in FP32 (hi = bf16(zs), lo = bf16(zs - hi), the
  // subtraction exact in FP32): its error is the rounding of lo, as with an FP64 split,
  // plus 2^-24 relative from zs itself. Two consecutive samples per thread, so that the
  // planes are written as 4-byte pairs.
  const double denom = a.ref_compat ? (double)((float)n - 1.f) : (double)(n - 1);
  const double scale = 1.0 / sqrt(denom);
  const long long n_pad = a.n_pad[b], K = a.kdim[b];
  __nv_bfloat16 *pr = P + a.tc_off[b] + v * K;
  for (long long k = 2 * (long long)threadIdx.x; k < n_pad; k += 2 * kStdThreads) {
    double z0 = 0.0, z1 = 0.0;
    if (k < n) {
      const double xv = (double)x[k];
      z0 = isnan(xv) ? 0.0 : (xv - mean) * inv_sd;
      z[k] = z0;
    }
    if (k + 1 < n) {
      const double xv = (double)x[k + 1];
      z1 = isnan(xv) ? 0.0 : (xv - mean) * inv_sd;
      z[k + 1] = z1;
    }
    const float s0 = (float)(z0 * scale), s1 = (float)(z1 * scale);
    const __nv_bfloat162 hi = __floats2bfloat162_rn(s0, s1);
    const float2 hf = __bfloat1622float2(hi);
    const __nv_bfloat162 lo = __floats2bfloat162_rn(s0 - hf.x, s1 - hf.y);
    *reinterpret_cast<__nv_bfloat162 *>(pr + k) = hi;
    *reinterpret_cast<__nv_bfloat162 *>(pr + n_pad + k) = lo;
  }
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
                              __nv_bfloat16 *P, __nv_bfloat16 *Q, cudaStream_t s) {
  const bool split = P != nullptr;
  const unsigned grid = (unsigned)total_rows;
  if (f32) {
    if (split)
      standardise_kernel<float, true><<<grid, kStdThreads, 0, s>>>((const float *)X, a, Z, P, Q);
    else
      standardise_kernel<float, false><<<grid, kStdThreads, 0, s>>>((const float *)X, a, Z, P, Q);
  } else {
    if (split)
      standardise_kernel<double, true><<<grid, kStdThreads, 0, s>>>((const double *)X, a, Z, P, Q);
    else
      standardise_kernel<double, false><<<grid, kStdThreads, 0, s>>>((const double *)X, a, Z, P, Q);
  }
  HPC_LAUNCH_CHECK("standardise_kernel");
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
