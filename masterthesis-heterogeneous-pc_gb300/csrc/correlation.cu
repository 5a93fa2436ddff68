// Correlation: column standardisation and the FP64 Gram.
//
// Replaces gpuMeans / gpuSD / gpuPMCC (src/correlation/corHelper.cu:8-116), which
// launch one 64-thread block per (i, j) pair and re-read both columns for every
// pair. Here one block per variable standardises its column once (NaN-skipping
// mean, SD with the n-1 denominator, z = (x - mean) / sd, missing samples as 0 so
// that a product with a missing sample contributes nothing -- the reference's
// pairwise NaN skip, corHelper.cu:101), and the correlation is the register- and
// shared-memory-tiled Gram C = Z^T Z / (n - 1) over upper-triangle tiles only,
// mirrored on write.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>

#include "internal.cuh"

namespace hpc {
namespace {

constexpr int kStdThreads = 256;

template <typename TIn>
__global__ void __launch_bounds__(kStdThreads) standardise_kernel(const TIn *__restrict__ X, int64_t n,
                                                                  int64_t p, int ref_compat,
                                                                  double *__restrict__ Z) {
  const int64_t v = blockIdx.x;
  if (v >= p) return;
  const TIn *x = X + v * n;
  double *z = Z + v * n;
  __shared__ double red[kStdThreads / 32];
  __shared__ long long redc[kStdThreads / 32];
  __shared__ double mean_s, sd_s;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;

  double s = 0.0;
  long long c = 0;
  for (int64_t k = threadIdx.x; k < n; k += kStdThreads) {
    double a = (double)x[k];
    if (!isnan(a)) { s += a; ++c; }
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  if (lane == 0) { red[wid] = s; redc[wid] = c; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    long long tc = 0;
    for (int w = 0; w < kStdThreads / 32; ++w) { t += red[w]; tc += redc[w]; }
    mean_s = t / (double)tc;
  }
  __syncthreads();
  const double mean = mean_s;
  double ss = 0.0;
  for (int64_t k = threadIdx.x; k < n; k += kStdThreads) {
    double a = (double)x[k];
    if (!isnan(a)) { double d = a - mean; ss += d * d; }
  }
  for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
  __syncthreads();
  if (lane == 0) red[wid] = ss;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kStdThreads / 32; ++w) t += red[w];
    if (ref_compat)  // corHelper.cu:75: sqrtf of (sum / (dim - 1.f))
      sd_s = (double)sqrtf((float)(t / (double)((float)n - 1.f)));
    else
      sd_s = sqrt(t / (double)(n - 1));
  }
  __syncthreads();
  const double sd = sd_s;
  for (int64_t k = threadIdx.x; k < n; k += kStdThreads) {
    double a = (double)x[k];
    z[k] = isnan(a) ? 0.0 : (a - mean) / sd;
  }
}

// FP64 Gram, 64 x 64 output tile per block, K staged 16 at a time through shared
// memory, 4 x 4 outputs per thread.
constexpr int BM = 64, BK = 16, GT = 256;

__global__ void __launch_bounds__(GT) gram_f64_kernel(const double *__restrict__ Z, int64_t n, int64_t p,
                                                      int nb, double denom, double *__restrict__ C) {
  // linear block id -> (bi, bj) with bi <= bj over the upper triangle of tiles
  int64_t t = blockIdx.x;
  int bi = 0;
  {
    // row bi holds nb - bi tiles
    int64_t rem = t;
    while (rem >= nb - bi) { rem -= nb - bi; ++bi; }
    t = rem;
  }
  const int bj = bi + (int)t;
  const int64_t a0 = (int64_t)bi * BM, b0 = (int64_t)bj * BM;
  __shared__ double As[BK][BM + 1];
  __shared__ double Bs[BK][BM + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

  for (int64_t k0 = 0; k0 < n; k0 += BK) {
    // 64 columns x 16 k = 1024 values per operand, 4 per thread
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      int idx = threadIdx.x + r * GT;  // 0..1023
      int col = idx >> 4, kk = idx & 15;
      int64_t k = k0 + kk;
      int64_t va = a0 + col, vb = b0 + col;
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
    int64_t a = a0 + ty + 16 * i;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int64_t b = b0 + tx + 16 * j;
      if (a < p && b < p && a <= b) {
        double v = acc[i][j] / denom;
        C[a * p + b] = v;
        C[b * p + a] = v;
      }
    }
  }
}

__global__ void to_f32_kernel(const double *__restrict__ C, int64_t count, float *__restrict__ C32) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    C32[i] = (float)C[i];
}

}  // namespace

hpc_status launch_standardise_f64(const double *X, int64_t n, int64_t p, int ref_compat, double *Z,
                                  cudaStream_t s) {
  standardise_kernel<double><<<(unsigned)p, kStdThreads, 0, s>>>(X, n, p, ref_compat, Z);
  HPC_LAUNCH_CHECK("standardise_kernel<double>");
  return HPC_OK;
}

hpc_status launch_standardise_f32(const float *X, int64_t n, int64_t p, int ref_compat, double *Z,
                                  cudaStream_t s) {
  standardise_kernel<float><<<(unsigned)p, kStdThreads, 0, s>>>(X, n, p, ref_compat, Z);
  HPC_LAUNCH_CHECK("standardise_kernel<float>");
  return HPC_OK;
}

hpc_status launch_gram_f64(const double *Z, int64_t n, int64_t p, double denom, double *C, cudaStream_t s) {
  const int nb = (int)((p + BM - 1) / BM);
  const int64_t tiles = (int64_t)nb * (nb + 1) / 2;
  gram_f64_kernel<<<(unsigned)tiles, GT, 0, s>>>(Z, n, p, nb, denom, C);
  HPC_LAUNCH_CHECK("gram_f64_kernel");
  return HPC_OK;
}

hpc_status launch_to_f32(const double *C, int64_t count, float *C32, cudaStream_t s) {
  int blocks = (int)std::min<int64_t>((count + 255) / 256, 152 * 16);
  to_f32_kernel<<<blocks, 256, 0, s>>>(C, count, C32);
  HPC_LAUNCH_CHECK("to_f32_kernel");
  return HPC_OK;
}

}  // namespace hpc
