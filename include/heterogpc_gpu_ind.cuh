/*
 * heterogpc_gpu_ind.cuh -- the reference's device-side independence statistics,
 * GPU::calcPValue and GPU::pValL1 (src/executor/independence/gpuInd.cuh:1-6,
 * gpuInd.cu:4-19 of milanpro/Masterthesis-Heterogeneous-PC), header-only and callable
 * from host and device code (the reference compiles them as separate __device__
 * functions, which a shared library cannot export).
 *
 * Semantics as the reference's device versions: |r| clamped to 0.9999999 (NaN -> 0),
 * z = sqrt(n - 3) * atanh(|r|) written as 0.5 * log1p(2r / (1 - r)), p = 2 (1 - Phi(z)).
 * On the device Phi is CUDA's normcdf, as in the reference; on the host it is
 * 1 - erfc(z / sqrt 2) / 2. Note that 1 - Phi(z) loses relative precision for large z
 * (p below about 1e-10); the CPU statistics of heterogpc.h (hpc_calc_pvalue,
 * the reference's CPU::calcPValue) use the complement directly.
 */
#ifndef HETEROGPC_GPU_IND_CUH
#define HETEROGPC_GPU_IND_CUH

#include <math.h>

#ifdef __CUDACC__
#define HPC_HD __host__ __device__ __forceinline__
#else
#define HPC_HD inline
#endif

namespace GPU {

HPC_HD double calcPValue(double r, int sampleSize) {
  r = isnan(r) ? 0.0 : fmin(0.9999999, fabs(r));
  const double absz = sqrt(sampleSize - 3.0) * 0.5 * log1p(2.0 * r / (1.0 - r));
#ifdef __CUDA_ARCH__
  return 2.0 * (1.0 - normcdf(absz));
#else
  return 2.0 * (1.0 - (1.0 - 0.5 * erfc(absz / 1.4142135623730950488)));
#endif
}

// with edge i, j given k: x1 = r_ij, x2 = r_ik, x3 = r_jk
HPC_HD double pValL1(double x1, double x2, double x3, int sampleSize) {
  const double r = (x1 - x2 * x3) / sqrt((1.0 - x3 * x3) * (1.0 - x2 * x2));
  return calcPValue(r, sampleSize);
}

}  // namespace GPU

#undef HPC_HD
#endif /* HETEROGPC_GPU_IND_CUH */
