// FP64-accurate correlation Gram on the 5th-generation tensor cores (tcgen05 + TMA),
// by exact integer digits (an Ozaki-style splitting).
//
// Replaces the reference's FP64 gpuPMCC (src/correlation/corHelper.cu:79-116) where
// the correlation has to be FP64-accurate (HPC_PREC_MIXED): GB300's FP64 pipe gives
// about 1 TFLOP/s, so the p=2000, n=5000 Gram takes 20 ms in SIMT FP64; here it runs
// as BF16 tensor-core products that are exact.
//
//   y_v = z_v * 2^-e_v                  (e_v: the exponent of max |z_v|, so |y_v| <= 1)
//   y_v = sum_{t=1..7} d_t(v) 2^-7t     (d_1 = rint(128 y), then the remainders 7 bits
//                                        at a time: integers, |d_1| <= 128, |d_t| <= 64,
//                                        all exact in BF16; 49 bits of y)
//   sum_k y_a y_b = sum_{t+u<=8} 2^-7(t+u) sum_k d_t(a) d_u(b)   (dropped pairs < 2^-56)
//
// Each digit product is an integer of at most 2^14, so a sum over 1024 samples is an
// integer of at most 2^24: exact in the tensor core's FP32 accumulator. The kernel
// runs, per 128 x 128 tile of the upper triangle, the 28 digit pairs one after another
// (each a K = n_pad GEMM read by TMA straight from the digit planes), restarts the
// TMEM accumulator every 1024 samples, and the drain warps add the exact group sums
// into 64-bit fixed-point integers (LSB 2^-47 of sum y_a y_b) with integer
// instructions -- the FP64 pipe would be the bottleneck. The epilogue scales by
// 2^(e_a + e_b) / (n - 1) and writes the FP64 entry (both triangles) and its FP32
// rounding. Error: the 49-bit digits and the 2^-47 fixed point give |error| below
// 1e-13 on the correlation for n <= 32768 (the fixed point's range bounds n).
//
// Structure (one CTA of 10 warps per tile, 4-stage shared-memory ring, two 128-column
// TMEM accumulators): warp 0 lane 0 TMA producer, warp 1 lane 0 MMA issuer
// (tcgen05.mma.kind::f16, M = N = 128, K = 16), warps 2-9 drain (TMEM lane quadrant
// warp % 4, 64 columns each). Every mbarrier wait is bounded; on time-out the CTA
// records kErrTimeout, stops issuing, waits (bounded) for its copies and MMAs, frees
// its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "internal.cuh"
#include "tc_common.cuh"

namespace hpc {
namespace {

constexpr int EM = 128, EN = 128, EK = 64;   // tile 128 x 128, 64 samples (128 B) per stage
constexpr int kDigits = 7;
constexpr int kPairs = 28;                   // (t, u), t + u <= 8 (1-based)
constexpr int kGroupKb = 16;                 // k-blocks per exact group: 1024 samples
constexpr int kSampleAlign = EK * kGroupKb;  // n is padded to whole groups
constexpr int kStagesE = 4;
constexpr int kStageBytesE = (EM + EN) * EK * 2;  // 32 KB
constexpr int kTmemColsE = 256;              // two 128-column accumulators
constexpr int kAccWarpsE = 8;
constexpr int kThreadsE = 64 + 32 * kAccWarpsE;
constexpr int kFixL = 47;                    // fixed-point LSB 2^-47

// digit pair q -> 0-based digits (t, u) with t + u = s - 2, pairs ordered by s = 2..8
__device__ __forceinline__ void emu_pair(int q, int *t, int *u, int *s) {
  int ss = 2;
  while (q >= ss - 1) {
    q -= ss - 1;
    ++ss;
  }
  *t = q;
  *u = ss - 2 - q;
  *s = ss;
}

struct alignas(1024) EmuSmem {
  uint8_t stage[kStagesE][kStageBytesE];
  uint64_t full[kStagesE];
  uint64_t empty[kStagesE];
  uint64_t acc_full[2];
  uint64_t acc_empty[2];
  uint64_t drain;
  uint32_t tmem_base;
  int abort;
};

__device__ __forceinline__ bool aborted(EmuSmem &sm) { return *(volatile int *)&sm.abort != 0; }
__device__ __forceinline__ void fail(EmuSmem &sm, int *err) {
  atomicOr(err, kErrTimeout);
  atomicExch(&sm.abort, 1);
}

// One block per variable (rows beyond p are written as zero digits): the exponent of
// max |z| and the seven digits of z * 2^-e for every sample (zero beyond n).
__global__ void __launch_bounds__(256) emu_digits_kernel(const double *__restrict__ Z, int64_t p, int64_t n,
                                                         int64_t n_pad, __nv_bfloat16 *__restrict__ D,
                                                         int *__restrict__ E) {
  const int64_t v = blockIdx.x;
  __nv_bfloat16 *dv = D + v * (int64_t)kDigits * n_pad;
  __shared__ double red[8];
  __shared__ int s_e;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  double m = 0.0;
  if (v < p)
    for (int64_t k = threadIdx.x; k < n; k += blockDim.x) m = fmax(m, fabs(Z[v * n + k]));
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) red[wid] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double mm = 0.0;
    for (int w = 0; w < 8; ++w) mm = fmax(mm, red[w]);
    int e = 0;
    if (mm > 0.0) frexp(mm, &e);  // mm = f 2^e, f in [0.5, 1): 2^e > mm
    s_e = e;
    E[v] = e;
  }
  __syncthreads();
  const int e = s_e;
  for (int64_t k = threadIdx.x; k < n_pad; k += blockDim.x) {
    double r = (v < p && k < n) ? ldexp(Z[v * n + k], 7 - e) : 0.0;  // 128 y, exact
#pragma unroll
    for (int t = 0; t < kDigits; ++t) {
      const double d = rint(r);  // |d| <= 128, an integer: exact in BF16
      dv[t * n_pad + k] = __double2bfloat16(d);
      r = (r - d) * 128.0;       // exact: the remainder and a power of two
    }
  }
}

__global__ void __launch_bounds__(kThreadsE, 1)
    gram_emu_kernel(const __grid_constant__ CUtensorMap map, int64_t p, int64_t n_pad, double denom,
                    const int *__restrict__ E, double *__restrict__ C64, float *__restrict__ C32, int *err) {
  extern __shared__ uint8_t smem_raw[];
  EmuSmem &sm = *reinterpret_cast<EmuSmem *>((((uintptr_t)smem_raw) + 1023) & ~(uintptr_t)1023);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // tile (bi, bj), bi <= bj, row-major over the upper triangle of 128-blocks
  const int nb = (int)((p + EM - 1) / EM);
  long long t = blockIdx.x;
  int bi = 0;
  while (t >= nb - bi) {
    t -= nb - bi;
    ++bi;
  }
  const int bj = bi + (int)t;
  const int kbp = (int)(n_pad / EK);         // k-blocks per digit pair
  const int kblocks = kPairs * kbp;
  const int groups = kblocks / kGroupKb;
  const int gpp = kbp / kGroupKb;            // groups per pair
  const uint32_t idesc = idesc_bf16(EM, EN);

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStagesE; ++s) {
      mbar_init(&sm.full[s], 1);
      mbar_init(&sm.empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&sm.acc_full[b], 1);
      mbar_init(&sm.acc_empty[b], kAccWarpsE);
    }
    mbar_init(&sm.drain, 1);
    sm.abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sm.tmem_base)),
                 "r"(kTmemColsE));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = sm.tmem_base;

  int issued = 0;
  if (warp == 0 && lane == 0) {
    // TMA producer: pair q's k-block kb of digit t (rows of block bi) and u (block bj)
    for (int kg = 0; kg < kblocks; ++kg) {
      const int s = kg % kStagesE;
      if (kg >= kStagesE && !mbar_wait(&sm.empty[s], ((kg / kStagesE) + 1) & 1)) {
        fail(sm, err);
        break;
      }
      if (aborted(sm)) break;
      int dt, du, ss;
      emu_pair(kg / kbp, &dt, &du, &ss);
      const int kb = kg % kbp;
      mbar_arrive_expect_tx(&sm.full[s], kStageBytesE);
      tma_load_2d(sm.stage[s], &map, (int)(dt * n_pad) + kb * EK, bi * EM, &sm.full[s]);
      tma_load_2d(sm.stage[s] + EM * EK * 2, &map, (int)(du * n_pad) + kb * EK, bj * EN, &sm.full[s]);
      ++issued;
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer: group g (1024 samples of one digit pair) into TMEM buffer g % 2
    for (int g = 0; g < groups && !aborted(sm); ++g) {
      const int b = g & 1;
      if (g >= 2 && !mbar_wait(&sm.acc_empty[b], ((g >> 1) + 1) & 1)) {
        fail(sm, err);
        break;
      }
      const uint32_t dcol = tmem + (uint32_t)(b * EN);
      for (int kg = g * kGroupKb; kg < (g + 1) * kGroupKb; ++kg) {
        const int s = kg % kStagesE;
        if (!mbar_wait(&sm.full[s], (kg / kStagesE) & 1)) {
          fail(sm, err);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t a0 = smem_u32(sm.stage[s]), b0 = a0 + EM * EK * 2;
#pragma unroll
        for (int k = 0; k < EK / 16; ++k)
          mma_bf16(dcol, smem_desc_sw128(a0 + k * 32), smem_desc_sw128(b0 + k * 32), idesc,
                   (kg > g * kGroupKb || k > 0) ? 1u : 0u);
        mma_commit(&sm.empty[s]);
      }
      mma_commit(&sm.acc_full[b]);
    }
    mma_commit(&sm.drain);
    if (!mbar_wait(&sm.drain, 0)) fail(sm, err);
  } else if (warp >= 2) {
    // drain: rows 32 (warp % 4) .. + 31 (TMEM lanes), columns 64 ((warp - 2) / 4) .. + 63
    const int quad = warp & 3;
    const int half = (warp - 2) >> 2;
    constexpr int kCols = EN / 2;
    long long acc[kCols];
#pragma unroll
    for (int q = 0; q < kCols; ++q) acc[q] = 0;
    bool ok = true;
    for (int g = 0; g < groups; ++g) {
      const int b = g & 1;
      if (!mbar_wait(&sm.acc_full[b], (g >> 1) & 1)) {
        fail(sm, err);
        ok = false;
        break;
      }
      __syncwarp();
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      int dt, du, ss;
      emu_pair(g / gpp, &dt, &du, &ss);
      const int sh = kFixL - 7 * ss;  // the group sum's weight 2^-7s in units of 2^-47
#pragma unroll
      for (int c0 = 0; c0 < kCols; c0 += 32) {
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(b * EN + half * kCols + c0), v);
#pragma unroll
        for (int q = 0; q < 32; ++q) {
          const long long gi = (long long)__float2int_rn(v[q]);  // an integer below 2^24: exact
          acc[c0 + q] += sh >= 0 ? gi * (1ll << sh) : (gi >> (-sh));
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.acc_empty[b]);
    }
    if (ok && !aborted(sm)) {
      const int64_t row = (int64_t)bi * EM + quad * 32 + lane;
      const int64_t col0 = (int64_t)bj * EN + half * kCols;
      const int er = row < p ? E[row] : 0;
#pragma unroll 4
      for (int cc = 0; cc < kCols; ++cc) {
        const int64_t col = col0 + cc;
        if (row < p && col < p && col >= row) {
          const double v = ldexp((double)acc[cc], er + E[col] - kFixL) / denom;
          C64[col * p + row] = v;  // the warp's lanes: consecutive rows, one column
          C64[row * p + col] = v;
          if (C32) {
            C32[col * p + row] = (float)v;
            C32[row * p + col] = (float)v;
          }
        }
      }
    }
  }
  if (warp == 0 && lane == 0 && sm.abort) {
    for (int s = 0; s < kStagesE; ++s) {
      const int fills = issued / kStagesE + (s < issued % kStagesE ? 1 : 0);
      if (fills > 0) mbar_wait(&sm.full[s], (fills - 1) & 1);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemColsE));
  }
}

int64_t emu_n_pad(int64_t n) { return (n + kSampleAlign - 1) / kSampleAlign * kSampleAlign; }

}  // namespace

// The exact-digit Gram serves one instance of at least 256 variables (below that the
// SIMT FP64 Gram is as fast) and at most 32768 samples (the fixed point's range).
bool emu_eligible(int64_t p, int64_t n) { return p >= 256 && n <= 32768; }
int64_t emu_p_pad(int64_t p) { return (p + EM - 1) / EM * EM; }
int64_t emu_digit_elems(int64_t p, int64_t n) { return emu_p_pad(p) * kDigits * emu_n_pad(n); }

hpc_status launch_gram_emu(const double *Z, int64_t p, int64_t n, double denom, __nv_bfloat16 *D, int *E,
                           CUtensorMap * /*unused*/, double *C64, float *C32, int *err, cudaStream_t s) {
  const int64_t n_pad = emu_n_pad(n), p_pad = emu_p_pad(p);
  emu_digits_kernel<<<(unsigned)p_pad, 256, 0, s>>>(Z, p, n, n_pad, D, E);
  HPC_LAUNCH_CHECK("emu_digits_kernel");
  CUtensorMap map;
  hpc_status st = tc_make_map(&map, D, p_pad, kDigits * n_pad, EM);
  if (st != HPC_OK) return st;
  const int smem = (int)sizeof(EmuSmem) + 1024;
  HPC_CUDA(cudaFuncSetAttribute(gram_emu_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  const long long nb = p_pad / EM, tiles = nb * (nb + 1) / 2;
  gram_emu_kernel<<<(unsigned)tiles, kThreadsE, smem, s>>>(map, p, n_pad, denom, E, C64, C32, err);
  HPC_LAUNCH_CHECK("gram_emu_kernel");
  return HPC_OK;
}

}  // namespace hpc
