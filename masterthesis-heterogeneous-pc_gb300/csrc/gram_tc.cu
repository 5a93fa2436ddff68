// Split-BF16 correlation Gram on the 5th-generation tensor cores (tcgen05 + TMA).
//
// Replaces the reference's gpuPMCC (src/correlation/corHelper.cu:79-116), which
// spends one 64-thread block of FP64 SIMT work per (i, j) pair, with the one dense
// contraction of the path done on the tensor cores:
//
//   z  = (x - mean) / sd / sqrt(n - 1)          (FP64, per variable)
//   hi = bf16(z),  lo = bf16(z - hi)
//   T  = [hi | lo]                              (two planes of n_pad, K-major rows)
//   C  = hi.hi + hi.lo + lo.hi + lo.lo          (FP32 accumulation in TMEM)
//
// so one BF16 GEMM with K = 4 n_pad gives the products of the split: the producer reads
// plane q >> 1 for A and plane q & 1 for B in the q-th quarter of K. With lo.lo the
// product of the two 16-bit representations is complete and what is left is the
// rounding of lo (2^-17 relative per value), which averages out over n samples;
// without it a systematic error of about 2^-18 |r| remains. Tiles are 128 rows x 256
// columns (one N = 256 MMA per K-step: 48 KB of operands per 2 x 128 x 256 x 64 flops,
// a third more work per byte of L2 traffic than square 128-tiles), over the column
// blocks that reach the upper triangle; each entry with col >= row is written twice
// (direct and mirrored), so C is exactly symmetric.
//
// The tensor core rounds its FP32 accumulator once per MMA; along K = 3n that is
// thousands of roundings with a systematic bias (measured about 3e-5 on sums of
// magnitude 1). So the accumulation restarts every kGroup k-blocks in one of two
// TMEM buffers while the epilogue warps drain the other into FP32 registers
// (round-to-nearest adds): about 3n/256 register additions per output instead.
//
// Kernel structure (one CTA of 10 warps per tile, 4-stage shared-memory ring):
//   warp 0 lane 0   TMA producer: cp.async.bulk.tensor of the A (128 rows of P) and B
//                   (256 rows of Q) x 64 K tiles, 128-byte swizzle, into stage s,
//                   completion counted on full[s] (expect_tx)
//   warp 1 lane 0   MMA issuer: 4 x tcgen05.mma.kind::f16 (M=128, N=256, K=16) per
//                   stage into TMEM buffer g % 2 (256 columns each), tcgen05.commit
//                   to empty[s] (frees the stage) and, after each group of kGroup
//                   stages, to acc_full[g % 2]
//   warps 2-9       accumulate: tcgen05.ld 32x32b of their TMEM lane quadrant
//                   (warp % 4) and column half ((warp - 2) / 4), add into 128
//                   registers per thread, arrive on acc_empty[g % 2]; finally write
//                   the tile
// Every mbarrier wait is bounded by a %globaltimer deadline; on time-out the CTA
// records kErrTimeout, stops issuing, waits (bounded) for what it already issued,
// frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "internal.cuh"
#include "tc_common.cuh"

namespace hpc {
namespace {

constexpr int TM = 128, TN = 256, TK = 64;  // tile: 128 x 256 outputs, 64 bf16 (128 B) of K per stage
constexpr int kStages = 4;
constexpr int kSlices = 4;       // K = kSlices * n_pad: hi.hi, hi.lo, lo.hi, lo.lo
constexpr int kPlanes = 2;       // the operand holds hi and lo
constexpr int kStageBytesA = TM * TK * 2;   // 16 KB
constexpr int kStageBytesB = TN * TK * 2;   // 32 KB
constexpr int kStageBytes = kStageBytesA + kStageBytesB;
constexpr int kTmemCols = 512;   // two 256-column accumulators
constexpr int kGroup = 4;        // k-blocks (16 MMAs) per accumulation group
constexpr int kAccWarps = 8;     // two per TMEM lane quadrant, 128 columns each
constexpr int kBand = 16;        // row blocks per band of the tile order (even)
constexpr int kThreadsTc = 64 + 32 * kAccWarps;  // producer warp, MMA warp, accumulator warps

// operand rows padded to the column-block size, so that every TMA box lies inside
__host__ __device__ __forceinline__ int64_t tc_p_pad_dev(int64_t p) { return (p + TN - 1) / TN * TN; }

// the tiles of one instance: 128-row blocks bi, and for each the 256-column blocks
// bj >= bi / 2 (those holding entries with col >= row)
__host__ __device__ __forceinline__ int tc_col_blocks(int64_t p) { return (int)((tc_p_pad_dev(p) + TN - 1) / TN); }

struct alignas(1024) TcSmem {
  uint8_t stage[kStages][kStageBytes];
  uint64_t full[kStages];
  uint64_t empty[kStages];
  uint64_t acc_full[2];
  uint64_t acc_empty[2];
  uint64_t drain;
  uint32_t tmem_base;
  int abort;
};

__device__ __forceinline__ bool aborted(TcSmem &sm) { return *(volatile int *)&sm.abort != 0; }
__device__ __forceinline__ void fail(TcSmem &sm, int *err) {
  atomicOr(err, kErrTimeout);
  atomicExch(&sm.abort, 1);
}

__global__ void __launch_bounds__(kThreadsTc, 1)
    gram_tc_kernel(float *__restrict__ Call, TcArgs ta) {
  extern __shared__ uint8_t smem_raw[];
  TcSmem &sm = *reinterpret_cast<TcSmem *>((((uintptr_t)smem_raw) + 1023) & ~(uintptr_t)1023);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  // instance, then tile (bi, bj), bi <= bj, over the upper triangle of its tiles
  const long long tt = blockIdx.x;
  const int inst = find_inst(ta.tile_prefix, ta.count, tt);
  long long t = tt - ta.tile_prefix[inst];
  const int64_t p = ta.p[inst];
  const int nbc = tc_col_blocks(p);
  const int kbq = (int)((ta.n[inst] + TK - 1) / TK);  // k-blocks per product
  const int64_t n_pad = (int64_t)kbq * TK;
  const int kblocks = kSlices * kbq;
  const CUtensorMap *mapP = ta.maps + 2 * inst, *mapQ = ta.maps + 2 * inst + 1;
  float *__restrict__ C = Call + ta.c_off[inst];
  int *err = ta.err;
  // tiles in bands of kBand row blocks, each band column block by column block, so
  // that the CTAs running at one time share a few A and B blocks that stay in L2
  const int nb = (int)(tc_p_pad_dev(p) / TM);
  int b0 = 0;
  for (;;) {
    const int b1 = min(nb, b0 + kBand);
    long long cnt = 0;
    for (int r = b0; r < b1; ++r) cnt += nbc - r / 2;
    if (t < cnt || b1 >= nb) break;
    t -= cnt;
    b0 = b1;
  }
  int bi = b0, bj = b0 / 2;
  for (;; ++bj) {
    // rows of the band whose column blocks start at or before bj (bi / 2 <= bj)
    const int rows = min(min(nb, b0 + kBand), 2 * bj + 2) - b0;
    if (t < rows) {
      bi = b0 + (int)t;
      break;
    }
    t -= rows;
  }

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&sm.full[s], 1);
      mbar_init(&sm.empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&sm.acc_full[b], 1);
      mbar_init(&sm.acc_empty[b], kAccWarps);  // one arrival per accumulator warp
    }
    mbar_init(&sm.drain, 1);
    sm.abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sm.tmem_base)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = sm.tmem_base;

  int issued = 0;  // producer: stage fills issued
  if (warp == 0 && lane == 0) {
    // TMA producer
    for (int kb = 0; kb < kblocks; ++kb) {
      const int s = kb % kStages;
      if (kb >= kStages && !mbar_wait(&sm.empty[s], ((kb / kStages) + 1) & 1)) {
        fail(sm, err);
        break;
      }
      if (aborted(sm)) break;
      mbar_arrive_expect_tx(&sm.full[s], kStageBytes);
      const int q = kb / kbq, kq = (kb - q * kbq) * TK;  // product q: planes (q >> 1, q & 1)
      tma_load_2d(sm.stage[s], mapP, (q >> 1) * (int)n_pad + kq, bi * TM, &sm.full[s]);
      tma_load_2d(sm.stage[s] + kStageBytesA, mapQ, (q & 1) * (int)n_pad + kq, bj * TN, &sm.full[s]);
      ++issued;
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer: group g accumulates k-blocks [g*kGroup, (g+1)*kGroup) into buffer g % 2
    const int groups = (kblocks + kGroup - 1) / kGroup;
    for (int g = 0; g < groups && !aborted(sm); ++g) {
      const int b = g & 1;
      if (g >= 2 && !mbar_wait(&sm.acc_empty[b], ((g >> 1) + 1) & 1)) {
        fail(sm, err);
        break;
      }
      const uint32_t dcol = tmem + (uint32_t)(b * TN);
      const int kb_end = min(kblocks, (g + 1) * kGroup);
      for (int kb = g * kGroup; kb < kb_end; ++kb) {
        const int s = kb % kStages;
        if (!mbar_wait(&sm.full[s], (kb / kStages) & 1)) {
          fail(sm, err);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t a0 = smem_u32(sm.stage[s]), b0 = a0 + kStageBytesA;
#pragma unroll
        for (int k = 0; k < TK / 16; ++k) {
          // 16 bf16 = 32 bytes further along K inside the 128-byte swizzled row
          mma_bf16(dcol, smem_desc_sw128(a0 + k * 32), smem_desc_sw128(b0 + k * 32), idesc_bf16(TM, TN),
                   (kb > g * kGroup || k > 0) ? 1u : 0u);
        }
        mma_commit(&sm.empty[s]);
      }
      mma_commit(&sm.acc_full[b]);  // arrives when this group's MMAs have completed
    }
    // every MMA issued above has completed before TMEM is freed
    mma_commit(&sm.drain);
    if (!mbar_wait(&sm.drain, 0)) fail(sm, err);
  } else if (warp >= 2) {
    // accumulator warps: TMEM lane quadrant warp % 4 = rows 32*(warp%4) .. +31, and
    // column half (warp - 2) / 4
    const int quad = warp & 3;
    const int half = (warp - 2) >> 2;
    constexpr int kCols = TN / 2;
    float acc[kCols];
#pragma unroll
    for (int q = 0; q < kCols; ++q) acc[q] = 0.f;
    const int groups = (kblocks + kGroup - 1) / kGroup;
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
#pragma unroll
      for (int c0 = 0; c0 < kCols; c0 += 32) {
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(b * TN + half * kCols + c0), v);
#pragma unroll
        for (int q = 0; q < 32; ++q) acc[c0 + q] += v[q];
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.acc_empty[b]);
    }
    if (ok && !aborted(sm)) {
      const int64_t row = (int64_t)bi * TM + quad * 32 + lane;
      const int64_t col0 = (int64_t)bj * TN + half * kCols;
      // mirrored copy: for a fixed column the warp's lanes hold 32 consecutive rows,
      // i.e. a contiguous run of C[col][...]: coalesced as it is
#pragma unroll
      for (int cc = 0; cc < kCols; ++cc) {
        const int64_t col = col0 + cc;
        if (row < p && col < p && col >= row) C[col * p + row] = acc[cc];
      }
      // direct copy through the idle stage buffer (every MMA has completed): each
      // warp transposes 32 x 32 blocks (33-float rows, no bank conflicts) so that its
      // lanes write 32 consecutive columns of one row per store
      float *tb = reinterpret_cast<float *>(sm.stage[0]) + (warp - 2) * 32 * 33;
#pragma unroll
      for (int c0 = 0; c0 < kCols; c0 += 32) {
#pragma unroll
        for (int q = 0; q < 32; ++q) tb[lane * 33 + q] = acc[c0 + q];
        __syncwarp();
        const int64_t col = col0 + c0 + lane;
#pragma unroll 4
        for (int k = 0; k < 32; ++k) {
          const int64_t rw = (int64_t)bi * TM + quad * 32 + k;
          if (rw < p && col < p && col >= rw) C[rw * p + col] = tb[k * 33 + lane];
        }
        __syncwarp();
      }
    }
  }
  // before freeing TMEM and exiting, the producer's copies must have landed: wait
  // (bounded) for the last phase of every stage it filled
  if (warp == 0 && lane == 0 && sm.abort) {
    for (int s = 0; s < kStages; ++s) {
      const int fills = issued / kStages + (s < issued % kStages ? 1 : 0);
      if (fills > 0) mbar_wait(&sm.full[s], (fills - 1) & 1);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
  }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
    else
      cudaGetLastError();
  }
  return fn;
}

hpc_status make_map(CUtensorMap *m, const __nv_bfloat16 *base, int64_t rows, int64_t K, int box_rows) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) {
    set_error("cuTensorMapEncodeTiled is not available from the driver");
    return HPC_ERR_CUDA;
  }
  cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(K * 2)};
  cuuint32_t box[2] = {(cuuint32_t)TK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void *)base, dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
    return HPC_ERR_CUDA;
  }
  return HPC_OK;
}

}  // namespace

int64_t tc_n_pad(int64_t n) { return (n + TK - 1) / TK * TK; }
int64_t tc_p_pad(int64_t p) { return tc_p_pad_dev(p); }
int64_t tc_k(int64_t n) { return kPlanes * tc_n_pad(n); }

long long gram_tc_tiles(int64_t p) {
  const long long nb = tc_p_pad(p) / TM, nbc = tc_col_blocks(p);
  long long t = 0;
  for (long long bi = 0; bi < nb; ++bi) t += nbc - bi / 2;
  return t;
}

// Tensor maps of one instance's operand planes (tc_p_pad(p) rows of tc_k(n) bf16), for
// the A (128-row) and B (256-row) tiles; P and Q may be the same buffer.
// a 2-D BF16 tensor map (rows x K, K contiguous, 64-column x box_rows boxes, 128-byte
// swizzle) for the other tensor-core kernels
hpc_status tc_make_map(CUtensorMap *m, const __nv_bfloat16 *base, int64_t rows, int64_t K, int box_rows) {
  return make_map(m, base, rows, K, box_rows);
}

hpc_status tc_make_maps(CUtensorMap *mp, CUtensorMap *mq, const __nv_bfloat16 *P, const __nv_bfloat16 *Q,
                        int64_t p, int64_t n) {
  hpc_status st;
  if ((st = make_map(mp, P, tc_p_pad(p), tc_k(n), TM)) != HPC_OK) return st;
  return make_map(mq, Q, tc_p_pad(p), tc_k(n), TN);
}

// C (p x p FP32 per instance, row-major) = P Q^T over upper-triangle tiles, mirrored;
// blocks flattened over all instances' tiles.
hpc_status launch_gram_tc(float *C, const TcArgs &a, long long total_tiles, cudaStream_t s) {
  const int smem = (int)sizeof(TcSmem) + 1024;
  HPC_CUDA(cudaFuncSetAttribute(gram_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  gram_tc_kernel<<<(unsigned)total_tiles, kThreadsTc, smem, s>>>(C, a);
  HPC_LAUNCH_CHECK("gram_tc_kernel");
  return HPC_OK;
}

}  // namespace hpc
