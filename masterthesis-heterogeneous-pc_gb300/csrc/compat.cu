// The reference's correlation and compaction entry points under their own names
// (include/heterogpc_compat.h): gpuPMCC (src/correlation/corOwn.cu:10-48) on top of the
// C ABI, and callCompact (src/independence/compact.cu:91-99) as a kernel that works on
// the caller's MMState buffers in place.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <limits>

#include "../../include/heterogpc_compat.h"
#include "internal.cuh"

namespace hpc {
namespace {

// One warp per row of the caller's p x p int adjacency: ballots over 32 columns at a
// time give each neighbour its slot in ascending order (the scan of compactCUTiled,
// compact.cu:4-89, without its shared-memory tiles), the rest of the row up to slot
// p - 2 is zeroed and the count goes to slot p - 1.
__global__ void compact_rows_kernel(const int *__restrict__ adj, int *__restrict__ out, int64_t p, int64_t row0,
                                    int64_t row1, int *max_adj) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t row = row0 + ((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5); row < row1; row += nw) {
    const int *a = adj + row * p;
    int *o = out + row * p;
    int cnt = 0;
    for (int64_t c0 = 0; c0 < p; c0 += 32) {
      const int64_t c = c0 + lane;
      const bool nb = c < p && a[c] != 0;
      const unsigned m = __ballot_sync(0xffffffffu, nb);
      if (nb) o[cnt + __popc(m & ((1u << lane) - 1u))] = (int)c;
      cnt += __popc(m);
    }
    __syncwarp();
    for (int64_t k = cnt + lane; k < p - 1; k += 32) o[k] = 0;
    if (lane == 0) {
      o[p - 1] = cnt;
      atomicMax_system(max_adj, cnt);
    }
  }
}

void fill_nan(double *v, size_t n) {
  for (size_t i = 0; i < n; ++i) v[i] = std::numeric_limits<double>::quiet_NaN();
}

}  // namespace
}  // namespace hpc

using namespace hpc;

void gpuPMCC(const double *h_mat, uint64_t n, int dim, double *cors, int deviceId, bool verbose) {
  if (!h_mat || !cors || n < 2 || dim < 4) {
    set_error("gpuPMCC: null pointer or too small a problem (n = %llu variables, dim = %d observations)",
              (unsigned long long)n, dim);
    if (cors && n) fill_nan(cors, (size_t)(n * n));
    return;
  }
  if (verbose) printf("Cor started with N=%llu, dim=%i\n", (unsigned long long)n, dim);
  hpc_opts o;
  hpc_opts_default(&o);
  o.device = deviceId;
  o.precision = HPC_PREC_FP64;
  o.max_level = 0;
  o.ref_compat_sd = 1;  // the reference's SD is rounded through float (corHelper.cu:75)
  hpc_ctx *c = nullptr;
  hpc_status s = hpc_ctx_create(&c, (int64_t)n, dim, &o);
  if (s == HPC_OK) s = hpc_correlation_f64(c, h_mat);
  if (s == HPC_OK) s = hpc_get_correlation(c, cors);
  if (c) hpc_ctx_destroy(c);
  if (s != HPC_OK) {
    fill_nan(cors, (size_t)(n * n));
    fprintf(stderr, "gpuPMCC: %s\n", hpc_last_error_string());
    return;
  }
  if (verbose) printf("PMCC successful \n");
}

void callCompact(MMState *state, int deviceId, int idx, int numberOfGPUs, int d_rowCount) {
  (void)numberOfGPUs;
  if (!state || !state->adj || !state->adj_compact || !state->max_adj || state->p < 2 || idx < 0 ||
      d_rowCount < 0) {
    set_error("callCompact: null state buffer or bad row range");
    return;
  }
  auto fail = [](cudaError_t e, const char *what) {
    cuda_fail(e, what, __FILE__, __LINE__);
    fprintf(stderr, "callCompact: %s\n", hpc_last_error_string());
  };
  cudaError_t e = cudaSetDevice(deviceId);
  if (e != cudaSuccess) return fail(e, "cudaSetDevice");
  const int64_t p = (int64_t)state->p;
  const int64_t row0 = (int64_t)idx * d_rowCount;
  const int64_t row1 = std::min<int64_t>(p, row0 + d_rowCount);
  // the reference resets max_adj on the host before its launch (compact.cu:94)
  if ((e = cudaMemset(state->max_adj, 0, sizeof(int))) != cudaSuccess) return fail(e, "cudaMemset(max_adj)");
  if (row1 > row0) {
    const int64_t warps = row1 - row0;
    const unsigned blocks = (unsigned)std::min<int64_t>((warps + 7) / 8, 152 * 16);
    compact_rows_kernel<<<blocks, 256>>>(state->adj, state->adj_compact, p, row0, row1, state->max_adj);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail(e, "compact_rows_kernel");
  }
  if ((e = cudaDeviceSynchronize()) != cudaSuccess) return fail(e, "cudaDeviceSynchronize");
}
