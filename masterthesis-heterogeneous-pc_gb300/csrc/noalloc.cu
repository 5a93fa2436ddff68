// Correlation matrix without any device allocation.
//
// Some callers cannot allocate device memory at the moment they need a
// correlation matrix: a plugin inside a host application that owns all of the
// GPU's memory through its own pool and forbids other allocations, or a
// latency-critical caller that cannot afford cudaMalloc / cudaFree, which may
// synchronise the whole device. hpc_correlation_noalloc_f64 serves them: the
// caller passes the observations and the output matrix (device memory it
// already owns), and the standardised copy of the data that the Gram reads
// lives in one file-scope __device__ array instead of a cudaMalloc'd buffer.
//
// Limits and rules:
//  * n_obs * p <= HPC_NOALLOC_MAX_ELEMS (4,194,304 FP64 values, 32 MiB). The
//    array is part of the library image, so every GPU that loads the library
//    holds these 32 MiB until the process exits. Larger inputs are rejected
//    with HPC_ERR_CAPACITY before anything is launched.
//  * Host code cannot use the array's name as a device address (on the host it
//    names a host-side stand-in). The first call on each device looks the
//    address up with cudaGetSymbolAddress, with that device current, and
//    caches it; make that first call on a device before any stream capture.
//  * Every call shares the one array and it keeps the last call's contents.
//    Nothing here needs it cleared: the standardisation writes every one of the
//    n_obs * p values the Gram then reads. Calls whose work overlaps on the GPU
//    (different streams, or different host threads) race on the array; order
//    them on one stream or serialise them.
//  * The shapes the grouped kernels read (offsets, sizes, tile counts) also live in
//    a file-scope __device__ struct, written by a one-thread kernel (the values
//    travel as its launch parameter, so no host memory is copied and the call does
//    not wait for the stream) on the caller's stream, and are shared between calls
//    the same way.
//  * No cudaMalloc, cudaFree or allocating library routine is called.
#include <cuda_runtime.h>

#include <mutex>

#include "internal.cuh"

namespace hpc {
namespace {

constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_corr_scratch[HPC_NOALLOC_MAX_ELEMS];

// Shape metadata of one instance in the layout the grouped standardisation and Gram
// kernels read (StdArgs / GramArgs with count = 1).
struct NoallocMeta {
  long long row_prefix[2], x_off, z_off, n, tc_off, n_pad, kdim;
  long long tile_prefix[2], c_off, p;
  double denom;
};
static __device__ NoallocMeta g_meta;

// writes the shapes of this call where the grouped kernels read them
__global__ void set_meta_kernel(NoallocMeta m) { g_meta = m; }

std::mutex g_scratch_mu;
double *g_scratch_addr[kMaxDevices] = {};
NoallocMeta *g_meta_addr[kMaxDevices] = {};

hpc_status scratch_for_current_device(double **out, NoallocMeta **meta) {
  int dev = -1;
  HPC_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("device ordinal %d outside the supported range [0, %d)", dev, kMaxDevices);
    return HPC_ERR_INVALID_ARG;
  }
  std::lock_guard<std::mutex> g(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_corr_scratch);
    if (e != cudaSuccess || !ptr) {
      cudaGetLastError();
      set_error("cudaGetSymbolAddress of the correlation scratch failed on device %d: %s", dev,
                cudaGetErrorString(e));
      return HPC_ERR_CUDA;
    }
    g_scratch_addr[dev] = (double *)ptr;
    void *mp = nullptr;
    e = cudaGetSymbolAddress(&mp, g_meta);
    if (e != cudaSuccess || !mp) {
      cudaGetLastError();
      set_error("cudaGetSymbolAddress of the correlation metadata failed on device %d: %s", dev,
                cudaGetErrorString(e));
      g_scratch_addr[dev] = nullptr;
      return HPC_ERR_CUDA;
    }
    g_meta_addr[dev] = (NoallocMeta *)mp;
  }
  *out = g_scratch_addr[dev];
  *meta = g_meta_addr[dev];
  return HPC_OK;
}

}  // namespace
}  // namespace hpc

extern "C" hpc_status hpc_correlation_noalloc_f64(const double *X_dev, int64_t n_obs, int64_t p, int ref_compat_sd,
                                                  double *C_dev, void *stream) {
  using namespace hpc;
  if (!X_dev || !C_dev) {
    set_error("null observation or output pointer");
    return HPC_ERR_INVALID_ARG;
  }
  if (p < 1 || n_obs < 2) {
    set_error("p = %lld, n_obs = %lld: need p >= 1 and n_obs >= 2", (long long)p, (long long)n_obs);
    return HPC_ERR_INVALID_ARG;
  }
  if (n_obs > HPC_NOALLOC_MAX_ELEMS / p) {
    set_error("n_obs * p = %lld exceeds the allocation-free limit of %lld values; use hpc_correlation_device_f64",
              (long long)n_obs * (long long)p, (long long)HPC_NOALLOC_MAX_ELEMS);
    return HPC_ERR_CAPACITY;
  }
  double *Z = nullptr;
  NoallocMeta *md = nullptr;
  hpc_status s = scratch_for_current_device(&Z, &md);
  if (s != HPC_OK) return s;
  cudaStream_t st = (cudaStream_t)stream;
  NoallocMeta m{};
  m.row_prefix[0] = 0;
  m.row_prefix[1] = p;
  m.n = n_obs;
  m.tile_prefix[0] = 0;
  m.tile_prefix[1] = gram_f64_tiles(p);
  m.p = p;
  m.denom = ref_compat_sd ? (double)((float)n_obs - 1.f) : (double)(n_obs - 1);
  set_meta_kernel<<<1, 1, 0, st>>>(m);
  HPC_LAUNCH_CHECK("set_meta_kernel");
  StdArgs sa{};
  sa.count = 1;
  sa.row_prefix = md->row_prefix;
  sa.x_off = &md->x_off;
  sa.z_off = &md->z_off;
  sa.n = &md->n;
  sa.tc_off = &md->tc_off;
  sa.n_pad = &md->n_pad;
  sa.kdim = &md->kdim;
  sa.ref_compat = ref_compat_sd;
  if ((s = launch_standardise(X_dev, false, sa, p, Z, nullptr, 0, nullptr, st)) != HPC_OK) return s;
  GramArgs ga{};
  ga.count = 1;
  ga.tile_prefix = md->tile_prefix;
  ga.z_off = &md->z_off;
  ga.c_off = &md->c_off;
  ga.n = &md->n;
  ga.p = &md->p;
  ga.denom = &md->denom;
  return launch_gram_f64(Z, C_dev, ga, gram_f64_tiles(p), st);
}
