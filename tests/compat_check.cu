// Drop-in check of the reference-named entry points exported by libheterogpc.so
// (include/heterogpc_compat.h, include/heterogpc_gpu_ind.cuh): a program written the
// way a caller of the reference's corOwn.cuh / compact.cuh / gpuInd.cuh is, linked
// against the library. tests/test_gpu_compat.py builds it with nvcc, runs it and
// compares its outputs with the oracle. Usage: compat_check <output directory>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "../include/heterogpc.h"
#include "../include/heterogpc_compat.h"
#include "../include/heterogpc_gpu_ind.cuh"

static void put(const std::string &dir, const char *name, const void *data, size_t bytes) {
  FILE *f = fopen((dir + "/" + name).c_str(), "wb");
  if (!f || fwrite(data, 1, bytes, f) != bytes) {
    fprintf(stderr, "cannot write %s\n", name);
    exit(2);
  }
  fclose(f);
}

__global__ void pvalues_kernel(const double *r, const double *x, int n_obs, int k, double *p0, double *p1) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < k) {
    p0[t] = GPU::calcPValue(r[t], n_obs);
    p1[t] = GPU::pValL1(x[3 * t], x[3 * t + 1], x[3 * t + 2], n_obs);
  }
}

int main(int argc, char **argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: compat_check <output directory>\n");
    return 2;
  }
  const std::string dir = argv[1];
  // observations: column-major dim x n (arma::mat), from the library's generator
  const int p = 40, dim = 500;
  hpc_sem_params prm = {p, dim, HPC_GRAPH_ER, 3.0, 2, 0.1, 1.0, 77};
  std::vector<double> X((size_t)p * dim), cors((size_t)p * p);
  if (hpc_sem_generate(&prm, X.data(), nullptr, nullptr, nullptr) != HPC_OK) return 3;
  X[3 * dim + 5] = X[3 * dim + 17] = std::nan("");  // missing samples of variable 3
  gpuPMCC(X.data(), p, dim, cors.data(), 0, false);
  put(dir, "X.f64", X.data(), X.size() * 8);
  put(dir, "cors.f64", cors.data(), cors.size() * 8);

  // an MMState in managed memory, as the reference's constructor makes it
  // (src/util/state.cu:3-44), with a symmetric random adjacency
  const int q = 70;
  MMState st{};
  st.p = q;
  if (cudaMallocManaged(&st.adj, sizeof(int) * q * q) != cudaSuccess ||
      cudaMallocManaged(&st.adj_compact, sizeof(int) * q * q) != cudaSuccess ||
      cudaMallocManaged(&st.max_adj, sizeof(int)) != cudaSuccess)
    return 4;
  uint64_t s = 12345;
  for (int i = 0; i < q; ++i) st.adj[i * q + i] = 0;
  for (int i = 0; i < q; ++i)
    for (int j = i + 1; j < q; ++j) {
      s = s * 6364136223846793005ull + 1442695040888963407ull;
      const int v = (int)((s >> 33) % 100) < (i < 5 ? 90 : 12);  // a few dense rows
      st.adj[i * q + j] = st.adj[j * q + i] = v;
    }
  for (int k = 0; k < q * q; ++k) st.adj_compact[k] = -7;
  callCompact(&st, 0, 0, 1, q);  // every row on one GPU
  put(dir, "adj.i32", st.adj, sizeof(int) * q * q);
  put(dir, "compact_all.i32", st.adj_compact, sizeof(int) * q * q);
  put(dir, "max_all.i32", st.max_adj, sizeof(int));
  for (int k = 0; k < q * q; ++k) st.adj_compact[k] = -7;
  callCompact(&st, 0, 1, 3, 24);  // the second of three row blocks of 24 rows
  put(dir, "compact_blk.i32", st.adj_compact, sizeof(int) * q * q);
  put(dir, "max_blk.i32", st.max_adj, sizeof(int));

  // the device statistics against their host versions (written for the oracle check)
  const int k = 64, n_obs = 900;
  std::vector<double> r(k), x(3 * k), p0(k), p1(k), h0(k), h1(k);
  for (int t = 0; t < k; ++t) {
    r[t] = -0.99 + 1.98 * t / (k - 1);
    x[3 * t] = 0.6 * r[t];
    x[3 * t + 1] = 0.3 - 0.004 * t;
    x[3 * t + 2] = -0.2 + 0.006 * t;
    h0[t] = GPU::calcPValue(r[t], n_obs);
    h1[t] = GPU::pValL1(x[3 * t], x[3 * t + 1], x[3 * t + 2], n_obs);
  }
  r[3] = std::nan("");
  h0[3] = GPU::calcPValue(r[3], n_obs);
  double *dr, *dx, *d0, *d1;
  cudaMalloc(&dr, 8 * k);
  cudaMalloc(&dx, 24 * k);
  cudaMalloc(&d0, 8 * k);
  cudaMalloc(&d1, 8 * k);
  cudaMemcpy(dr, r.data(), 8 * k, cudaMemcpyHostToDevice);
  cudaMemcpy(dx, x.data(), 24 * k, cudaMemcpyHostToDevice);
  pvalues_kernel<<<1, 64>>>(dr, dx, n_obs, k, d0, d1);
  if (cudaDeviceSynchronize() != cudaSuccess) return 5;
  cudaMemcpy(p0.data(), d0, 8 * k, cudaMemcpyDeviceToHost);
  cudaMemcpy(p1.data(), d1, 8 * k, cudaMemcpyDeviceToHost);
  put(dir, "r.f64", r.data(), 8 * k);
  put(dir, "x.f64", x.data(), 24 * k);
  put(dir, "dev_p0.f64", p0.data(), 8 * k);
  put(dir, "dev_p1.f64", p1.data(), 8 * k);
  put(dir, "host_p0.f64", h0.data(), 8 * k);
  put(dir, "host_p1.f64", h1.data(), 8 * k);
  printf("compat_check ok\n");
  return 0;
}
