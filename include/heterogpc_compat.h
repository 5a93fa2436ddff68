/*
 * heterogpc_compat.h -- the reference's correlation and compaction entry points with
 * their own C++ names and signatures, exported by libheterogpc.so, for callers written
 * against milanpro/Masterthesis-Heterogeneous-PC (paths relative to its source tree).
 *
 * These are C++ declarations (C++ linkage, as the reference declares them), so that an
 * object file compiled against the reference's corOwn.cuh / compact.cuh links against
 * libheterogpc.so unchanged. New code should use the C ABI in heterogpc.h.
 */
#ifndef HETEROGPC_COMPAT_H
#define HETEROGPC_COMPAT_H

#include <stdint.h>

/* The reference's state struct (src/util/state.cuh:29-56), data members in the same order
 * and of the same types (statusbool is bool in the reference's default build), so that a
 * pointer to the caller's MMState can be passed through. Only the members callCompact
 * reads or writes are used: p, adj, adj_compact, max_adj. */
struct MMState {
  bool ats;
  double *pMax;
  int *adj;
  int *adj_compact;
  double *cor;
  int *sepSets;
  uint64_t p;
  int observations;
  double alpha;
  int maxCondSize;
  int *max_adj;
  int *lock;
  int maxLevel;
  bool *node_status;
  bool gpu_done;
};

/* Replaces gpuPMCC (src/correlation/corOwn.cuh:3, corOwn.cu:10-48): the p x p Pearson
 * correlation (row-major, written to cors) of h_mat, column-major dim x n (n = variables,
 * dim = observations, each variable's samples contiguous: arma::mat's layout), computed on
 * device deviceId with the reference's arithmetic: NaN samples skipped pairwise and the
 * standard deviation rounded through float (corHelper.cu:22-28,75,98-106). Synchronous.
 * The reference exits the process on a CUDA error; here cors is filled with NaN and the
 * reason is left in hpc_last_error_string(). */
void gpuPMCC(const double *h_mat, uint64_t n, int dim, double *cors, int deviceId, bool verbose);

/* Replaces callCompact (src/independence/compact.cuh:7-8, compact.cu:91-99): for rows
 * idx * d_rowCount ... (idx + 1) * d_rowCount - 1 (and < p), the ascending ids of the
 * row's neighbours (adj[row * p + j] != 0) go to adj_compact[row * p + 0 ..], the rest of
 * the row up to slot p - 2 is zeroed, the count goes to adj_compact[row * p + p - 1], and
 * *max_adj receives the largest count (reset first, as the reference does on the host).
 * adj, adj_compact and max_adj must be device-accessible (managed memory, as MMState
 * allocates them, or device memory). numberOfGPUs is accepted for the signature's sake.
 * Synchronous; errors as gpuPMCC. */
void callCompact(MMState *state, int deviceId, int idx, int numberOfGPUs, int d_rowCount);

#endif /* HETEROGPC_COMPAT_H */
