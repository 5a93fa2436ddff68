// SkeletonCalculator, GPUExecutor, CPU:: statistics and printSepsets over the C ABI.
// Reference shapes: src/independence/skeleton.cpp:13-190, src/executor/gpuExecutor.cu:9-122,
// src/executor/independence/cpuInd.cpp:8-38, src/util/sepset_util.hpp:9-60.
#include <algorithm>
#include <chrono>
#include <climits>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <thread>
#include <unordered_map>

#include "heterogpc.hpp"

void hpc_check(hpc_status s) {
  if (s != HPC_OK) throw HpcException(s, std::string(hpc_status_string(s)) + ": " + hpc_last_error_string());
}

namespace CPU {
double calcPValue(double r, int sampleSize) { return hpc_calc_pvalue(r, sampleSize); }
double pValL1(double x1, double x2, double x3, int sampleSize) { return hpc_pval_l1(x1, x2, x3, sampleSize); }
double pValLN(const double *M, int k, int observations) { return hpc_pval_ln(M, k, observations); }
}  // namespace CPU

TestResult GPUExecutor::executeLevel(int level, bool /*workstealing*/, bool verbose) {
  auto start = std::chrono::system_clock::now();
  hpc_check(hpc_run_level(state, level, &last));
  auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::system_clock::now() - start).count();
  if (verbose)
    std::cout << "\tGPU is done. Time: " << ms << " ms. Tests: " << last.executed_tests << " of "
              << last.potential_tests << ", FP64 re-tests: " << last.retests << std::endl;
  TestResult r;
  r.duration = (unsigned long long)ms;
  r.tests64 = last.executed_tests;
  r.tests = (int)std::min<long long>(last.executed_tests, INT_MAX);
  return r;
}

SkeletonCalculator::SkeletonCalculator(int maxLevel, double alpha, bool workstealing, std::string csvExportFile,
                                       int numThreads, bool verbose)
    : maxLevel_(maxLevel),
      alpha_(alpha),
      workstealing_(workstealing),
      csvExportFile_(std::move(csvExportFile)),
      numThreads_(numThreads),
      verbose_(verbose) {}

SkeletonCalculator::~SkeletonCalculator() {
  if (ctx_) hpc_ctx_destroy(ctx_);
}

void SkeletonCalculator::set_heterogeneity(Heterogeneity h) { heterogeneity_ = h; }
void SkeletonCalculator::set_gpu_list(std::vector<int> gpuList) {
  if (!gpuList.empty()) gpuList_ = std::move(gpuList);
}
void SkeletonCalculator::set_precision(int precision) { precision_ = precision; }

std::shared_ptr<Matrix> SkeletonCalculator::read_csv_file(const std::string &input_file) {
  if (verbose_) std::cout << "Reading file: " << input_file << std::endl;
  if (input_file.size() > 4 && input_file.compare(input_file.size() - 4, 4, ".npy") == 0)
    return NPYLoader::read_npy_to_mat(input_file);  // binary input, no reference counterpart
  if (input_file.find(".csv") == std::string::npos) {
    std::cout << "Cannot process file '" << input_file << "'." << std::endl;
    std::cout << "Has to be .csv format." << std::endl;
    std::exit(-1);  // the reference's CLI behaviour (skeleton.cpp:44-49)
  }
  std::vector<std::string> names;
  return CSVParser::read_csv_to_mat(input_file, names);
}

void SkeletonCalculator::create_context(int64_t p, int64_t n) {
  if (ctx_) hpc_ctx_destroy(ctx_);
  ctx_ = nullptr;
  hpc_opts o;
  hpc_opts_default(&o);
  o.device = gpuList_.front();
  o.alpha = alpha_;
  o.max_level = maxLevel_;
  o.precision = precision_;
  o.verbose = 0;
  hpc_check(hpc_ctx_create(&ctx_, p, n, &o));
  p_ = p;
  n_ = n;
}

void SkeletonCalculator::add_observations(const std::string &input_file, bool) {
  auto m = read_csv_file(input_file);
  create_context(m->n_cols, m->n_rows);
  hpc_check(hpc_correlation_f64(ctx_, m->memptr()));
}

void SkeletonCalculator::add_correlation_matrix(const std::string &input_file, int observation_count, bool) {
  auto m = read_csv_file(input_file);
  if (m->n_rows != m->n_cols) throw HpcException(HPC_ERR_INVALID_ARG, "correlation matrix is not square");
  create_context(m->n_cols, observation_count);
  // column-major symmetric matrix: the row-major load reads the same values
  // (for a non-symmetric file this is the transpose, as the reference's memcpy
  // of arma memory into state.cor is, skeleton.cpp:64)
  hpc_check(hpc_load_correlation(ctx_, m->memptr()));
}

void SkeletonCalculator::initialize_balancer(std::tuple<float, float, float>) {}

LevelMetrics SkeletonCalculator::calcLevel(int level) {
  auto start = std::chrono::system_clock::now();
  GPUExecutor gpu(ctx_, (int)std::min<int64_t>(INT_MAX, p_ * (p_ - 1) / 2), gpuList_);
  gpu.enqueueSplitTask(SplitTask{0, (int)p_});
  TestResult g = gpu.executeLevel(level, workstealing_, verbose_);
  last_ = gpu.last;
  if (verbose_) std::cout << "Max row length: " << gpu.last.max_degree << std::endl;
  int64_t levelDur =
      std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::system_clock::now() - start).count();
  TestResult c{0, 0, 0};
  return LevelMetrics{levelDur, 0, std::make_tuple(c, g)};
}

void SkeletonCalculator::export_metrics(const std::vector<LevelMetrics> &levelMetrics, int64_t executionDuration,
                                        int nrEdges) {
  if (csvExportFile_.empty()) return;
  if (verbose_) std::cout << "Export metrics to CSV file: " << csvExportFile_ << std::endl;
  std::ofstream f(csvExportFile_, std::ios::app | std::ios::out);
  // columns of skeleton.cpp:83-98: numGPUs, numOMPThreads, nrEdges,
  // {levelDur, balanceDur, cpuDur, gpuDur} per level, executionDuration
  f << (heterogeneity_ == Heterogeneity::CPUOnly ? 0 : (int)1) << ",";
  f << numThreads_ << ",";
  f << nrEdges << ",";
  for (const auto &m : levelMetrics) {
    const auto &res = std::get<2>(m);
    f << std::get<0>(m) << "," << std::get<1>(m) << "," << std::get<0>(res).duration << "," << std::get<1>(res).duration
      << ",";
  }
  f << executionDuration << std::endl;
}

void SkeletonCalculator::run(bool print_sepsets) {
  if (!ctx_) throw HpcException(HPC_ERR_STATE, "no observations or correlation matrix added");
  const int maxCondSize = std::max(maxLevel_, 1);
  if (verbose_) {
    std::cout << "Using following GPUs:" << std::endl;
    std::cout << "\t" << gpuList_.front() << std::endl;
    std::cout << "maxCondSize: " << maxCondSize << "  observations: " << n_ << "  p: " << p_
              << " number of GPUS: " << 1 << std::endl;
  }
  auto start = std::chrono::system_clock::now();
  std::vector<LevelMetrics> metrics;
  const int top = maxLevel_ < 0 ? HPC_MAX_LEVEL : maxLevel_;
  for (int lvl = 0; lvl <= top; ++lvl) {
    metrics.push_back(calcLevel(lvl));
    // with an open-ended max level, stop at the first level without tests
    if (maxLevel_ < 0 && lvl >= 1 && last_.potential_tests == 0) break;
  }
  int64_t executionDuration =
      std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::system_clock::now() - start).count();
  if (verbose_) std::cout << "Execution duration: " << executionDuration << " ms." << std::endl;
  nrEdges_ = printSepsets(ctx_, p_, maxCondSize, print_sepsets, verbose_);
  export_metrics(metrics, executionDuration, nrEdges_);
}

int printSepsets(hpc_ctx *ctx, int64_t p, int maxCondSize, bool showSepsets, bool verbose) {
  std::vector<uint8_t> adj((size_t)(p * p));
  hpc_check(hpc_get_adjacency(ctx, adj.data()));
  std::unordered_map<int64_t, hpc_sepset_record> recs;
  if (showSepsets) {
    int64_t n = 0;
    hpc_check(hpc_get_sepset_records(ctx, nullptr, 0, &n));
    std::vector<hpc_sepset_record> v((size_t)n);
    if (n) hpc_check(hpc_get_sepset_records(ctx, v.data(), n, &n));
    recs.reserve((size_t)n);
    for (const auto &r : v) recs[(int64_t)r.i * p + r.j] = r;
  }
  int nrEdges = 0;
  std::string out;
  for (int64_t i = 0; i < p; ++i) {
    for (int64_t j = i + 1; j < p; ++j) {
      if (adj[i * p + j]) {
        ++nrEdges;
        continue;
      }
      if (!showSepsets) continue;
      auto it = recs.find(i * p + j);
      if (it == recs.end()) {
        out += "Separation from " + std::to_string(i) + " to " + std::to_string(j) + "\n";
      } else {
        std::string s;
        for (int k = 0; k < std::min(it->second.level, maxCondSize); ++k) s += std::to_string(it->second.ids[k]) + " ";
        out += "Separation from " + std::to_string(i) + " to " + std::to_string(j) + " via " + s + "\n";
      }
      if (out.size() > (1u << 20)) {
        std::cout << out;
        out.clear();
      }
    }
  }
  std::cout << out;
  if (verbose) std::cout << "Total number of edges: " << nrEdges << std::endl;
  return nrEdges;
}
