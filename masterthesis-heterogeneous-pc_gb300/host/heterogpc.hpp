// C++ host interface of the GB300 skeleton library, mirroring the reference's
// classes so that code written against them keeps compiling:
//   SplitTask / TestResult          src/util/indep_util.hpp:4-16
//   Executor / GPUExecutor          src/executor/executor.hpp:6-22, src/executor/gpuExecutor.cuh:3-14
//   SkeletonCalculator              src/independence/skeleton.hpp:10-73
//   CPU::calcPValue/pValL1/pValLN   src/executor/independence/cpuInd.hpp:3-10
//   CSVParser::read_csv_to_mat      src/util/csv_parser.hpp:6-9
//   printSepsets                    src/util/sepset_util.hpp:9-60
// Everything computes through the C ABI (include/heterogpc.h) on one GPU; the
// balancer and heterogeneity settings of the reference have no CPU side to steer
// and are accepted as no-ops.
#pragma once
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/heterogpc.h"

// src/util/indep_util.hpp:4-16
struct SplitTask {
  int row;
  int rowCount;
};

struct TestResult {
  unsigned long long duration;  // ms
  int tests;                    // executed CI tests (saturated to INT_MAX)
  long long tests64;            // executed CI tests
};

enum class Heterogeneity { All, CPUOnly, GPUOnly };

// Thrown for any failing C ABI call; carries the status and the library message.
struct HpcException : std::runtime_error {
  hpc_status status;
  HpcException(hpc_status s, const std::string &m) : std::runtime_error(m), status(s) {}
};
void hpc_check(hpc_status s);

// Observation or correlation matrix as read from CSV: column-major n_rows x n_cols
// (each column -- a variable -- contiguous), the arma::mat layout of the reference.
struct Matrix {
  int64_t n_rows = 0, n_cols = 0;
  std::vector<double> data;
  const double *colptr(int64_t c) const { return data.data() + c * n_rows; }
  double *memptr() { return data.data(); }
};

namespace CSVParser {
// src/util/csv_parser.cpp:20-77: comma separated doubles, optional header line.
std::shared_ptr<Matrix> read_csv_to_mat(const std::string &filename, std::vector<std::string> &column_names);
}  // namespace CSVParser

namespace NPYLoader {
// binary input (no reference counterpart): a 2-D float64/float32 .npy file, rows =
// observations, columns = variables, read into the column-major layout above
std::shared_ptr<Matrix> read_npy_to_mat(const std::string &filename);
}  // namespace NPYLoader

namespace CPU {
double calcPValue(double r, int sampleSize);
double pValL1(double x1, double x2, double x3, int sampleSize);
// M: row-major k x k correlation submatrix ordered (i, j, S...)
double pValLN(const double *M, int k, int observations);
}  // namespace CPU

struct Executor {
  std::vector<SplitTask> tasks;
  void enqueueSplitTask(SplitTask task) { tasks.push_back(task); }
  void cleanupSplitTasks() { tasks.clear(); }
};

// One level of CI tests on the GPU (src/executor/gpuExecutor.cu:9-122). The
// device work queue covers every row, so the split tasks only matter for
// compatibility.
struct GPUExecutor : Executor {
  int maxEdgeCount;
  std::vector<int> gpuList;
  hpc_ctx *state;
  GPUExecutor(hpc_ctx *state, int maxEdgeCount, std::vector<int> gpuList)
      : maxEdgeCount(maxEdgeCount), gpuList(std::move(gpuList)), state(state) {}
  TestResult executeLevel(int level, bool workstealing, bool verbose = false);
  hpc_level_stats last{};
};

typedef std::tuple<int64_t, int64_t, std::tuple<TestResult, TestResult>> LevelMetrics;

class SkeletonCalculator {
 public:
  SkeletonCalculator(int maxLevel, double alpha, bool workstealing, std::string csvExportFile, int numThreads,
                     bool verbose = false);
  ~SkeletonCalculator();
  SkeletonCalculator(const SkeletonCalculator &) = delete;
  SkeletonCalculator &operator=(const SkeletonCalculator &) = delete;

  void set_heterogeneity(Heterogeneity heterogeneity);
  void set_gpu_list(std::vector<int> gpuList);
  // precision of the CI tests (hpc_precision); default HPC_PREC_MIXED
  void set_precision(int precision);
  std::shared_ptr<Matrix> read_csv_file(const std::string &input_file);
  void add_observations(const std::string &input_file, bool use_p9_ats = false);
  void add_correlation_matrix(const std::string &input_file, int observation_count, bool use_p9_ats = false);
  void initialize_balancer(std::tuple<float, float, float> balancer_thresholds);
  void run(bool print_sepsets);
  LevelMetrics calcLevel(int level);
  void export_metrics(const std::vector<LevelMetrics> &levelMetrics, int64_t executionDuration, int nrEdges);

  hpc_ctx *context() const { return ctx_; }
  int edges() const { return nrEdges_; }

 private:
  void create_context(int64_t p, int64_t n);
  int maxLevel_;
  double alpha_;
  bool workstealing_;
  std::string csvExportFile_;
  int numThreads_;
  bool verbose_;
  int precision_ = HPC_PREC_MIXED;
  Heterogeneity heterogeneity_ = Heterogeneity::All;
  std::vector<int> gpuList_{0};
  hpc_ctx *ctx_ = nullptr;
  int64_t p_ = 0, n_ = 0;
  int nrEdges_ = 0;
  hpc_level_stats last_{};
};

// src/util/sepset_util.hpp:9-60: counts the i<j edges left and, with showSepsets,
// prints "Separation from i to j via ..." lines in the reference's format.
int printSepsets(hpc_ctx *ctx, int64_t p, int maxCondSize, bool showSepsets, bool verbose);
