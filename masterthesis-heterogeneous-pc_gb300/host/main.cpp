// heterogpc command line (src/main.cpp:17-141): same flags, defaults, messages and
// exit codes. Flags that steer the reference's CPU side (--cpu-only, -w, --row-mult*,
// --power9-ats, -t) are accepted; every CI test here runs on the GPU work queue,
// so they change nothing and a note says so. New: --precision fp64|mixed|mixed-tc,
// --autotune and --tune-file (the CI tests' tile policy, hpc_autotune / hpc_tune_*).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "heterogpc.hpp"

#ifdef __linux__
static const std::string DEFAULT_INPUT_FILE = "../../data/cooling_house.csv";
#else
static const std::string DEFAULT_INPUT_FILE = "../../../data/cooling_house.csv";
#endif

namespace {

struct Opt {
  std::string long_name;
  char short_name;
  bool takes_value;
  bool multitoken;
  std::string help;
  std::string deflt;
};

const std::vector<Opt> kOpts = {
    {"help", 0, false, false, "produce a help message", ""},
    {"input-file", 'i', true, false, "input file", DEFAULT_INPUT_FILE},
    {"alpha", 'a', true, false, "alpha value", "0.05"},
    {"observations", 'o', true, false, "observation count", ""},
    {"row-mult", 0, true, false, "maximum rows balanced multiplier level 0,1,4+ (no effect here)", "0.2"},
    {"row-mult2", 0, true, false, "maximum rows balanced multiplier level 2 (no effect here)", "0.2"},
    {"row-mult3", 0, true, false, "maximum rows balanced multiplier level 3 (no effect here)", "0.1"},
    {"max-level", 'm', true, false, "maximum level (-1: until no edge has enough neighbours)", "4"},
    {"corr", 0, false, false, "input file is a correlation matrix", ""},
    {"gpus", 'g', true, true, "GPU deviceIds that should be used (the first one runs)", ""},
    {"thread-count", 't', true, false, "number of host threads (no effect here)", ""},
    {"csv-export", 0, true, false, "Export runtimes execution metrics to CSV", ""},
    {"gpu-only", 0, false, false, "execution on gpu only", ""},
    {"cpu-only", 0, false, false, "execution on cpu only (no effect here: the GPU runs every test)", ""},
    {"power9-ats", 0, false, false, "Use power9 system allocator for ATS (no effect here)", ""},
    {"workstealing", 'w', false, false, "use workstealing CPU executor (no effect here)", ""},
    {"print-sepsets", 'p', false, false, "prints-sepsets", ""},
    {"verbose", 'v', false, false, "verbose output", ""},
    {"precision", 0, true, false, "CI-test precision: fp64, mixed (default) or mixed-tc", "mixed"},
    {"autotune", 0, false, false, "time the tile-policy candidates on this input before the run", ""},
    {"tune-file", 0, true, false, "tile-policy table: loaded before the run, written after --autotune", ""},
    {"io-benchmark", 0, false, false, "only read the input file (.csv or .npy) and report the read rate", ""},
};

const Opt *find_long(const std::string &n) {
  for (const auto &o : kOpts)
    if (o.long_name == n) return &o;
  return nullptr;
}
const Opt *find_short(char c) {
  for (const auto &o : kOpts)
    if (o.short_name == c) return &o;
  return nullptr;
}

void print_help() {
  std::cout << "Allowed options:\n";
  for (const auto &o : kOpts) {
    std::string s = "  ";
    if (o.short_name) s += std::string("-") + o.short_name + " [ --" + o.long_name + " ]";
    else s += "--" + o.long_name;
    if (o.takes_value) s += " arg";
    if (!o.deflt.empty()) s += " (=" + o.deflt + ")";
    if (s.size() < 42) s += std::string(42 - s.size(), ' ');
    std::cout << s << " " << o.help << "\n";
  }
}

struct ParseError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// values[name] = list of values ("" for flags)
std::map<std::string, std::vector<std::string>> parse(int argc, char const *argv[]) {
  std::map<std::string, std::vector<std::string>> v;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    const Opt *o = nullptr;
    std::string val;
    bool have_val = false;
    if (a.rfind("--", 0) == 0) {
      std::string name = a.substr(2);
      size_t eq = name.find('=');
      if (eq != std::string::npos) {
        val = name.substr(eq + 1);
        name = name.substr(0, eq);
        have_val = true;
      }
      o = find_long(name);
      if (!o) throw ParseError("unrecognised option '" + a + "'");
    } else if (a.size() >= 2 && a[0] == '-' && !(a[1] >= '0' && a[1] <= '9') && a[1] != '.') {
      o = find_short(a[1]);
      if (!o) throw ParseError("unrecognised option '" + a + "'");
      if (a.size() > 2) {
        val = a.substr(2);
        have_val = true;
      }
    } else {
      throw ParseError("unexpected positional argument '" + a + "'");
    }
    auto &slot = v[o->long_name];
    if (!o->takes_value) {
      if (have_val) throw ParseError("option '--" + o->long_name + "' does not take any arguments");
      slot.push_back("");
      continue;
    }
    if (!have_val) {
      if (i + 1 >= argc) throw ParseError("the required argument for option '--" + o->long_name + "' is missing");
      val = argv[++i];
    }
    if (!slot.empty() && !o->multitoken) throw ParseError("option '--" + o->long_name + "' cannot be specified more than once");
    slot.push_back(val);
    if (o->multitoken)
      while (i + 1 < argc && argv[i + 1][0] != '-') slot.push_back(argv[++i]);
  }
  return v;
}

double to_double(const std::string &name, const std::string &s) {
  char *e = nullptr;
  double d = std::strtod(s.c_str(), &e);
  if (s.empty() || *e) throw ParseError("the argument ('" + s + "') for option '--" + name + "' is invalid");
  return d;
}

int to_int(const std::string &name, const std::string &s) {
  char *e = nullptr;
  long d = std::strtol(s.c_str(), &e, 10);
  if (s.empty() || *e) throw ParseError("the argument ('" + s + "') for option '--" + name + "' is invalid");
  return (int)d;
}

}  // namespace

int main(int argc, char const *argv[]) {
  std::map<std::string, std::vector<std::string>> vm;
  try {
    vm = parse(argc, argv);
  } catch (const ParseError &e) {
    std::cerr << "Error: " << e.what() << "\n";
    return 1;
  }
  if (vm.count("help")) {
    print_help();
    return 0;
  }
  auto get = [&](const char *n) -> std::string {
    auto it = vm.find(n);
    if (it != vm.end() && !it->second.empty()) return it->second.front();
    return find_long(n)->deflt;
  };
  double alpha;
  int maxLevel, numberOfThreads = (int)std::thread::hardware_concurrency();
  std::vector<int> gpus;
  int precision = HPC_PREC_MIXED;
  try {
    alpha = to_double("alpha", get("alpha"));
    maxLevel = to_int("max-level", get("max-level"));
    if (vm.count("thread-count")) numberOfThreads = to_int("thread-count", get("thread-count"));
    for (const char *n : {"row-mult", "row-mult2", "row-mult3"}) to_double(n, get(n));
    if (vm.count("gpus"))
      for (const auto &g : vm["gpus"]) gpus.push_back(to_int("gpus", g));
    const std::string prec = get("precision");
    if (prec == "fp64") precision = HPC_PREC_FP64;
    else if (prec == "mixed") precision = HPC_PREC_MIXED;
    else if (prec == "mixed-tc") precision = HPC_PREC_MIXED_TC;
    else throw ParseError("the argument ('" + prec + "') for option '--precision' is invalid");
  } catch (const ParseError &e) {
    std::cerr << "Error: " << e.what() << "\n";
    return 1;
  }
  const bool verbose = vm.count("verbose") != 0;
  const bool workstealing = vm.count("workstealing") != 0;
  const std::string inputFile = get("input-file");
  const std::string csvExportFile = vm.count("csv-export") ? get("csv-export") : "";
  if (vm.count("cpu-only") || workstealing || vm.count("power9-ats") || vm.count("row-mult") ||
      vm.count("row-mult2") || vm.count("row-mult3"))
    std::cerr << "note: --cpu-only, --workstealing, --power9-ats and --row-mult* have no effect: "
                 "every CI test runs on the GPU work queue\n";
  if (gpus.size() > 1) std::cerr << "note: one GPU per process; using device " << gpus.front() << "\n";

  if (vm.count("io-benchmark")) {
    // the input reader alone: values and megabytes of the file per second
    try {
      SkeletonCalculator probe(maxLevel, alpha, false, "", numberOfThreads, false);
      FILE *fh = std::fopen(inputFile.c_str(), "rb");
      long long fbytes = 0;
      if (fh) {
        std::fseek(fh, 0, SEEK_END);
        fbytes = std::ftell(fh);
        std::fclose(fh);
      }
      const auto t0 = std::chrono::steady_clock::now();
      auto m = probe.read_csv_file(inputFile);
      const double s_ = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      std::printf("read %lld x %lld values from %lld bytes in %.3f s: %.1f MB/s of file, %.1f M values/s\n",
                  (long long)m->n_rows, (long long)m->n_cols, fbytes, s_, fbytes / s_ / 1e6,
                  (double)(m->n_rows * m->n_cols) / s_ / 1e6);
    } catch (const HpcException &e) {
      std::cerr << "Error: " << e.what() << "\n";
      return 2;
    }
    return 0;
  }
  try {
    // the tile-policy table is read first (a bad file fails before any GPU work)
    const std::string tuneFile = vm.count("tune-file") ? get("tune-file") : "";
    if (!tuneFile.empty() && !vm.count("autotune")) {
      const hpc_status st = hpc_tune_load(tuneFile.c_str());
      if (st != HPC_OK) throw HpcException(st, hpc_last_error_string());
    }
    SkeletonCalculator sk(maxLevel, alpha, workstealing, csvExportFile, numberOfThreads, verbose);
    if (vm.count("gpu-only")) sk.set_heterogeneity(Heterogeneity::GPUOnly);
    else if (vm.count("cpu-only")) sk.set_heterogeneity(Heterogeneity::CPUOnly);
    if (!gpus.empty()) sk.set_gpu_list(gpus);
    sk.set_precision(precision);
    const bool print_sepsets = vm.count("print-sepsets") != 0;
    if (vm.count("corr")) {
      if (!vm.count("observations")) {
        std::cout << "Observation count needed with correlation matrix input" << std::endl;
        return -1;
      }
      sk.add_correlation_matrix(inputFile, to_int("observations", get("observations")));
    } else {
      sk.add_observations(inputFile);
    }
    sk.initialize_balancer({(float)to_double("row-mult", get("row-mult")), (float)to_double("row-mult2", get("row-mult2")),
                            (float)to_double("row-mult3", get("row-mult3"))});
    if (vm.count("autotune")) {
      int entries = 0;
      hpc_status st = hpc_autotune(sk.context(), nullptr, 0, 1, nullptr, &entries);
      if (st != HPC_OK) throw HpcException(st, hpc_last_error_string());
      std::cerr << "autotune: " << entries << " tile-policy entries" << std::endl;
      if (!tuneFile.empty() && (st = hpc_tune_save(tuneFile.c_str())) != HPC_OK)
        throw HpcException(st, hpc_last_error_string());
    }
    sk.run(print_sepsets);
  } catch (const HpcException &e) {
    std::cerr << "Error: " << e.what() << "\n";
    return 2;
  } catch (const ParseError &e) {
    std::cerr << "Error: " << e.what() << "\n";
    return 1;
  }
  return 0;
}
