// Binary input of the heterogpc CLI: NumPy .npy files (format versions 1-3, little-
// endian float64 or float32, two dimensions, C or Fortran order), the fast alternative
// to the reference's text-only reader (src/util/csv_parser.cpp:20-77, whose
// observation and --corr inputs, src/independence/skeleton.cpp:53-65, are CSV only).
// The array's rows are observations and its columns variables, as in the CSV files;
// the result is column-major (each variable contiguous), the layout of the C ABI's
// observation input. A Fortran-order float64 file is read straight into place; other
// files are read in one piece and converted or transposed in parallel, in blocks.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "heterogpc.hpp"

namespace {

[[noreturn]] void bad(const std::string &file, const std::string &why) {
  throw HpcException(HPC_ERR_INVALID_ARG, "cannot read '" + file + "' as .npy: " + why);
}

// the value of `key` in the header dictionary, e.g. 'descr': '<f8'
std::string field(const std::string &hdr, const std::string &key) {
  const size_t k = hdr.find("'" + key + "'");
  if (k == std::string::npos) return "";
  size_t v = hdr.find(':', k);
  if (v == std::string::npos) return "";
  ++v;
  while (v < hdr.size() && hdr[v] == ' ') ++v;
  size_t e = v;
  if (hdr[v] == '(') {
    e = hdr.find(')', v);
    return e == std::string::npos ? "" : hdr.substr(v, e - v + 1);
  }
  if (hdr[v] == '\'') {
    e = hdr.find('\'', v + 1);
    return e == std::string::npos ? "" : hdr.substr(v + 1, e - v - 1);
  }
  while (e < hdr.size() && hdr[e] != ',' && hdr[e] != '}') ++e;
  return hdr.substr(v, e - v);
}

template <typename F>
void parallel_rows(int64_t n, F f) {
  const unsigned nth = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  std::vector<std::thread> pool;
  for (unsigned t = 0; t < nth; ++t)
    pool.emplace_back([&, t]() {
      const int64_t a = n * t / nth, b = n * (t + 1) / nth;
      f(a, b);
    });
  for (auto &th : pool) th.join();
}

}  // namespace

std::shared_ptr<Matrix> NPYLoader::read_npy_to_mat(const std::string &filename) {
  FILE *f = std::fopen(filename.c_str(), "rb");
  if (!f) {
    std::printf("Could not find file '%s'\n", filename.c_str());
    std::exit(1);  // as the CSV reader (src/util/csv_parser.cpp:22-25)
  }
  unsigned char pre[10];
  if (std::fread(pre, 1, 10, f) != 10 || std::memcmp(pre, "\x93NUMPY", 6) != 0) {
    std::fclose(f);
    bad(filename, "no .npy magic");
  }
  const int major = pre[6];
  uint32_t hlen = pre[8] | (pre[9] << 8);
  if (major >= 2) {  // versions 2 and 3: a 4-byte header length
    unsigned char ext[2];
    if (std::fread(ext, 1, 2, f) != 2) {
      std::fclose(f);
      bad(filename, "truncated header");
    }
    hlen |= (uint32_t)ext[0] << 16 | (uint32_t)ext[1] << 24;
  }
  std::string hdr(hlen, '\0');
  if (std::fread(&hdr[0], 1, hlen, f) != hlen) {
    std::fclose(f);
    bad(filename, "truncated header");
  }
  const std::string descr = field(hdr, "descr"), order = field(hdr, "fortran_order"), shape = field(hdr, "shape");
  int esize = 0;
  if (descr == "<f8" || descr == "|f8") esize = 8;
  else if (descr == "<f4" || descr == "|f4") esize = 4;
  else {
    std::fclose(f);
    bad(filename, "dtype '" + descr + "' (float64 or float32, little-endian, are read)");
  }
  long long rr = -1, cc = -1;
  if (std::sscanf(shape.c_str(), "(%lld, %lld)", &rr, &cc) != 2 || rr < 1 || cc < 1) {
    std::fclose(f);
    bad(filename, "shape " + shape + " (two dimensions are read)");
  }
  const int64_t rows = rr, cols = cc;
  const bool fortran = order.find("True") != std::string::npos;
  auto m = std::make_shared<Matrix>();
  m->n_rows = rows;
  m->n_cols = cols;
  m->data.resize((size_t)(rows * cols));
  const size_t count = (size_t)(rows * cols);
  if (fortran && esize == 8) {  // already column-major float64
    const size_t got = std::fread(m->data.data(), 8, count, f);
    std::fclose(f);
    if (got != count) bad(filename, "truncated data");
    return m;
  }
  std::vector<unsigned char> raw(count * (size_t)esize);
  const size_t got = std::fread(raw.data(), (size_t)esize, count, f);
  std::fclose(f);
  if (got != count) bad(filename, "truncated data");
  auto load = [&](size_t idx) -> double {
    if (esize == 8) {
      double v;
      std::memcpy(&v, raw.data() + idx * 8, 8);
      return v;
    }
    float v;
    std::memcpy(&v, raw.data() + idx * 4, 4);
    return (double)v;
  };
  double *out = m->data.data();
  if (fortran) {
    parallel_rows((int64_t)count, [&](int64_t a, int64_t b) {
      for (int64_t i = a; i < b; ++i) out[i] = load((size_t)i);
    });
    return m;
  }
  // C order (row = observation): transpose in 64 x 64 blocks, column blocks per thread
  constexpr int64_t kB = 64;
  const int64_t cb = (cols + kB - 1) / kB;
  parallel_rows(cb, [&](int64_t a, int64_t b) {
    for (int64_t jb = a; jb < b; ++jb)
      for (int64_t i0 = 0; i0 < rows; i0 += kB)
        for (int64_t j = jb * kB; j < std::min(cols, (jb + 1) * kB); ++j)
          for (int64_t i = i0; i < std::min(rows, i0 + kB); ++i) out[j * rows + i] = load((size_t)(i * cols + j));
  });
  return m;
}
