// CSV reader of the heterogpc CLI (replaces CSVParser::read_csv_to_mat,
// src/util/csv_parser.cpp:20-77): comma-separated numbers, one observation per line,
// an optional header line (detected as in the reference: the first field does not
// parse as a number). The result is column-major (each variable contiguous), the
// layout of the reference's arma::mat and of the C ABI's observation input.
// The file is parsed in parallel by line ranges.
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <limits>
#include <thread>

#include "heterogpc.hpp"

namespace {

bool parse_number(const char *&s, const char *end, double &v) {
  while (s < end && (*s == ' ' || *s == '\t')) ++s;
  if (s >= end) return false;
  char *e = nullptr;
  v = std::strtod(s, &e);
  if (e == s) return false;
  s = e;
  return true;
}

}  // namespace

std::shared_ptr<Matrix> CSVParser::read_csv_to_mat(const std::string &filename, std::vector<std::string> &column_names) {
  FILE *f = std::fopen(filename.c_str(), "rb");
  if (!f) {
    std::cout << "Could not find file '" << filename << '\'' << std::endl;
    std::exit(1);  // src/util/csv_parser.cpp:22-25
  }
  std::string buf;
  std::fseek(f, 0, SEEK_END);
  long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  buf.resize(sz > 0 ? (size_t)sz : 0);
  if (sz > 0 && std::fread(&buf[0], 1, (size_t)sz, f) != (size_t)sz) buf.clear();
  std::fclose(f);
  const char *b = buf.data(), *end = b + buf.size();
  // header: first field is not a number
  {
    const char *s = b;
    double v;
    if (!parse_number(s, end, v)) {
      const char *nl = b;
      while (nl < end && *nl != '\n' && *nl != '\r') ++nl;
      std::string line(b, nl);
      size_t pos = 0;
      while (true) {
        size_t c = line.find(',', pos);
        column_names.push_back(line.substr(pos, c == std::string::npos ? std::string::npos : c - pos));
        if (c == std::string::npos) break;
        pos = c + 1;
      }
      b = nl;
    }
  }
  // line starts
  std::vector<const char *> lines;
  for (const char *s = b; s < end;) {
    while (s < end && (*s == '\n' || *s == '\r')) ++s;
    if (s >= end) break;
    lines.push_back(s);
    while (s < end && *s != '\n' && *s != '\r') ++s;
  }
  auto m = std::make_shared<Matrix>();
  if (lines.empty()) return m;
  // columns from the first line
  int64_t cols = 1;
  for (const char *s = lines[0]; s < end && *s != '\n' && *s != '\r'; ++s)
    if (*s == ',') ++cols;
  const int64_t rows = (int64_t)lines.size();
  m->n_rows = rows;
  m->n_cols = cols;
  m->data.assign((size_t)(rows * cols), 0.0);
  unsigned nth = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  std::vector<std::thread> pool;
  std::vector<int> bad(nth, 0);
  for (unsigned t = 0; t < nth; ++t) {
    pool.emplace_back([&, t]() {
      for (int64_t r = t; r < rows; r += nth) {
        const char *s = lines[r];
        const char *le = s;
        while (le < end && *le != '\n' && *le != '\r') ++le;
        for (int64_t c = 0; c < cols; ++c) {
          double v = std::numeric_limits<double>::quiet_NaN();
          const char *fs = s;
          if (!parse_number(s, le, v)) {
            // empty or non-numeric field: missing value
            v = std::numeric_limits<double>::quiet_NaN();
            s = fs;
            if (c + 1 < cols) bad[t] = 1;
          }
          m->data[(size_t)(c * rows + r)] = v;
          while (s < le && *s != ',') ++s;
          if (s < le) ++s;
        }
      }
    });
  }
  for (auto &th : pool) th.join();
  return m;
}
