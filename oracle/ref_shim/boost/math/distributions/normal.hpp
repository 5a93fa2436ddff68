// ORACLE -- test infrastructure only.
// Stand-in for Boost.Math's standard normal distribution as used by
// src/executor/independence/cpuInd.cpp:11-13: cdf(complement(normal(), z)) is the
// upper tail, erfc(z / sqrt(2)) / 2 by its published definition.
#pragma once
#include <cmath>
namespace boost {
namespace math {
struct normal {};
template <class Dist>
struct complemented_dist {
  Dist d;
  double x;
};
template <class Dist>
inline complemented_dist<Dist> complement(const Dist &d, double x) {
  return complemented_dist<Dist>{d, x};
}
inline double cdf(const complemented_dist<normal> &c) {
  return std::erfc(c.x / 1.41421356237309504880) / 2.0;
}
template <class T>
inline bool isnan(T v) { return std::isnan(v); }
}  // namespace math
}  // namespace boost
