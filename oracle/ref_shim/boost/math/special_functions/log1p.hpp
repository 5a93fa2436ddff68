// ORACLE -- test infrastructure only. Stand-in for boost::math::log1p.
#pragma once
#include <cmath>
namespace boost {
namespace math {
inline double log1p(double x) { return std::log1p(x); }
}  // namespace math
}  // namespace boost
