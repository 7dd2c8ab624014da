// hc_count.hpp -- an arithmetic type that counts floating-point operations.
//
// TEST INFRASTRUCTURE ONLY.  Instantiating the oracle's templates with Counted
// tallies the operations of the reference's algorithm as the oracle states it:
// each +, -, *, / is one operation, each sqrt one, fabs / fmin / fmax /
// comparisons none (they are selects, not arithmetic); pow counts one.  The
// tally gives the algorithmic FLOPs of a face (or cell) of the residual path
// that the FP64-roof comparison of the measurement uses.
#pragma once

#include <cmath>
#include <limits>

namespace hco {

struct OpCount {
  long long add = 0, mul = 0, div = 0, sqrt = 0, pow = 0;
  long long total() const { return add + mul + div + sqrt + pow; }
};
inline thread_local OpCount g_ops;

struct Counted {
  double v = 0;
  constexpr Counted() = default;
  constexpr Counted(double x) : v(x) {}

  friend Counted operator+(const Counted& a, const Counted& b) { ++g_ops.add; return Counted(a.v + b.v); }
  friend Counted operator-(const Counted& a, const Counted& b) { ++g_ops.add; return Counted(a.v - b.v); }
  friend Counted operator-(const Counted& a) { return Counted(-a.v); }
  friend Counted operator*(const Counted& a, const Counted& b) { ++g_ops.mul; return Counted(a.v * b.v); }
  friend Counted operator/(const Counted& a, const Counted& b) { ++g_ops.div; return Counted(a.v / b.v); }
  Counted& operator+=(const Counted& b) { return *this = *this + b; }
  Counted& operator-=(const Counted& b) { return *this = *this - b; }
  Counted& operator*=(const Counted& b) { return *this = *this * b; }
  Counted& operator/=(const Counted& b) { return *this = *this / b; }

  friend bool operator<(const Counted& a, const Counted& b) { return a.v < b.v; }
  friend bool operator>(const Counted& a, const Counted& b) { return a.v > b.v; }
  friend bool operator<=(const Counted& a, const Counted& b) { return a.v <= b.v; }
  friend bool operator>=(const Counted& a, const Counted& b) { return a.v >= b.v; }
  friend bool operator==(const Counted& a, const Counted& b) { return a.v == b.v; }
  friend bool operator!=(const Counted& a, const Counted& b) { return a.v != b.v; }
};

inline Counted fabs(const Counted& x) { return Counted(std::fabs(x.v)); }
inline Counted abs(const Counted& x) { return Counted(std::fabs(x.v)); }
inline Counted sqrt(const Counted& x) { ++g_ops.sqrt; return Counted(std::sqrt(x.v)); }
inline Counted fmax(const Counted& a, const Counted& b) { return Counted(std::fmax(a.v, b.v)); }
inline Counted fmin(const Counted& a, const Counted& b) { return Counted(std::fmin(a.v, b.v)); }
inline Counted pow(const Counted& a, const Counted& b) { ++g_ops.pow; return Counted(std::pow(a.v, b.v)); }
inline Counted freeze(const Counted& x) { return x; }

}  // namespace hco

template <> struct std::numeric_limits<hco::Counted> {
  static constexpr bool is_specialized = true;
  static constexpr hco::Counted min() noexcept { return hco::Counted(std::numeric_limits<double>::min()); }
  static constexpr hco::Counted max() noexcept { return hco::Counted(std::numeric_limits<double>::max()); }
  static constexpr hco::Counted lowest() noexcept { return hco::Counted(std::numeric_limits<double>::lowest()); }
  static constexpr hco::Counted epsilon() noexcept { return hco::Counted(std::numeric_limits<double>::epsilon()); }
};
