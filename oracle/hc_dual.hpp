// hc_dual.hpp -- forward-mode dual numbers for the oracle.
//
// TEST INFRASTRUCTURE ONLY.  Dual{v, d} carries a value and its derivative
// along one input direction; instantiating the oracle's templates with it
// (Solver<Dual>) differentiates the same code that pins the forward parity,
// exactly (no truncation error), branch by branch: comparisons look at values
// only, so every limiter / upwind / entropy-fix switch takes the branch the
// FP64 run takes and the derivative is that branch's.  The timestep is held at
// its value (hco::freeze), as the frozen-timestep discrete adjoint assumes.
#pragma once

#include <cmath>
#include <limits>

namespace hco {

struct Dual {
  double v = 0, d = 0;
  constexpr Dual() = default;
  constexpr Dual(double x) : v(x), d(0) {}
  constexpr Dual(double x, double dx) : v(x), d(dx) {}

  friend constexpr Dual operator+(const Dual& a, const Dual& b) { return {a.v + b.v, a.d + b.d}; }
  friend constexpr Dual operator-(const Dual& a, const Dual& b) { return {a.v - b.v, a.d - b.d}; }
  friend constexpr Dual operator-(const Dual& a) { return {-a.v, -a.d}; }
  friend constexpr Dual operator*(const Dual& a, const Dual& b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
  friend constexpr Dual operator/(const Dual& a, const Dual& b) {
    const double q = a.v / b.v;
    return {q, (a.d - q * b.d) / b.v};
  }
  Dual& operator+=(const Dual& b) { return *this = *this + b; }
  Dual& operator-=(const Dual& b) { return *this = *this - b; }
  Dual& operator*=(const Dual& b) { return *this = *this * b; }
  Dual& operator/=(const Dual& b) { return *this = *this / b; }

  friend constexpr bool operator<(const Dual& a, const Dual& b) { return a.v < b.v; }
  friend constexpr bool operator>(const Dual& a, const Dual& b) { return a.v > b.v; }
  friend constexpr bool operator<=(const Dual& a, const Dual& b) { return a.v <= b.v; }
  friend constexpr bool operator>=(const Dual& a, const Dual& b) { return a.v >= b.v; }
  friend constexpr bool operator==(const Dual& a, const Dual& b) { return a.v == b.v; }
  friend constexpr bool operator!=(const Dual& a, const Dual& b) { return a.v != b.v; }
};

// derivative of |x| taken as sign(x), 0 at 0 (the branch x >= 0 of the kink)
inline Dual fabs(const Dual& x) { return x.v < 0 ? -x : (x.v > 0 ? x : Dual(0.0, 0.0)); }
inline Dual abs(const Dual& x) { return fabs(x); }
inline Dual sqrt(const Dual& x) {
  const double s = std::sqrt(x.v);
  return {s, s > 0 ? 0.5 * x.d / s : 0.0};
}
inline Dual fmax(const Dual& a, const Dual& b) { return (a.v < b.v) ? b : a; }
inline Dual fmin(const Dual& a, const Dual& b) { return (b.v < a.v) ? b : a; }
inline Dual fmax(const Dual& a, double b) { return fmax(a, Dual(b)); }
inline Dual fmax(double a, const Dual& b) { return fmax(Dual(a), b); }
inline Dual fmin(const Dual& a, double b) { return fmin(a, Dual(b)); }
inline Dual fmin(double a, const Dual& b) { return fmin(Dual(a), b); }
inline Dual pow(const Dual& a, const Dual& b) {
  const double p = std::pow(a.v, b.v);
  const double da = (a.v != 0) ? b.v * std::pow(a.v, b.v - 1) * a.d : 0.0;
  const double db = (a.v > 0) ? p * std::log(a.v) * b.d : 0.0;
  return {p, da + db};
}
inline Dual pow(const Dual& a, double b) { return pow(a, Dual(b)); }
inline Dual pow(double a, const Dual& b) { return pow(Dual(a), b); }

// the timestep's derivative is dropped unless a caller asks to keep it (to
// compare with central differences of the plain oracle, whose timestep moves)
inline thread_local bool g_freeze_dt = true;
inline Dual freeze(const Dual& x) { return g_freeze_dt ? Dual(x.v, 0.0) : x; }

}  // namespace hco

template <> struct std::numeric_limits<hco::Dual> {
  static constexpr bool is_specialized = true;
  static constexpr hco::Dual min() noexcept { return hco::Dual(std::numeric_limits<double>::min()); }
  static constexpr hco::Dual max() noexcept { return hco::Dual(std::numeric_limits<double>::max()); }
  static constexpr hco::Dual lowest() noexcept { return hco::Dual(std::numeric_limits<double>::lowest()); }
  static constexpr hco::Dual epsilon() noexcept { return hco::Dual(std::numeric_limits<double>::epsilon()); }
};
