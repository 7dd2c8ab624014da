// Host-side check of the double-float arithmetic in hc_df64.cuh against
// double: relative errors of +, -, *, /, sqrt on random operands, including
// near-cancelling differences (error then measured against the operands).
#include "../../hyperboliconvergence_gb300/csrc/hc_df64.cuh"

#include <cstdio>
#include <random>

using hc::df64;

int main() {
  std::mt19937_64 g(42);
  std::uniform_real_distribution<double> u(-1.0, 1.0), e(-8.0, 8.0);
  double worst[5] = {0, 0, 0, 0, 0};
  for (int k = 0; k < 200000; ++k) {
    const double a = u(g) * std::pow(10.0, e(g)), b = u(g) * std::pow(10.0, e(g));
    const double c = (k % 7 == 0) ? a * (1 + 1e-9 * u(g)) : b;  // near-cancellation cases
    const df64 A(a), B(b), Cc(c);
    const double scale_add = std::fabs(a) + std::fabs(c);
    const double r[5] = {
        std::fabs((A + Cc).to_double() - (a + c)) / scale_add,
        std::fabs((A - Cc).to_double() - (a - c)) / scale_add,
        std::fabs((A * B).to_double() - a * b) / std::fabs(a * b),
        std::fabs((A / B).to_double() - a / b) / std::fabs(a / b),
        std::fabs(sqrt(fabs(A)).to_double() - std::sqrt(std::fabs(a))) / std::sqrt(std::fabs(a))};
    for (int i = 0; i < 5; ++i) worst[i] = std::fmax(worst[i], r[i]);
  }
  std::printf("add %.3e sub %.3e mul %.3e div %.3e sqrt %.3e\n", worst[0], worst[1], worst[2], worst[3], worst[4]);
  // 2^-45 ~ 2.8e-14 bounds every operation
  for (double w : worst)
    if (!(w < 2.9e-14)) return 1;
  return 0;
}
