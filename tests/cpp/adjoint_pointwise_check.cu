// Host-side check of the reverse pointwise functions in hc_adjoint.cuh against
// central differences of the forward functions in hc_physics.cuh (FP64):
// limiter derivatives (away from their kinks) and the Roe and Rusanov face
// flux adjoints (x_bar = (dF/dx)^T F_bar for both face states).
#include "../../hyperboliconvergence_gb300/csrc/hc_adjoint.cuh"

#include <cmath>
#include <cstdio>
#include <random>

using namespace hc;

namespace {

double limit_fd(int kind, double a, double b, int wrt) {
  const double h = 1e-7 * std::fmax(std::fabs(a), std::fabs(b));
  if (wrt == 0) return (limit<double>(kind, a + h, b) - limit<double>(kind, a - h, b)) / (2 * h);
  return (limit<double>(kind, a, b + h) - limit<double>(kind, a, b - h)) / (2 * h);
}

template <int FK> Flux5<double> flux(const Gas<double>& g, double nx, double ny, double A, const double* ql,
                                     const double* qr) {
  const St<double> l = prim_state(g, ql[0], ql[1], ql[2], ql[3]);
  const St<double> r = prim_state(g, qr[0], qr[1], qr[2], qr[3]);
  if constexpr (FK == FLUX_ROE) return roe_flux(g, nx, ny, A, l, r);
  else return rusanov_flux(nx, ny, A, l, r);
}

template <int FK> double flux_check(std::mt19937_64& rng) {
  std::uniform_real_distribution<double> U(-1.0, 1.0), P(0.5, 2.0);
  const Gas<double> g = make_gas<double>(1.4, 287.058, 0.3);
  double worst = 0;
  for (int t = 0; t < 2000; ++t) {
    const double th = 3.14159265358979 * U(rng);
    const double nx = std::cos(th), ny = std::sin(th), A = P(rng);
    double ql[4] = {U(rng), U(rng), P(rng), P(rng)}, qr[4] = {U(rng), U(rng), P(rng), P(rng)};
    double Fb[4] = {U(rng), U(rng), U(rng), U(rng)};
    double qlb[4] = {0, 0, 0, 0}, qrb[4] = {0, 0, 0, 0};
    if constexpr (FK == FLUX_ROE) roe_flux_adj(g, nx, ny, A, ql, qr, Fb, qlb, qrb);
    else rusanov_flux_adj(g, nx, ny, A, ql, qr, Fb, qlb, qrb);
    double scale = 0;
    for (int v = 0; v < 4; ++v) scale = std::fmax(scale, std::fmax(std::fabs(qlb[v]), std::fabs(qrb[v])));
    for (int side = 0; side < 2; ++side)
      for (int v = 0; v < 4; ++v) {
        double* q = side ? qr : ql;
        const double x = q[v], h = 1e-6 * std::fmax(1.0, std::fabs(x));
        q[v] = x + h;
        const Flux5<double> fp = flux<FK>(g, nx, ny, A, ql, qr);
        q[v] = x - h;
        const Flux5<double> fm = flux<FK>(g, nx, ny, A, ql, qr);
        q[v] = x;
        double fd = 0;
        for (int k = 0; k < 4; ++k) fd += Fb[k] * (fp.f[k] - fm.f[k]) / (2 * h);
        const double ad = side ? qrb[v] : qlb[v];
        worst = std::fmax(worst, std::fabs(fd - ad) / std::fmax(scale, 1e-12));
      }
  }
  return worst;
}

}  // namespace

int main() {
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  const int kinds[] = {LIM_NOLIMIT2, LIM_NOLIMIT3, LIM_VANALBADA, LIM_MINMOD, LIM_VANLEER};
  const char* names[] = {"nolimit2", "nolimit3", "vanalbada", "minmod", "vanleer"};
  int fails = 0;
  for (int k = 0; k < 5; ++k) {
    double worst = 0;
    for (int t = 0; t < 20000; ++t) {
      const double a = U(rng), b = U(rng);
      // stay away from the kinks: a = 0, b = 0, a = b
      if (std::fabs(a) < 1e-3 || std::fabs(b) < 1e-3 || std::fabs(a - b) < 1e-3) continue;
      double da, db;
      limit_grad<double>(kinds[k], a, b, &da, &db);
      const double fa = limit_fd(kinds[k], a, b, 0), fb = limit_fd(kinds[k], a, b, 1);
      worst = std::fmax(worst, std::fmax(std::fabs(da - fa), std::fabs(db - fb)));
    }
    std::printf("limiter %-9s max |d_ad - d_fd| %.3e\n", names[k], worst);
    if (!(worst < 1e-6)) ++fails;
  }
  const double roe = flux_check<FLUX_ROE>(rng), rus = flux_check<FLUX_RUSANOV>(rng);
  std::printf("roe flux adjoint %.3e, rusanov flux adjoint %.3e (relative to the largest adjoint)\n", roe, rus);
  if (!(roe < 1e-6)) ++fails;
  if (!(rus < 1e-6)) ++fails;
  return fails;
}
