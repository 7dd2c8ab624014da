// oracle_count.cpp -- algorithmic floating-point operation tally of the residual
// path: the oracle instantiated with the counting type of hc_count.hpp.
//
// TEST INFRASTRUCTURE ONLY (read by the measurement to state FLOPs per cell and
// stage beside the FP64 roof).  The tally runs one RK step of the Euler oracle on
// a periodic 16 x 16 mesh (every face interior) with a smooth non-uniform state,
// so each limiter and flux takes its common branches.
#include "hc_count.hpp"
#include "hc_oracle_solver.hpp"

#include <cmath>

using namespace hco;

extern "C" {

// out[0] operations per cell per RK stage (faces, gradients, update, timestep),
// out[1..5] its adds, muls, divs, sqrts, pows; out[6] operations of one interior
// face (reconstruction, limiter, flux); out[7] of one cell's qmetric.
void hco_flop_tally(int flux, int lim, int rk, double* out) {
  // the counter is per thread: tally on one thread
  const int threads = omp_get_max_threads();
  omp_set_num_threads(1);
  const int n = 16;
  Solver<Counted> s;
  s.ni = n; s.nj = n;
  s.nodes.resize(size_t(n + 1) * (n + 1) * 2);
  for (int i = 0; i <= n; ++i)
    for (int j = 0; j <= n; ++j) {
      s.nodes[(size_t(i) * (n + 1) + j) * 2 + 0] = double(i) / n;
      s.nodes[(size_t(i) * (n + 1) + j) * 2 + 1] = double(j) / n;
    }
  for (int k = 0; k < 4; ++k) s.bc[k] = BC_PERIODIC;
  s.flux = flux; s.lim = lim; s.rk = rk; s.dtmode = DT_GLOBAL; s.cfl = 0.5;
  s.sp = air_species<Counted>();
  s.sp.minf = 0.3;
  s.setup();
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      const double x = (i + 0.5) / n, y = (j + 0.5) / n;
      Counted* q = &s.q0[(size_t(i) * n + j) * 4];
      q[0] = 0.4 + 0.05 * std::sin(2 * pi * x) * std::cos(2 * pi * y);
      q[1] = 0.1 + 0.05 * std::cos(2 * pi * x + 0.3);
      q[2] = 1.0 + 0.1 * std::sin(2 * pi * (x + y));
      q[3] = 0.714 + 0.05 * std::cos(2 * pi * (x - 2 * y));
    }
  const RKTable<double> tab = rk_table<double>(rk);
  g_ops = OpCount{};
  s.step(1);
  const OpCount step = g_ops;
  const double per = double(n) * n * tab.nstages;
  out[0] = step.total() / per;
  out[1] = step.add / per; out[2] = step.mul / per; out[3] = step.div / per;
  out[4] = step.sqrt / per; out[5] = step.pow / per;
  // one interior i-face between cells (3,5) and (4,5), state of the stepped solver
  s.qmetrics(s.q0);
  const size_t a = s.cid(3, 5), b = s.cid(4, 5);
  g_ops = OpCount{};
  s.muscl(surface(s.node(4, 5), s.node(4, 6)), s.cells[a].c, s.cells[b].c, &s.q0[a * 4], &s.q0[b * 4], s.xm[a],
          s.xm[b], s.qm[a], s.qm[b]);
  out[6] = double(g_ops.total());
  g_ops = OpCount{};
  s.qmetrics(s.q0);
  out[7] = double(g_ops.total()) / (double(n) * n);
  omp_set_num_threads(threads);
}

}  // extern "C"
