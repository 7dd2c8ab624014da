// oracle_dual.cpp -- objectives of an RK run of the CPU oracle and their exact
// directional derivatives (the oracle instantiated with forward-mode Dual).
//
// TEST INFRASTRUCTURE ONLY: the reference gradient the discrete adjoint of the
// product is checked against.  Objectives follow the product's definitions:
//   drag: J = scale/N * sum_{n=1..N} F(q_n),  F = -sum_wall A p_w (n_in . dir),
//         p_w the interior pressure extrapolated to the face with the cell's
//         full LSQ gradient (the wall flux of inviscidWall.ipp:33-72);
//   l2:   J = sum_cells sum_v w_v (q_N - target)_v^2 on primitive variables.
// Timesteps are frozen at their values (hco::freeze) unless asked otherwise.
#include "hc_dual.hpp"
#include "hc_oracle_solver.hpp"

using namespace hco;

namespace {

template <class R> R wall_force(Solver<R>& s, double dirx, double diry) {
  s.qmetrics(s.q0);
  R F = 0.0;
  for (int side = 0; side < 4; ++side) {
    if (s.bc[side] != BC_WALL) continue;
    for (int k = 0; k < s.nface(side); ++k) {
      const size_t c = s.side_cell(side, k);
      const Face<R> f = s.bface_in(side, k);
      const R dir[2] = {s.cells[c].c[0] - f.c[0], s.cells[c].c[1] - f.c[1]};
      R dq[4];
      solve(factor(s.xm[c]), s.qm[c], dir, dq);
      const FluxRes<R> w = wall_flux(s.sp, f, &s.q0[c * 4], dq);
      F = F - (w.f[0] * dirx + w.f[1] * diry);
    }
  }
  return F;
}

// R = double: plain objective; R = Dual: objective and its derivative along
// (dq0, dref).  Returns J (value, derivative).
template <class R>
void run_objective(int ni, int nj, const double* nodes, const int* bc, int flux, int lim, int rk, double cfl,
                   const double* species, const double* const* ref, const double* const* dref, const double* q0,
                   const double* dq0, int nsteps, int kind, double scale, double dirx, double diry,
                   const double* target, const double* weight, double* out) {
  Solver<R> s;
  s.ni = ni; s.nj = nj;
  s.nodes.assign(nodes, nodes + size_t(ni + 1) * (nj + 1) * 2);
  for (int k = 0; k < 4; ++k) s.bc[k] = bc[k];
  s.flux = flux; s.lim = lim; s.rk = rk; s.dtmode = DT_GLOBAL; s.cfl = cfl;
  s.sp = air_species<R>();
  s.sp.gamma = species[0]; s.sp.Rgas = species[1]; s.sp.minf = species[2];
  s.sp.gamma1 = R(1.) / (s.sp.gamma - R(1.));
  s.setup();
  const size_t n = size_t(ni) * nj;
  auto val = [](const double* a, const double* da, size_t k) -> R {
    if constexpr (std::is_same_v<R, double>) return a[k];
    else return R(a[k], da ? da[k] : 0.0);
  };
  for (int side = 0; side < 4; ++side) {
    if (!ref || !ref[side]) continue;
    const size_t nf = s.nface(side);
    for (size_t k = 0; k < nf; ++k)
      for (int v = 0; v < 4; ++v)
        s.ghost[side][k * 8 + 4 + v] = val(ref[side], dref ? dref[side] : nullptr, v * nf + k);
  }
  for (size_t c = 0; c < n; ++c)
    for (int v = 0; v < 4; ++v) s.q0[c * 4 + v] = val(q0, dq0, v * n + c);
  R J = 0.0;
  for (int st = 0; st < nsteps; ++st) {
    s.step(1);
    if (kind == 0) J = J + wall_force(s, dirx, diry) * (scale / nsteps);
  }
  if (kind == 1)
    for (size_t c = 0; c < n; ++c)
      for (int v = 0; v < 4; ++v) {
        const R d = s.q0[c * 4 + v] - target[v * n + c];
        J = J + weight[v] * d * d;
      }
  if constexpr (std::is_same_v<R, double>) { out[0] = J; out[1] = 0.0; }
  else { out[0] = J.v; out[1] = J.d; }
}

}  // namespace

extern "C" {

// J of an RK run (global timestep) from q0 (4 planes), reference layers ref[side]
// (4 planes of nface values, NULL when unused).  out[0] = J.
void hco_objective(int ni, int nj, const double* nodes, const int* bc, int flux, int lim, int rk, double cfl,
                   const double* species, const double* const* ref, const double* q0, int nsteps, int kind,
                   double scale, double dirx, double diry, const double* target, const double* weight,
                   double* out) {
  run_objective<double>(ni, nj, nodes, bc, flux, lim, rk, cfl, species, ref, nullptr, q0, nullptr, nsteps, kind,
                        scale, dirx, diry, target, weight, out);
}

// Same plus the exact derivative of J along the direction (dq0, dref) (dref may
// be NULL, or hold NULL sides), with the timesteps frozen (freeze_dt != 0, the
// adjoint's derivative) or moving with the state.  out = {J, dJ}.
void hco_objective_jvp(int ni, int nj, const double* nodes, const int* bc, int flux, int lim, int rk, double cfl,
                       const double* species, const double* const* ref, const double* const* dref,
                       const double* q0, const double* dq0, int nsteps, int kind, double scale, double dirx,
                       double diry, const double* target, const double* weight, int freeze_dt, double* out) {
  g_freeze_dt = freeze_dt != 0;
  run_objective<Dual>(ni, nj, nodes, bc, flux, lim, rk, cfl, species, ref, dref, q0, dq0, nsteps, kind, scale,
                      dirx, diry, target, weight, out);
}

}  // extern "C"
