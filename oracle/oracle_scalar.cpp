// oracle_scalar.cpp -- extern "C" surface of the scalar-advection oracle
// (hc_oracle_scalar.hpp): solver and pointwise functions.
//
// TEST INFRASTRUCTURE ONLY: the product library never links this.
#include "hc_dual.hpp"
#include "hc_oracle_scalar.hpp"

using namespace hco;
using SS = ScalarSolver<double>;

static Face<double> face7(const double* f) {
  Face<double> o;
  o.area = f[0]; o.c[0] = f[1]; o.c[1] = f[2]; o.n[0] = f[3]; o.n[1] = f[4]; o.t[0] = f[5]; o.t[1] = f[6];
  return o;
}

namespace {

// L2 objective of an RK run of the scalar oracle (global timestep):
// J = sum_cells sum_v weight[v] (q_N - target)_v^2 on {u, v, q}.  R = Dual: J and its
// derivative along (dq0, dref), timesteps frozen unless g_freeze_dt is false.
template <class R>
void run_scalar_objective(int ni, int nj, const double* nodes, const int* bc, int flux, int lim, int rk, double cfl,
                          const double* const* ref, const double* const* dref, const double* q0, const double* dq0,
                          int nsteps, const double* target, const double* weight, double* out) {
  ScalarSolver<R> s;
  s.geo.ni = ni; s.geo.nj = nj;
  s.geo.nodes.assign(nodes, nodes + size_t(ni + 1) * (nj + 1) * 2);
  for (int k = 0; k < 4; ++k) s.bc[k] = bc[k];
  s.flux = flux; s.lim = lim; s.rk = rk; s.dtmode = DT_GLOBAL; s.cfl = cfl;
  s.setup();
  auto val = [](const double* a, const double* da, size_t k) -> R {
    if constexpr (std::is_same_v<R, double>) return a[k];
    else return R(a[k], da ? da[k] : 0.0);
  };
  for (int side = 0; side < 4; ++side) {
    if (!ref || !ref[side]) continue;
    const size_t nf = s.geo.nface(side);
    const double* d = (dref && dref[side]) ? dref[side] : nullptr;
    for (size_t k = 0; k < nf; ++k)
      for (int v = 0; v < 3; ++v) s.ghost[side][k * 6 + 3 + v] = val(ref[side], d, v * nf + k);
  }
  const size_t n = size_t(ni) * nj;
  for (size_t c = 0; c < n; ++c)
    for (int v = 0; v < 3; ++v) s.q0[c * 3 + v] = val(q0, dq0, v * n + c);
  s.step(nsteps);
  R J = 0.0;
  for (size_t c = 0; c < n; ++c)
    for (int v = 0; v < 3; ++v) {
      const R d = s.q0[c * 3 + v] - target[v * n + c];
      J = J + weight[v] * d * d;
    }
  if constexpr (std::is_same_v<R, double>) { out[0] = J; out[1] = 0.0; }
  else { out[0] = J.v; out[1] = J.d; }
}

}  // namespace

extern "C" {

// J of the scalar L2 objective (bc SBC_*, flux SFLUX_*; states and reference layers
// 3 planes); with dq0 / dref non-null also its exact derivative along them
// (freeze_dt != 0: timesteps held at their values).  out = {J, dJ}.
void hcos_objective(int ni, int nj, const double* nodes, const int* bc, int flux, int lim, int rk, double cfl,
                    const double* const* ref, const double* const* dref, const double* q0, const double* dq0,
                    int nsteps, const double* target, const double* weight, int freeze_dt, double* out) {
  if (!dq0 && !dref) {
    run_scalar_objective<double>(ni, nj, nodes, bc, flux, lim, rk, cfl, ref, nullptr, q0, nullptr, nsteps, target,
                                 weight, out);
    return;
  }
  g_freeze_dt = freeze_dt != 0;
  run_scalar_objective<Dual>(ni, nj, nodes, bc, flux, lim, rk, cfl, ref, dref, q0, dq0, nsteps, target, weight,
                             out);
}


// bc: SBC_* per side; flux: SFLUX_*; states are 3 planes {u, v, q} of ni*nj values
void* hcos_create(int ni, int nj, const double* nodes, const int* bc, int flux, int lim, int rk, int dtmode,
                  double cfl) {
  SS* s = new SS();
  s->geo.ni = ni; s->geo.nj = nj;
  s->geo.nodes.assign(nodes, nodes + size_t(ni + 1) * (nj + 1) * 2);
  for (int k = 0; k < 4; ++k) s->bc[k] = bc[k];
  s->flux = flux; s->lim = lim; s->rk = rk; s->dtmode = dtmode; s->cfl = cfl;
  s->setup();
  return s;
}
void hcos_destroy(void* h) { delete static_cast<SS*>(h); }
void hcos_set_ghost_ref(void* h, int side, const double* planes) {
  SS* s = static_cast<SS*>(h);
  const size_t nf = s->geo.nface(side);
  for (size_t k = 0; k < nf; ++k)
    for (int v = 0; v < 3; ++v) s->ghost[side][k * 6 + 3 + v] = planes[v * nf + k];
}
void hcos_set_state(void* h, const double* soa) {
  SS* s = static_cast<SS*>(h);
  const size_t n = size_t(s->ni()) * s->nj();
  for (size_t c = 0; c < n; ++c)
    for (int v = 0; v < 3; ++v) s->q0[c * 3 + v] = soa[v * n + c];
}
void hcos_get_state(void* h, double* soa) {
  SS* s = static_cast<SS*>(h);
  const size_t n = size_t(s->ni()) * s->nj();
  for (size_t c = 0; c < n; ++c)
    for (int v = 0; v < 3; ++v) soa[v * n + c] = s->q0[c * 3 + v];
}
// 4 planes: 3 flux sums and the spectral-radius sum
void hcos_residual(void* h, double* out) {
  SS* s = static_cast<SS*>(h);
  const size_t n = size_t(s->ni()) * s->nj();
  s->residual(s->q0, s->res[0]);
  for (size_t c = 0; c < n; ++c) {
    for (int v = 0; v < 3; ++v) out[v * n + c] = s->res[0][c].f[v];
    out[3 * n + c] = s->res[0][c].lam;
  }
}
void hcos_step(void* h, int nsteps, double* out_dt_t) {
  SS* s = static_cast<SS*>(h);
  s->step(nsteps);
  out_dt_t[0] = s->last_dt;
  out_dt_t[1] = s->t;
}

// pointwise: flux of kind SFLUX_* (out: 3 fluxes + lambda); Riemann ghost value
void hcos_flux(int kind, const double* face, const double* ql, const double* qr, double* out4) {
  const SFlux<double> r = scalar_flux(kind, face7(face), ql, qr);
  for (int v = 0; v < 3; ++v) out4[v] = r.f[v];
  out4[3] = r.lam;
}
void hcos_bc_riemann(const double* face, const double* qi, const double* qb, double* out3) {
  scalar_bc_riemann(face7(face), qi, qb, out3);
}

}  // extern "C"
