// oracle_scalar.cpp -- extern "C" surface of the scalar-advection oracle
// (hc_oracle_scalar.hpp): solver and pointwise functions.
//
// TEST INFRASTRUCTURE ONLY: the product library never links this.
#include "hc_oracle_scalar.hpp"

using namespace hco;
using SS = ScalarSolver<double>;

static Face<double> face7(const double* f) {
  Face<double> o;
  o.area = f[0]; o.c[0] = f[1]; o.c[1] = f[2]; o.n[0] = f[3]; o.n[1] = f[4]; o.t[0] = f[5]; o.t[1] = f[6];
  return o;
}

extern "C" {

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
