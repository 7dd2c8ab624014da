// oracle_1d.cpp -- extern "C" surface of the one-dimensional Euler oracle.
//
// TEST INFRASTRUCTURE ONLY: the product library never links this.
#include "hc_oracle_1d.hpp"
#include "hc_oracle_smooth.hpp"

using namespace hco;
using S1 = Solver1D<double>;

extern "C" {

// nodes: nc + 1 coordinates; bc[2] (BC_*); ref: 2 x 3 primitive reference values
// {u, rho, p} (left, right); species = {gamma, R, minf}
void* hco1_create(int nc, const double* nodes, const int* bc, int flux, int lim, int rk, int dtmode, double cfl,
                  const double* species, const double* ref) {
  S1* s = new S1();
  s->nc = nc;
  s->x.assign(nodes, nodes + nc + 1);
  s->bc[0] = bc[0]; s->bc[1] = bc[1];
  s->flux = flux; s->lim = lim; s->rk = rk; s->dtmode = dtmode; s->cfl = cfl;
  s->sp = air_species<double>();
  s->sp.gamma = species[0]; s->sp.Rgas = species[1]; s->sp.minf = species[2];
  s->sp.gamma1 = 1. / (s->sp.gamma - 1.);
  for (int side = 0; side < 2; ++side)
    for (int v = 0; v < 3; ++v) s->ref[side][v] = ref ? ref[3 * side + v] : 0.0;
  s->setup();
  return s;
}
void hco1_destroy(void* h) { delete static_cast<S1*>(h); }
// state as 3 planes of nc primitive values {u, rho, p}
void hco1_set_state(void* h, const double* soa) {
  S1* s = static_cast<S1*>(h);
  for (int c = 0; c < s->nc; ++c)
    for (int v = 0; v < 3; ++v) s->q0[3 * c + v] = soa[v * s->nc + c];
}
void hco1_get_state(void* h, double* soa) {
  S1* s = static_cast<S1*>(h);
  for (int c = 0; c < s->nc; ++c)
    for (int v = 0; v < 3; ++v) soa[v * s->nc + c] = s->q0[3 * c + v];
}
// one residual evaluation: 4 planes (rho u, rho, rho E flux sums; lambda sum)
void hco1_residual(void* h, double* out) {
  S1* s = static_cast<S1*>(h);
  s->residual(s->q0, s->res[0]);
  for (int c = 0; c < s->nc; ++c)
    for (int v = 0; v < 4; ++v) out[v * s->nc + c] = s->res[0][c][v];
}
void hco1_step(void* h, int n, double* out_dt_t) {
  S1* s = static_cast<S1*>(h);
  s->step(n);
  out_dt_t[0] = s->last_dt;
  out_dt_t[1] = s->t;
}

// residual smoothing of the legacy 1D path (hc_oracle_smooth.hpp): nplanes planes of n
// values each; kind 0 implicit, 1 explicit; bc the reference's end character
void hco_smooth_1d(int kind, const double* r0, double* r1, long long n, int nplanes, double alpha, int bc) {
  for (int p = 0; p < nplanes; ++p) {
    const double* a = r0 + size_t(p) * n;
    double* b = r1 + size_t(p) * n;
    if (kind == 0) smooth_implicit_1d(a, b, size_t(n), alpha, char(bc));
    else smooth_explicit_1d(a, b, size_t(n), alpha, char(bc));
  }
}

}  // extern "C"
