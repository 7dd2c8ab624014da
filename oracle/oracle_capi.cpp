// oracle_capi.cpp -- extern "C" surface of the CPU oracle, for the tests and
// the CPU-baseline leg of the benchmark (loaded with ctypes).
//
// TEST INFRASTRUCTURE ONLY: the product library never links this.
#include "hc_oracle_solver.hpp"

#include <cstdlib>

using namespace hco;
using S = Solver<double>;

static Species<double> make_species(const double* sp) {
  Species<double> s = air_species<double>();
  s.gamma = sp[0];
  s.Rgas = sp[1];
  s.minf = sp[2];
  s.gamma1 = 1. / (s.gamma - 1.);
  return s;
}
static Face<double> make_face(const double* f) {
  Face<double> o;
  o.area = f[0]; o.c[0] = f[1]; o.c[1] = f[2]; o.n[0] = f[3]; o.n[1] = f[4]; o.t[0] = f[5]; o.t[1] = f[6];
  return o;
}
static void put_flux(const FluxRes<double>& r, double* out) {
  for (int v = 0; v < 4; ++v) out[v] = r.f[v];
  out[4] = r.lam;
}

extern "C" {

// ---------------------------------------------------------------- solver
void* hco_create(int ni, int nj, const double* nodes, const int* bc, int flux, int lim, int rk,
                 int dtmode, double cfl, const double* species) {
  S* s = new S();
  s->ni = ni; s->nj = nj;
  s->nodes.assign(nodes, nodes + size_t(ni + 1) * (nj + 1) * 2);
  for (int k = 0; k < 4; ++k) s->bc[k] = bc[k];
  s->flux = flux; s->lim = lim; s->rk = rk; s->dtmode = dtmode; s->cfl = cfl;
  s->sp = make_species(species);
  s->setup();
  return s;
}
void hco_destroy(void* h) { delete static_cast<S*>(h); }
// FIX_* corrections of the reference's defects (hc_set_corrections)
void hco_set_corrections(void* h, unsigned mask) { static_cast<S*>(h)->sp.fixes = mask; }
// solution basis (BASIS_*) of the state and ghost layers
void hco_set_basis(void* h, int basis) { static_cast<S*>(h)->basis = basis; }
// AUSM+up low-Mach scaling pair (SCALING_*) and the species' lref and dt
void hco_set_low_mach(void* h, int vscale, int pscale, double lref, double dt) {
  S* s = static_cast<S*>(h);
  s->vscale = vscale; s->pscale = pscale;
  s->sp.lref = lref; s->sp.dt = dt;
}

// reference (layer-1) values of side `side`: 4 planes of nface primitive values
void hco_set_ghost_ref(void* h, int side, const double* prim) {
  S* s = static_cast<S*>(h);
  const size_t nf = s->nface(side);
  for (size_t k = 0; k < nf; ++k)
    for (int v = 0; v < 4; ++v) s->ghost[side][k * 8 + 4 + v] = prim[v * nf + k];
}
// ghost (layer-0) values of side `side` after the last boundary update: 4 planes
void hco_get_ghost(void* h, int side, double* prim) {
  S* s = static_cast<S*>(h);
  const size_t nf = s->nface(side);
  for (size_t k = 0; k < nf; ++k)
    for (int v = 0; v < 4; ++v) prim[v * nf + k] = s->ghost[side][k * 8 + v];
}
// state as 4 planes of ni*nj primitive values
void hco_set_state(void* h, const double* soa) {
  S* s = static_cast<S*>(h);
  const size_t n = size_t(s->ni) * s->nj;
  for (size_t c = 0; c < n; ++c)
    for (int v = 0; v < 4; ++v) s->q0[c * 4 + v] = soa[v * n + c];
}
void hco_get_state(void* h, double* soa) {
  S* s = static_cast<S*>(h);
  const size_t n = size_t(s->ni) * s->nj;
  for (size_t c = 0; c < n; ++c)
    for (int v = 0; v < 4; ++v) soa[v * n + c] = s->q0[c * 4 + v];
}
// one residual evaluation on the current state: 5 planes (4 flux sums + lambda sum)
void hco_residual(void* h, double* out) {
  S* s = static_cast<S*>(h);
  const size_t n = size_t(s->ni) * s->nj;
  s->residual(s->q0, s->res[0]);
  for (size_t c = 0; c < n; ++c) {
    for (int v = 0; v < 4; ++v) out[v * n + c] = s->res[0][c].f[v];
    out[4 * n + c] = s->res[0][c].lam;
  }
}
void hco_step(void* h, int nsteps, double* out_dt_t) {
  S* s = static_cast<S*>(h);
  s->step(nsteps);
  out_dt_t[0] = s->last_dt;
  out_dt_t[1] = s->t;
}
// branch signatures of one residual evaluation on the current state: (ni+1)*nj i-faces
// and ni*(nj+1) j-faces (codes of limit_piece / flux_bits); arg_i / arg_j (or null): the
// limiter arguments, 16 per face
void hco_face_signatures(void* h, uint64_t* sig_i, uint64_t* sig_j, double* arg_i, double* arg_j) {
  S* s = static_cast<S*>(h);
  std::fill(sig_i, sig_i + size_t(s->ni + 1) * s->nj, uint64_t(0));
  std::fill(sig_j, sig_j + size_t(s->ni) * (s->nj + 1), uint64_t(0));
  if (arg_i) std::fill(arg_i, arg_i + size_t(s->ni + 1) * s->nj * 16, 0.0);
  if (arg_j) std::fill(arg_j, arg_j + size_t(s->ni) * (s->nj + 1) * 16, 0.0);
  s->sig_i = sig_i;
  s->sig_j = sig_j;
  s->arg_i = arg_i;
  s->arg_j = arg_j;
  s->residual(s->q0, s->res[0]);
  s->sig_i = s->sig_j = nullptr;
  s->arg_i = s->arg_j = nullptr;
  if (arg_i && s->bc[0] == BC_PERIODIC)
    for (int j = 0; j < s->nj; ++j)
      std::copy(arg_i + size_t(j) * 16, arg_i + size_t(j) * 16 + 16, arg_i + (size_t(s->ni) * s->nj + j) * 16);
  if (arg_j && s->bc[2] == BC_PERIODIC)
    for (int i = 0; i < s->ni; ++i)
      std::copy(arg_j + size_t(i) * (s->nj + 1) * 16, arg_j + size_t(i) * (s->nj + 1) * 16 + 16,
                arg_j + (size_t(i) * (s->nj + 1) + s->nj) * 16);
  // the residual evaluates each periodic face pair once, at the lower index; the upper
  // copy (i = ni, j = nj) is the same face
  if (s->bc[0] == BC_PERIODIC)
    for (int j = 0; j < s->nj; ++j) sig_i[size_t(s->ni) * s->nj + j] = sig_i[size_t(j)];
  if (s->bc[2] == BC_PERIODIC)
    for (int i = 0; i < s->ni; ++i) sig_j[size_t(i) * (s->nj + 1) + s->nj] = sig_j[size_t(i) * (s->nj + 1)];
}
// cell volumes and centres: 3 planes
void hco_cells(void* h, double* out) {
  S* s = static_cast<S*>(h);
  const size_t n = size_t(s->ni) * s->nj;
  for (size_t c = 0; c < n; ++c) {
    out[c] = s->cells[c].vol; out[n + c] = s->cells[c].c[0]; out[2 * n + c] = s->cells[c].c[1];
  }
}
// dual-time stepping: outer physical steps of scheme (0 BDF1, 1 BDF2, 2 trapezium) with inner
// pseudo-time RK steps each; returns the physical dt (dt <= 0: from cfl_outer)
double hco_dual_time(void* h, int outer, double dt, double cfl_outer, int scheme, int inner) {
  return static_cast<S*>(h)->dual_time(outer, dt, cfl_outer, scheme, inner);
}
void hco_set_threads(int n) { omp_set_num_threads(n); }
int hco_get_threads(void) { return omp_get_max_threads(); }

// ---------------------------------------------------------------- pointwise
// face = {area, cx, cy, nx, ny, tx, ty}; species = {gamma, R, minf}; q primitive
void hco_flux(int kind, const double* species, const double* face, const double* ql, const double* qr,
              double* out5) {
  const Species<double> sp = make_species(species);
  put_flux(face_flux(kind, sp, make_face(face), prim2state(sp, ql), prim2state(sp, qr)), out5);
}
// AUSM+up with a low-Mach scaling pair (SCALING_*); species = {gamma, R, minf, lref, dt}
void hco_ausmpup_scaled(int vscale, int pscale, const double* species5, const double* face,
                        const double* ql, const double* qr, double* out5) {
  Species<double> sp = make_species(species5);
  sp.lref = species5[3];
  sp.dt = species5[4];
  put_flux(ausmpup_flux(sp, make_face(face), prim2state(sp, ql), prim2state(sp, qr), vscale, pscale), out5);
}
void hco_exact_flux(const double* species, const double* normal, const double* q, double* out5) {
  const Species<double> sp = make_species(species);
  put_flux(exact_flux(normal, prim2state(sp, q)), out5);
}
double hco_limit(int kind, double a, double b) { return limit<double>(kind, a, b); }
void hco_surface(const double* p0, const double* p1, double* out7) {
  const Face<double> f = surface(p0, p1);
  out7[0] = f.area; out7[1] = f.c[0]; out7[2] = f.c[1];
  out7[3] = f.n[0]; out7[4] = f.n[1]; out7[5] = f.t[0]; out7[6] = f.t[1];
}
void hco_volume(const double* p, double* out3) {
  const Cell<double> c = volume(p, p + 2, p + 4, p + 6);
  out3[0] = c.vol; out3[1] = c.c[0]; out3[2] = c.c[1];
}
// state of a primitive set: {p, r, t, h, u2, a2, u, v}
void hco_prim2state(const double* species, const double* q, double* out8) {
  const State<double> s = prim2state(make_species(species), q);
  out8[0] = s.p; out8[1] = s.r; out8[2] = s.t; out8[3] = s.h; out8[4] = s.u2; out8[5] = s.a2;
  out8[6] = s.u[0]; out8[7] = s.u[1];
}
void hco_prim2cons(const double* species, const double* q, double* qc) {
  prim2cons(make_species(species), q, qc);
}
void hco_cons2prim(const double* species, const double* qc, double* q) {
  cons2prim(make_species(species), qc, q);
}
// the pointwise functions on a field of basis `basis` (BASIS_*): flux, boundary update, wall flux
void hco_flux_basis(int kind, int basis, const double* species, const double* face, const double* ql,
                    const double* qr, double* out5) {
  const Species<double> sp = make_species(species);
  put_flux(face_flux(kind, sp, make_face(face), basis2state(sp, ql, basis), basis2state(sp, qr, basis)), out5);
}
void hco_bc_update_basis(int kind, int basis, const double* species, const double* face, const double* qi,
                         const double* qf, double* qb) {
  const Species<double> sp = make_species(species);
  if (kind == BC_RIEMANN) bc_riemann(sp, make_face(face), qi, qf, qb, basis);
  else bc_entropy(sp, make_face(face), qi, qf, qb, basis);
}
void hco_wall_flux_basis(int basis, const double* species, const double* face, const double* qi, const double* dq,
                         double* out5) {
  put_flux(wall_flux(make_species(species), make_face(face), qi, dq, basis), out5);
}
// flux and far-field update with FIX_* corrections
void hco_flux_fixed(int kind, unsigned fixes, const double* species, const double* face, const double* ql,
                    const double* qr, double* out5) {
  Species<double> sp = make_species(species);
  sp.fixes = fixes;
  put_flux(face_flux(kind, sp, make_face(face), prim2state(sp, ql), prim2state(sp, qr)), out5);
}
void hco_bc_update_fixed(int kind, unsigned fixes, const double* species, const double* face, const double* qi,
                         const double* qf, double* qb) {
  Species<double> sp = make_species(species);
  sp.fixes = fixes;
  if (kind == BC_RIEMANN) bc_riemann(sp, make_face(face), qi, qf, qb);
  else bc_entropy(sp, make_face(face), qi, qf, qb);
}
// kind: 2 = Riemann, 3 = Entropy (face normal into the domain)
void hco_bc_update(int kind, const double* species, const double* face, const double* qi,
                   const double* qf, double* qb) {
  const Species<double> sp = make_species(species);
  if (kind == BC_RIEMANN) bc_riemann(sp, make_face(face), qi, qf, qb);
  else bc_entropy(sp, make_face(face), qi, qf, qb);
}
void hco_wall_flux(const double* species, const double* face, const double* qi, const double* dq,
                   double* out5) {
  put_flux(wall_flux(make_species(species), make_face(face), qi, dq), out5);
}
// delta transforms about the state of primitive set q: 0 cons->prim, 1 prim->cons,
// 2 prim->char, 3 char->prim
void hco_delta(int kind, const double* species, const double* q, const double* din, double* dout) {
  const Species<double> sp = make_species(species);
  const State<double> s = prim2state(sp, q);
  if (kind == 0) dcons2dprim(sp, s, din, dout);
  else if (kind == 1) dprim2dcons(sp, s, din, dout);
  else if (kind == 2) dprim2dchar(sp, s, din, dout);
  else dchar2dprim(sp, s, din, dout);
}
void hco_rk_table(int kind, double* out) {  // {nstages, maxcfl, alpha[16], beta[4]}
  const RKTable<double> t = rk_table<double>(kind);
  out[0] = t.nstages; out[1] = t.maxcfl;
  for (int i = 0; i < 4; ++i) for (int j = 0; j < 4; ++j) out[2 + 4 * i + j] = t.alpha[i][j];
  for (int i = 0; i < 4; ++i) out[18 + i] = t.beta[i];
}

// ---------------------------------------------------------------- meshes
// make_cylinder_mesh (mesh/generate/twoD.h:139-179): i radial, j around; with
// stretch s != 1 the radial spacing grows geometrically (D6).
void hco_cylinder_nodes(int nr, int nth, double rc, double rb, double stretch, double* nodes) {
  const double dr = (rb - rc) / nr;
  const double dth = (2. * M_PI) / nth;
  const double dr0 = (stretch == 1.0) ? dr : (rb - rc) * (stretch - 1.) / (std::pow(stretch, nr) - 1.);
  for (int i = 0; i <= nr; ++i)
    for (int j = 0; j <= nth; ++j) {
      const double r = (stretch == 1.0) ? rc + i * dr
                                        : rc + dr0 * (std::pow(stretch, i) - 1.) / (stretch - 1.);
      const double th = j * dth;
      nodes[(size_t(i) * (nth + 1) + j) * 2 + 0] = r * cos(th);
      nodes[(size_t(i) * (nth + 1) + j) * 2 + 1] = r * sin(th);
    }
}
// make_linspace_mesh (mesh/generate/twoD.h:15-40)
void hco_linspace_nodes(int nx, int ny, double lox, double hix, double loy, double hiy, double* nodes) {
  const double dx = (hix - lox) / nx, dy = (hiy - loy) / ny;
  for (int i = 0; i <= nx; ++i)
    for (int j = 0; j <= ny; ++j) {
      nodes[(size_t(i) * (ny + 1) + j) * 2 + 0] = lox + i * dx;
      nodes[(size_t(i) * (ny + 1) + j) * 2 + 1] = loy + j * dy;
    }
}

}  // extern "C"
