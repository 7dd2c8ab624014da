// ref_probe.cpp -- extern "C" probe over the reference's own pointwise code.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/ref/build_ref.sh against the
// reference headers (lacrymose/hyperboliConvergence cpp/inc); used in this
// container to generate the golden vectors in tests/golden/ that pin the CPU
// oracle.  Signatures match oracle/oracle_capi.cpp's hco_* pointwise functions.
#include <iostream>

#include <conservationLaws/euler/euler.h>
#include <conservationLaws/euler/boundaryConditions.h>
#include <conservationLaws/euler/boundary/riemann.ipp>
#include <conservationLaws/euler/boundary/entropy.ipp>
#include <conservationLaws/euler/boundary/inviscidWall.ipp>
#include <limiters/limiter.h>
#include <geometry/geometry.h>
#include <mesh/mesh.h>
#include <mesh/generate/twoD.h>
#include <ode.h>

#include <cmath>
#include <limits>

using Real = double;
constexpr LawType Law = LawType::Euler;
using PrimSet = VariableSet<Law, 2, EulerBases::Primitive, Real>;
using PrimDel = VariableDelta<Law, 2, EulerBases::Primitive, Real>;
using ConsSet = VariableSet<Law, 2, EulerBases::Conserved, Real>;
using ConsDel = VariableDelta<Law, 2, EulerBases::Conserved, Real>;
using CharDel = VariableDelta<Law, 2, EulerBases::Characteristic, Real>;
using StateT = State<Law, 2, Real>;
using Fr = FluxResult<Law, 2, Real>;

static Species<Law, Real> species_of(const double* sp) {
  Species<Law, Real> s = get_air_species<Real>();
  s.gamma = sp[0];
  s.R = sp[1];
  s.minf = sp[2];
  s.gamma1 = 1. / (s.gamma - 1.);
  return s;
}
static geom::Surface<2, Real> face_of(const double* f) {
  geom::Surface<2, Real> s;
  s.area = f[0];
  s.centre = geom::Point<2, Real>{f[1], f[2]};
  s.metric[0] = geom::Direction<2, Real>{f[3], f[4]};
  s.metric[1] = geom::Direction<2, Real>{f[5], f[6]};
  return s;
}
static PrimSet prim_of(const double* q) { return PrimSet{q[0], q[1], q[2], q[3]}; }
static void put(const Fr& r, double* out) {
  for (int v = 0; v < 4; ++v) out[v] = r.flux[v];
  out[4] = r.lambda;
}

// AusmPlusUP<V, P> for the nine low-Mach scalings (0 Convective, 1 Acoustic, 2 Adaptive);
// species = {gamma, R, minf, lref, dt}
template <LowMachScaling V, LowMachScaling P>
static void ausm_vp(const Species<Law, Real>& sp, const geom::Surface<2, Real>& f, const PrimSet& l,
                    const PrimSet& r, double* out5) {
  put(AusmPlusUP<V, P>{}(sp, f, l, r), out5);
}
template <LowMachScaling V, LowMachScaling P>
static void slau_vp(const Species<Law, Real>& sp, const geom::Surface<2, Real>& f, const PrimSet& l,
                    const PrimSet& r, double* out5) {
  put(Slau<V, P>{}(sp, f, l, r), out5);
}
template <LowMachScaling V>
static void slau_v(int pscale, const Species<Law, Real>& sp, const geom::Surface<2, Real>& f,
                   const PrimSet& l, const PrimSet& r, double* out5) {
  switch (pscale) {
    case 0: slau_vp<V, LowMachScaling::Convective>(sp, f, l, r, out5); break;
    case 1: slau_vp<V, LowMachScaling::Acoustic>(sp, f, l, r, out5); break;
    default: slau_vp<V, LowMachScaling::Adaptive>(sp, f, l, r, out5);
  }
}
template <LowMachScaling V>
static void ausm_v(int pscale, const Species<Law, Real>& sp, const geom::Surface<2, Real>& f,
                   const PrimSet& l, const PrimSet& r, double* out5) {
  switch (pscale) {
    case 0: ausm_vp<V, LowMachScaling::Convective>(sp, f, l, r, out5); break;
    case 1: ausm_vp<V, LowMachScaling::Acoustic>(sp, f, l, r, out5); break;
    default: ausm_vp<V, LowMachScaling::Adaptive>(sp, f, l, r, out5);
  }
}
extern "C" {

// kind numbering follows oracle/hc_oracle.hpp (FLUX_*); kind 1 (SLAU upwinded
// by the mass flux) has no reference counterpart and returns NaN.
void ref_flux(int kind, const double* species, const double* face, const double* ql, const double* qr,
              double* out5) {
  const auto sp = species_of(species);
  const auto f = face_of(face);
  const PrimSet l = prim_of(ql), r = prim_of(qr);
  switch (kind) {
    case 0: put(RoeFlux<Law>{}(sp, f, l, r), out5); break;
    case 2: put(Slau<LowMachScaling::Convective, LowMachScaling::Acoustic>{}(sp, f, l, r), out5); break;
    case 3: put(AusmPlusUP<LowMachScaling::Convective, LowMachScaling::Convective>{}(sp, f, l, r), out5); break;
    case 4: put(RusanovFlux<Law>{}(sp, f, l, r), out5); break;
    case 5: put(CentralFlux<Law>{}(sp, f, l, r), out5); break;
    case 6: put(RoeUnprecWS{}(sp, f, l, r), out5); break;
    default: for (int v = 0; v < 5; ++v) out5[v] = std::nan("");
  }
}

// Slau<V, P> for the nine low-Mach scalings; species = {gamma, R, minf, lref, dt}
void ref_slau_scaled(int vscale, int pscale, const double* species5, const double* face,
                     const double* ql, const double* qr, double* out5) {
  auto sp = species_of(species5);
  sp.lref = species5[3];
  sp.dt = species5[4];
  const auto f = face_of(face);
  const PrimSet l = prim_of(ql), r = prim_of(qr);
  switch (vscale) {
    case 0: slau_v<LowMachScaling::Convective>(pscale, sp, f, l, r, out5); break;
    case 1: slau_v<LowMachScaling::Acoustic>(pscale, sp, f, l, r, out5); break;
    default: slau_v<LowMachScaling::Adaptive>(pscale, sp, f, l, r, out5);
  }
}
void ref_ausmpup_scaled(int vscale, int pscale, const double* species5, const double* face,
                        const double* ql, const double* qr, double* out5) {
  auto sp = species_of(species5);
  sp.lref = species5[3];
  sp.dt = species5[4];
  const auto f = face_of(face);
  const PrimSet l = prim_of(ql), r = prim_of(qr);
  switch (vscale) {
    case 0: ausm_v<LowMachScaling::Convective>(pscale, sp, f, l, r, out5); break;
    case 1: ausm_v<LowMachScaling::Acoustic>(pscale, sp, f, l, r, out5); break;
    default: ausm_v<LowMachScaling::Adaptive>(pscale, sp, f, l, r, out5);
  }
}
void ref_exact_flux(const double* species, const double* normal, const double* q, double* out5) {
  const auto sp = species_of(species);
  put(exactFlux(sp, geom::Direction<2, Real>{normal[0], normal[1]}, set2State(sp, prim_of(q))), out5);
}
// kind numbering follows LIM_*; kind 7 (textbook van Leer) has no reference
// counterpart and returns NaN.
double ref_limit(int kind, double a, double b) {
  switch (kind) {
    case 0: return Limiters::NoLimit1{}.limit<Real>(a, b);
    case 1: return Limiters::NoLimit2{}.limit<Real>(a, b);
    case 2: return Limiters::NoLimit3{}.limit<Real>(a, b);
    case 3: return Limiters::VanAlbada2{}.limit<Real>(a, b);
    case 4: return Limiters::MinMod2{}.limit<Real>(a, b);
    case 5: return Limiters::Superbee2{}.limit<Real>(a, b);
    case 6: return Limiters::MonotonizedCentral2{}.limit<Real>(a, b);
    case 8: return Limiters::VanLeer2{}.limit<Real>(a, b);
    case 9: return Limiters::Cada3{}.limit<Real>(a, b);
    default: return std::nan("");
  }
}
void ref_surface(const double* p0, const double* p1, double* out7) {
  const auto s = geom::surface(geom::Point<2, Real>{p0[0], p0[1]}, geom::Point<2, Real>{p1[0], p1[1]});
  out7[0] = s.area; out7[1] = s.centre[0]; out7[2] = s.centre[1];
  out7[3] = s.metric[0][0]; out7[4] = s.metric[0][1]; out7[5] = s.metric[1][0]; out7[6] = s.metric[1][1];
}
void ref_volume(const double* p, double* out3) {
  const auto v = geom::volume(geom::Point<2, Real>{p[0], p[1]}, geom::Point<2, Real>{p[2], p[3]},
                              geom::Point<2, Real>{p[4], p[5]}, geom::Point<2, Real>{p[6], p[7]});
  out3[0] = v.volume; out3[1] = v.centre[0]; out3[2] = v.centre[1];
}
void ref_prim2state(const double* species, const double* q, double* out8) {
  const StateT s = set2State(species_of(species), prim_of(q));
  out8[0] = s.pressure(); out8[1] = s.density(); out8[2] = s.temperature();
  out8[3] = s.specificTotalEnthalpy(); out8[4] = s.velocity2(); out8[5] = s.speedOfSound2();
  out8[6] = s.velocity(0); out8[7] = s.velocity(1);
}
void ref_prim2cons(const double* species, const double* q, double* qc) {
  const ConsSet c = set2Set<ConsSet>(species_of(species), prim_of(q));
  for (int v = 0; v < 4; ++v) qc[v] = c[v];
}
void ref_cons2prim(const double* species, const double* qc, double* q) {
  const PrimSet p = set2Set<PrimSet>(species_of(species), ConsSet{qc[0], qc[1], qc[2], qc[3]});
  for (int v = 0; v < 4; ++v) q[v] = p[v];
}
// kind 2 = Riemann, 3 = Entropy; the face normal must point into the domain.
void ref_bc_update(int kind, const double* species, const double* face, const double* qi, const double* qf,
                   double* qb) {
  const auto sp = species_of(species);
  const auto f = face_of(face);
  geom::Volume<2, Real> cell;
  cell.volume = 1.;
  cell.centre = geom::Point<2, Real>{f.centre[0] + f.metric[0][0], f.centre[1] + f.metric[0][1]};
  PrimSet r;
  if (kind == 2)
    r = boundaryUpdate(std::integral_constant<EulerBCs, EulerBCs::Riemann>{}, sp, f, cell, prim_of(qi), prim_of(qf));
  else
    r = boundaryUpdate(std::integral_constant<EulerBCs, EulerBCs::Entropy>{}, sp, f, cell, prim_of(qi), prim_of(qf));
  for (int v = 0; v < 4; ++v) qb[v] = r[v];
}
void ref_wall_flux(const double* species, const double* face, const double* qi, const double* dq, double* out5) {
  const auto sp = species_of(species);
  const auto f = face_of(face);
  geom::Volume<2, Real> cell;
  cell.volume = 1.;
  cell.centre = f.centre;
  const PrimDel d{dq[0], dq[1], dq[2], dq[3]};
  put(boundaryFlux(std::integral_constant<EulerBCs, EulerBCs::InviscidWall>{}, sp, f, cell, d, prim_of(qi),
                   prim_of(qi), prim_of(qi)),
      out5);
}
// The same pointwise functions on a solution field in the conserved basis
// {rho u, rho v, rho, rho E}: inputs and outputs are ConsSet / ConsDel.
static ConsSet cons_of(const double* q) { return ConsSet{q[0], q[1], q[2], q[3]}; }
void ref_flux_cons(int kind, const double* species, const double* face, const double* ql, const double* qr,
                   double* out5) {
  const auto sp = species_of(species);
  const auto f = face_of(face);
  const ConsSet l = cons_of(ql), r = cons_of(qr);
  switch (kind) {
    case 0: put(RoeFlux<Law>{}(sp, f, l, r), out5); break;
    case 2: put(Slau<LowMachScaling::Convective, LowMachScaling::Acoustic>{}(sp, f, l, r), out5); break;
    case 3: put(AusmPlusUP<LowMachScaling::Convective, LowMachScaling::Convective>{}(sp, f, l, r), out5); break;
    case 4: put(RusanovFlux<Law>{}(sp, f, l, r), out5); break;
    case 5: put(CentralFlux<Law>{}(sp, f, l, r), out5); break;
    case 6: put(RoeUnprecWS{}(sp, f, l, r), out5); break;
    default: for (int v = 0; v < 5; ++v) out5[v] = std::nan("");
  }
}
void ref_bc_update_cons(int kind, const double* species, const double* face, const double* qi, const double* qf,
                        double* qb) {
  const auto sp = species_of(species);
  const auto f = face_of(face);
  geom::Volume<2, Real> cell;
  cell.volume = 1.;
  cell.centre = geom::Point<2, Real>{f.centre[0] + f.metric[0][0], f.centre[1] + f.metric[0][1]};
  ConsSet r;
  if (kind == 2)
    r = boundaryUpdate(std::integral_constant<EulerBCs, EulerBCs::Riemann>{}, sp, f, cell, cons_of(qi), cons_of(qf));
  else
    r = boundaryUpdate(std::integral_constant<EulerBCs, EulerBCs::Entropy>{}, sp, f, cell, cons_of(qi), cons_of(qf));
  for (int v = 0; v < 4; ++v) qb[v] = r[v];
}
void ref_wall_flux_cons(const double* species, const double* face, const double* qi, const double* dq,
                        double* out5) {
  const auto sp = species_of(species);
  const auto f = face_of(face);
  geom::Volume<2, Real> cell;
  cell.volume = 1.;
  cell.centre = f.centre;
  const ConsDel d{dq[0], dq[1], dq[2], dq[3]};
  put(boundaryFlux(std::integral_constant<EulerBCs, EulerBCs::InviscidWall>{}, sp, f, cell, d, cons_of(qi),
                   cons_of(qi), cons_of(qi)),
      out5);
}
// One-dimensional pointwise functions (nDim = 1: primitive sets {u, rho, p}, the face of a
// node with area 1 and normal +1, geometry/surface.ipp:4-11)
using Prim1 = VariableSet<Law, 1, EulerBases::Primitive, Real>;
static Prim1 prim1_of(const double* q) { return Prim1{q[0], q[1], q[2]}; }
static void put1(const FluxResult<Law, 1, Real>& r, double* out4) {
  for (int v = 0; v < 3; ++v) out4[v] = r.flux[v];
  out4[3] = r.lambda;
}
void ref_flux_1d(int kind, const double* species, const double* ql, const double* qr, double* out4) {
  const auto sp = species_of(species);
  const auto f = geom::surface(geom::Point<1, Real>{0.});
  const Prim1 l = prim1_of(ql), r = prim1_of(qr);
  switch (kind) {
    case 0: put1(RoeFlux<Law>{}(sp, f, l, r), out4); break;
    case 2: put1(Slau<LowMachScaling::Convective, LowMachScaling::Acoustic>{}(sp, f, l, r), out4); break;
    case 3: put1(AusmPlusUP<LowMachScaling::Convective, LowMachScaling::Convective>{}(sp, f, l, r), out4); break;
    case 4: put1(RusanovFlux<Law>{}(sp, f, l, r), out4); break;
    case 5: put1(CentralFlux<Law>{}(sp, f, l, r), out4); break;
    case 6: put1(RoeUnprecWS{}(sp, f, l, r), out4); break;
    default: for (int v = 0; v < 4; ++v) out4[v] = std::nan("");
  }
}
// boundary update of side 0 (left, face normal +1 into the domain) or 1 (right, the node's
// face flipped, spatial/boundary/boundaryUpdate.h:108-131); kind 2 Riemann, 3 Entropy
void ref_bc_update_1d(int kind, const double* species, int side, const double* qi, const double* qf, double* qb) {
  const auto sp = species_of(species);
  auto f = geom::surface(geom::Point<1, Real>{0.});
  if (side == 1) f = geom::flip(f);
  geom::Volume<1, Real> cell;
  cell.volume = 1.;
  cell.centre = geom::Point<1, Real>{f.metric[0][0]};
  Prim1 r;
  if (kind == 2)
    r = boundaryUpdate(std::integral_constant<EulerBCs, EulerBCs::Riemann>{}, sp, f, cell, prim1_of(qi), prim1_of(qf));
  else
    r = boundaryUpdate(std::integral_constant<EulerBCs, EulerBCs::Entropy>{}, sp, f, cell, prim1_of(qi), prim1_of(qf));
  for (int v = 0; v < 3; ++v) qb[v] = r[v];
}
// 0 cons->prim, 1 prim->cons, 2 prim->char, 3 char->prim about the state of q
void ref_delta(int kind, const double* species, const double* q, const double* din, double* dout) {
  const auto sp = species_of(species);
  const StateT s = set2State(sp, prim_of(q));
  if (kind == 0) {
    const PrimDel r = delta2Delta<PrimDel>(sp, s, ConsDel{din[0], din[1], din[2], din[3]});
    for (int v = 0; v < 4; ++v) dout[v] = r[v];
  } else if (kind == 1) {
    const ConsDel r = delta2Delta<ConsDel>(sp, s, PrimDel{din[0], din[1], din[2], din[3]});
    for (int v = 0; v < 4; ++v) dout[v] = r[v];
  } else if (kind == 2) {
    const CharDel r = delta2Delta<CharDel>(sp, s, PrimDel{din[0], din[1], din[2], din[3]});
    for (int v = 0; v < 4; ++v) dout[v] = r[v];
  } else {
    const PrimDel r = delta2Delta<PrimDel>(sp, s, CharDel{din[0], din[1], din[2], din[3]});
    for (int v = 0; v < 4; ++v) dout[v] = r[v];
  }
}
void ref_rk_table(int kind, double* out) {
  ODE::Explicit::RungeKutta<Real> t;
  if (kind == 0) t = ODE::Explicit::ssp11<Real>();
  else if (kind == 1) t = ODE::Explicit::ssp22<Real>();
  else if (kind == 2) t = ODE::Explicit::ssp33<Real>();
  else t = ODE::Explicit::ssp34<Real>();
  out[0] = t.nstages; out[1] = t.maxCFL;
  for (int i = 0; i < 4; ++i) for (int j = 0; j < 4; ++j) out[2 + 4 * i + j] = t.alpha[i][j];
  for (int i = 0; i < 4; ++i) out[18 + i] = t.beta[i];
}
void ref_cylinder_nodes(int nr, int nth, double rc, double rb, double* nodes) {
  const Mesh<2, Real> m = make_cylinder_mesh<Real>({rc, rb}, {size_t(nr), size_t(nth)});
  using Idx = typename Mesh<2, Real>::NodeArray::IdxType;
  for (int i = 0; i <= nr; ++i)
    for (int j = 0; j <= nth; ++j) {
      const auto& p = m.nodes(Idx{size_t(i), size_t(j)});
      nodes[(size_t(i) * (nth + 1) + j) * 2] = p[0];
      nodes[(size_t(i) * (nth + 1) + j) * 2 + 1] = p[1];
    }
}
void ref_linspace_nodes(int nx, int ny, double lox, double hix, double loy, double hiy, double* nodes) {
  const Mesh<2, Real> m = make_linspace_mesh<Real>(par::DualShape2{size_t(nx), size_t(ny)}, lox, hix, loy, hiy);
  using Idx = typename Mesh<2, Real>::NodeArray::IdxType;
  for (int i = 0; i <= nx; ++i)
    for (int j = 0; j <= ny; ++j) {
      const auto& p = m.nodes(Idx{size_t(i), size_t(j)});
      nodes[(size_t(i) * (ny + 1) + j) * 2] = p[0];
      nodes[(size_t(i) * (ny + 1) + j) * 2 + 1] = p[1];
    }
}

}  // extern "C"
