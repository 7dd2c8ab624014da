// ref_probe_scalar.cpp -- extern "C" probe over the reference's scalar
// advection law (conservationLaws/scalarAdvection): Rusanov and central fluxes
// and the Riemann (inflow/outflow) ghost update, conserved basis {u, v, q}.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/ref/build_ref.sh against the
// reference headers; used in this container to generate golden vectors.
#include <iostream>

#include <conservationLaws/scalarAdvection/scalarAdvection.h>
#include <conservationLaws/scalarAdvection/boundaryConditions.h>
#include <geometry/geometry.h>

using Real = double;
constexpr LawType Law = LawType::ScalarAdvection;
using ConsSet = VariableSet<Law, 2, ScalarAdvectionBases::Conserved, Real>;
using StateT = State<Law, 2, Real>;
using Fr = FluxResult<Law, 2, Real>;

static geom::Surface<2, Real> face_of(const double* f) {
  geom::Surface<2, Real> s;
  s.area = f[0];
  s.centre = geom::Point<2, Real>{f[1], f[2]};
  s.metric[0] = geom::Direction<2, Real>{f[3], f[4]};
  s.metric[1] = geom::Direction<2, Real>{f[5], f[6]};
  return s;
}
static ConsSet cons_of(const double* q) { return ConsSet{q[0], q[1], q[2]}; }
static void put(const Fr& r, double* out) {
  for (int v = 0; v < 3; ++v) out[v] = r.flux[v];
  out[3] = r.lambda;
}

extern "C" {

// kind 0: RusanovFlux, 1: CentralFlux; states in the conserved basis {u, v, q}
void ref_scalar_flux(int kind, const double* face, const double* ql, const double* qr, double* out4) {
  const Species<Law, Real> sp{};
  const geom::Surface<2, Real> f = face_of(face);
  const StateT sl = set2State(sp, cons_of(ql));
  const StateT sr = set2State(sp, cons_of(qr));
  if (kind == 0) put(RusanovFlux<Law>::flux(sp, f, sl, sr), out4);
  else put(CentralFlux<Law>::flux(sp, f, sl, sr), out4);
}

// Riemann ghost update: face normal into the domain, interior and boundary values
void ref_scalar_bc_riemann(const double* face, const double* qi, const double* qb, double* out3) {
  const Species<Law, Real> sp{};
  const geom::Surface<2, Real> f = face_of(face);
  const geom::Volume<2, Real> cell{};
  const ConsSet g = boundaryUpdate(std::integral_constant<ScalarAdvectionBCs, ScalarAdvectionBCs::Riemann>{}, sp, f,
                                   cell, cons_of(qi), cons_of(qb));
  for (int v = 0; v < 3; ++v) out3[v] = g[v];
}

}  // extern "C"
