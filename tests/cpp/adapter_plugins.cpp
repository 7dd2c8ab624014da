// The C++ adapter's reference-shaped plug-in points.
//
// Without arguments: reads lines "flux <kind> <area cx cy nx ny tx ty> <uL vL rL pL>
// <uR vR rR pR>" and "limit <kind> <a> <b>" from stdin and prints, per line, the result
// of the tag's own call (RoeFlux{}.flux(species, face, sl, sr), the FluxInterface call
// operator on primitive sets, Limiters::...{}.limit(a, b)), for the caller to hold to
// the reference's golden vectors.  Needs no GPU (host evaluation).
//
// With --run: a driver shaped like the reference's cpp/script/euler/cylinder2D.cpp
// (species, O-grid mesh, solution field with bcTypes, the boundary-condition tuple,
// make_muscl_flux, integrate with the reference's argument list) on the GPU, 5 steps.
#include <hcgpu/hcgpu.hpp>

#include <cstdio>
#include <iostream>
#include <sstream>
#include <string>

using namespace hcgpu;

namespace {

template <class Flux>
void print_flux(const Flux& f, const Species<double>& sp, const geom::Surface<double>& face,
                const PrimitiveSet<double>& ql, const PrimitiveSet<double>& qr) {
  const FluxResult<double> a = f.flux(sp, face, set2State(sp, ql), set2State(sp, qr));
  const FluxResult<double> b = f(sp, face, ql, qr);  // FluxInterface on two primitive sets
  for (int v = 0; v < 4; ++v)
    if (a.flux[v] != b.flux[v]) std::printf("call operators differ\n");
  std::printf("%.17g %.17g %.17g %.17g %.17g\n", a.flux[0], a.flux[1], a.flux[2], a.flux[3], a.lambda);
}

template <class Limiter> void print_limit(const Limiter& l, double a, double b) {
  const double x = l.limit(a, b);
  const std::array<double, 2> v = l(std::array<double, 2>{a, a}, std::array<double, 2>{b, b});
  if (v[0] != x || v[1] != x) std::printf("variable limiter differs\n");
  std::printf("%.17g\n", x);
}

int cylinder2d_shaped() {
  constexpr LawType Law = LawType::Euler;
  const auto rk = ODE::Explicit::ssp34<double>();
  const UnsteadyTimeControls<double> timeControls{.nTimesteps = 5, .cfl = 0.5};
  const double mach = 0.3, pressure = 1.0 / 1.4, density = 1.0;
  const Species<double> species = [&]() {
    Species<double> gas = get_air_species<double>();
    gas.minf = mach;
    return gas;
  }();
  const auto mesh = make_cylinder_mesh<double>({0.5, 20.}, {64, 128}, 1.01);
  SolutionField<double> q(mesh.ni, mesh.nj);
  const std::array<double, 4> qref{mach, 0.0, density, pressure};
  for (int i = 0; i < mesh.ni; ++i)
    for (int j = 0; j < mesh.nj; ++j)
      for (int v = 0; v < 4; ++v) q(v, i, j) = qref[v];
  for (int s = 0; s < 4; ++s) q.fill_boundary(s, qref);
  const std::tuple boundaryConditions{make_ghostCell_BCond<Law, BC::Riemann>(),
                                      make_ghostCell_BCond<Law, BC::Entropy>(),
                                      make_flux_BCond<Law, BC::InviscidWall>(), make_fixed_BCond<Law>(),
                                      make_periodic_BCond<Law>()};
  q.bcTypes = {BC::InviscidWall, BC::Riemann, BC::Periodic, BC::Periodic};
  const auto hoflux = make_muscl_flux(Limiters::VanAlbada2{}, RoeFlux{});
  const hc_step_stats st =
      integrate(execution::gpu_local_dt, timeControls, rk, hoflux, boundaryConditions, species, mesh, q);
  // a tuple without the wall's condition is refused
  bool refused = false;
  try {
    const std::tuple partial{make_ghostCell_BCond<Law, BC::Riemann>(), make_periodic_BCond<Law>()};
    integrate(execution::gpu_local_dt, timeControls, rk, hoflux, partial, species, mesh, q);
  } catch (const Error& e) {
    refused = e.status == HC_ERR_ARG;
  }
  std::printf("cylinder2d-shaped run: t %.6g, last dt %.6g, density residual %.6g, refused %d\n", st.t, st.dt,
              st.resnorm, int(refused));
  return (st.status == 0 && refused) ? 0 : 1;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc > 1 && std::string(argv[1]) == "--run") return cylinder2d_shaped();
  Species<double> sp = get_air_species<double>();
  std::string line;
  while (std::getline(std::cin, line)) {
    std::istringstream in(line);
    std::string what;
    int kind = 0;
    in >> what >> kind;
    if (what == "species") {  // "species 0 <gamma> <R> <minf>"
      in >> sp.gamma >> sp.R >> sp.minf;
      continue;
    }
    if (what == "limit") {
      double a, b;
      in >> a >> b;
      switch (kind) {
        case HC_LIM_NOLIMIT1: print_limit(Limiters::NoLimit1{}, a, b); break;
        case HC_LIM_NOLIMIT2: print_limit(Limiters::NoLimit2{}, a, b); break;
        case HC_LIM_NOLIMIT3: print_limit(Limiters::NoLimit3{}, a, b); break;
        case HC_LIM_VANALBADA: print_limit(Limiters::VanAlbada2{}, a, b); break;
        case HC_LIM_MINMOD: print_limit(Limiters::MinMod2{}, a, b); break;
        case HC_LIM_SUPERBEE: print_limit(Limiters::Superbee2{}, a, b); break;
        case HC_LIM_MC: print_limit(Limiters::MonotonizedCentral2{}, a, b); break;
        case HC_LIM_VANLEER: print_limit(Limiters::VanLeer2{}, a, b); break;
        case HC_LIM_VANLEER_REF: print_limit(Limiters::VanLeer2Ref{}, a, b); break;
        default: print_limit(Limiters::Cada3{}, a, b); break;
      }
      continue;
    }
    geom::Surface<double> face;
    in >> face.area >> face.centre[0] >> face.centre[1] >> face.metric[0][0] >> face.metric[0][1] >>
        face.metric[1][0] >> face.metric[1][1];
    PrimitiveSet<double> ql, qr;
    for (auto& x : ql) in >> x;
    for (auto& x : qr) in >> x;
    switch (kind) {
      case HC_FLUX_ROE: print_flux(RoeFlux{}, sp, face, ql, qr); break;
      case HC_FLUX_SLAU: print_flux(Slau{}, sp, face, ql, qr); break;
      case HC_FLUX_SLAU_REF: print_flux(SlauRef{}, sp, face, ql, qr); break;
      case HC_FLUX_AUSMPUP: print_flux(AusmPlusUP<>{}, sp, face, ql, qr); break;
      case HC_FLUX_RUSANOV: print_flux(RusanovFlux{}, sp, face, ql, qr); break;
      case HC_FLUX_CENTRAL: print_flux(CentralFlux{}, sp, face, ql, qr); break;
      case HC_FLUX_ROE_WS: print_flux(RoeUnprecWS{}, sp, face, ql, qr); break;
      default: print_flux(RoeFluxFaceFrame{}, sp, face, ql, qr); break;
    }
  }
  return 0;
}
