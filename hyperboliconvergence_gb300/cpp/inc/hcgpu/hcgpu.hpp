// hcgpu.hpp -- C++20 host adapter with the reference's interfaces for the
// residual-and-timestep path, forwarding to the C ABI of include/hc.h.
//
// A driver written against the reference (cpp/script/euler/cylinder2D.cpp,
// gresho2D.cpp) changes its namespace and its execution policy:
//
//   const auto rk  = hcgpu::ODE::Explicit::ssp34<double>();
//   const hcgpu::UnsteadyTimeControls<double> tc{.nTimesteps = 100, .cfl = 0.5};
//   const auto species = hcgpu::get_air_species<double>();
//   const auto mesh = hcgpu::make_cylinder_mesh<double>({0.5, 20.}, {512, 1024}, 1.01);
//   hcgpu::SolutionField<double> q(mesh.ni, mesh.nj);      // primitive basis
//   q.bcTypes = {BC::InviscidWall, BC::Riemann, BC::Periodic, BC::Periodic};
//   const auto hoflux = hcgpu::make_muscl_flux(hcgpu::Limiters::VanAlbada2{}, hcgpu::RoeFlux{});
//   const std::tuple bcs{hcgpu::make_ghostCell_BCond<Law, BC::Riemann>(),
//                        hcgpu::make_flux_BCond<Law, BC::InviscidWall>(),
//                        hcgpu::make_periodic_BCond<Law>()};
//   hcgpu::integrate(hcgpu::execution::gpu, tc, rk, hoflux, bcs, species, mesh, q);
//
// The flux and limiter tags are also the reference's plug-in points on the host: a flux
// tag satisfies the FluxFunctor shape (flux(species, face, sl, sr) and the CRTP call
// operators of FluxInterface) and a limiter tag has limit(a, b) with the component-wise
// call of VariableLimiterInterface; both evaluate the library's own pointwise code
// (hc_flux_eval, hc_limit_eval).
//
// Errors: the reference asserts; here every failing C-ABI status throws
// hcgpu::Error carrying the status and hc_last_error_string().
#pragma once

#include <hc.h>

#include <array>
#include <cmath>
#include <cstddef>
#include <limits>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

namespace hcgpu {

struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline void check(int status) {
  if (status != HC_OK) throw Error(status, hc_last_error_string());
}

// Species<Euler> (conservationLaws/euler/euler.h:48-60) and get_air_species
// (conservationLaws/euler/species.ipp:1-17)
template <class Real> struct Species {
  Real gamma, minf, lref, nu, pr, dt, R, gamma1;
};
template <class Real> Species<Real> get_air_species() {
  Species<Real> s{};
  s.gamma = 1.4; s.minf = 0.0001; s.lref = 1.; s.pr = 0.7; s.nu = 1.81e-5;
  s.dt = std::numeric_limits<Real>::max(); s.R = 287.058; s.gamma1 = 1. / (s.gamma - 1.);
  return s;
}

// LowMachScaling (conservationLaws/euler/euler.h:331-339)
enum class LowMachScaling { Convective = HC_SCALING_CONVECTIVE, Acoustic = HC_SCALING_ACOUSTIC,
                            Adaptive = HC_SCALING_ADAPTIVE };

// LawType (conservationLaws/base/declarations.h:7-18) of the laws this adapter drives
enum class LawType { Euler = HC_LAW_EULER, ScalarAdvection = HC_LAW_SCALAR };

namespace geom {
// Surface<2,Real> (geometry/geometry.h:64-70): area, centre and the face metric, whose
// rows are the unit normal and the unit tangent
template <class Real> struct Surface {
  Real area;
  std::array<Real, 2> centre;
  std::array<std::array<Real, 2>, 2> metric;
};
}  // namespace geom

// State<Euler,2,Real> (conservationLaws/euler/euler.h:62-83) and its accessors
template <class Real> struct State {
  std::array<Real, 8> state{};
  Real& pressure() { return state[0]; }
  Real& density() { return state[1]; }
  Real& temperature() { return state[2]; }
  Real& specificTotalEnthalpy() { return state[3]; }
  Real& velocity2() { return state[4]; }
  Real& speedOfSound2() { return state[5]; }
  Real& velocity(int i) { return state[6 + i]; }
  const Real& pressure() const { return state[0]; }
  const Real& density() const { return state[1]; }
  const Real& temperature() const { return state[2]; }
  const Real& specificTotalEnthalpy() const { return state[3]; }
  const Real& velocity2() const { return state[4]; }
  const Real& speedOfSound2() const { return state[5]; }
  const Real& velocity(int i) const { return state[6 + i]; }
};

// a primitive variable set {u, v, rho, p} (VariableSet<Euler,2,Primitive,Real>)
template <class Real> using PrimitiveSet = std::array<Real, 4>;

// set2State of a primitive set (conservationLaws/euler/transforms/primitive.ipp:24-60)
template <class Real> State<Real> set2State(const Species<Real>& sp, const PrimitiveSet<Real>& q) {
  State<Real> s;
  s.velocity(0) = q[0];
  s.velocity(1) = q[1];
  s.density() = q[2];
  s.pressure() = q[3];
  s.temperature() = q[3] / (q[2] * sp.R);
  s.velocity2() = q[0] * q[0] + q[1] * q[1];
  s.speedOfSound2() = sp.gamma * sp.R * s.temperature();
  s.specificTotalEnthalpy() = s.speedOfSound2() / (sp.gamma - Real(1)) + Real(0.5) * s.velocity2();
  return s;
}

// FluxResult<Euler,2,Real> (conservationLaws/base/base.h:57-83): the conserved flux
// components {rho u, rho v, rho, rho E} times the area, and the spectral radius times the area
template <class Real> struct FluxResult {
  std::array<Real, 4> flux;
  Real lambda;
};

// FluxInterface (conservationLaws/base/base.h:370-397): the call operators a FluxFunctor
// has, on two States or on two primitive sets
template <class Flux> struct FluxInterface {
  template <class Real>
  FluxResult<Real> operator()(const Species<Real>& species, const geom::Surface<Real>& face, const State<Real>& sl,
                              const State<Real>& sr) const {
    return static_cast<const Flux*>(this)->flux(species, face, sl, sr);
  }
  template <class Real>
  FluxResult<Real> operator()(const Species<Real>& species, const geom::Surface<Real>& face,
                              const PrimitiveSet<Real>& ql, const PrimitiveSet<Real>& qr) const {
    return static_cast<const Flux*>(this)->flux(species, face, set2State(species, ql), set2State(species, qr));
  }
};

namespace detail {
template <class Real>
FluxResult<Real> eval_flux(int id, int vscale, int pscale, const Species<Real>& sp, const geom::Surface<Real>& f,
                           const State<Real>& sl, const State<Real>& sr) {
  const double species[5] = {double(sp.gamma), double(sp.R), double(sp.minf), double(sp.lref), double(sp.dt)};
  const double face[7] = {double(f.area), double(f.centre[0]), double(f.centre[1]), double(f.metric[0][0]),
                          double(f.metric[0][1]), double(f.metric[1][0]), double(f.metric[1][1])};
  const double ql[4] = {double(sl.velocity(0)), double(sl.velocity(1)), double(sl.density()), double(sl.pressure())};
  const double qr[4] = {double(sr.velocity(0)), double(sr.velocity(1)), double(sr.density()), double(sr.pressure())};
  double out[5];
  check(hc_flux_eval(id, vscale, pscale, species, face, ql, qr, out));
  return FluxResult<Real>{{Real(out[0]), Real(out[1]), Real(out[2]), Real(out[3])}, Real(out[4])};
}
}  // namespace detail

// Flux tags: the FluxFunctor plug-in point (conservationLaws/base/concepts.h:97-107).  The
// id selects the device flux of a run; flux() evaluates the same pointwise code on the host.
template <int ID> struct FluxTag : FluxInterface<FluxTag<ID>> {
  static constexpr int id = ID;
  template <class Real>
  FluxResult<Real> flux(const Species<Real>& species, const geom::Surface<Real>& face, const State<Real>& sl,
                        const State<Real>& sr) const {
    return detail::eval_flux(ID, HC_SCALING_CONVECTIVE, HC_SCALING_CONVECTIVE, species, face, sl, sr);
  }
};
using RoeFlux = FluxTag<HC_FLUX_ROE>;
using RoeFluxFaceFrame = FluxTag<HC_FLUX_ROE_FACE>;  // the face-frame Roe dissipation (not in the reference)
using Slau = FluxTag<HC_FLUX_SLAU>;
using SlauRef = FluxTag<HC_FLUX_SLAU_REF>;
using RusanovFlux = FluxTag<HC_FLUX_RUSANOV>;
using CentralFlux = FluxTag<HC_FLUX_CENTRAL>;
using RoeUnprecWS = FluxTag<HC_FLUX_ROE_WS>;
template <LowMachScaling VFluxScaling = LowMachScaling::Convective,
          LowMachScaling PFluxScaling = LowMachScaling::Convective>
struct AusmPlusUP : FluxInterface<AusmPlusUP<VFluxScaling, PFluxScaling>> {
  static constexpr int id = HC_FLUX_AUSMPUP;
  static constexpr int vscale = int(VFluxScaling), pscale = int(PFluxScaling);
  template <class Real>
  FluxResult<Real> flux(const Species<Real>& species, const geom::Surface<Real>& face, const State<Real>& sl,
                        const State<Real>& sr) const {
    return detail::eval_flux(id, vscale, pscale, species, face, sl, sr);
  }
};

// VariableLimiterInterface (limiters/limiter.h:14-28): the limiter applied component by
// component to two variable deltas (any type with size() and operator[])
template <class Limiter> struct VariableLimiterInterface {
  template <class Delta> Delta operator()(const Delta& dq0, const Delta& dq1) const {
    Delta out = dq0;
    for (std::size_t i = 0; i < dq0.size(); ++i) out[i] = static_cast<const Limiter*>(this)->limit(dq0[i], dq1[i]);
    return out;
  }
};

// Limiter tags (limiters/limiter.h:43-131): limit(a, b) as the reference's limiters
// (limiters/limiter.ipp:8-161), evaluated by the library's pointwise code
template <int ID> struct LimiterTag : VariableLimiterInterface<LimiterTag<ID>> {
  static constexpr int id = ID;
  template <class Real> Real limit(const Real a, const Real b) const {
    double o = 0;
    check(hc_limit_eval(ID, double(a), double(b), &o));
    return Real(o);
  }
};
namespace Limiters {
using NoLimit1 = LimiterTag<HC_LIM_NOLIMIT1>;
using NoLimit2 = LimiterTag<HC_LIM_NOLIMIT2>;
using NoLimit3 = LimiterTag<HC_LIM_NOLIMIT3>;
using VanAlbada2 = LimiterTag<HC_LIM_VANALBADA>;
using MinMod2 = LimiterTag<HC_LIM_MINMOD>;
using Superbee2 = LimiterTag<HC_LIM_SUPERBEE>;
using MonotonizedCentral2 = LimiterTag<HC_LIM_MC>;
using VanLeer2 = LimiterTag<HC_LIM_VANLEER>;
using VanLeer2Ref = LimiterTag<HC_LIM_VANLEER_REF>;
using Cada3 = LimiterTag<HC_LIM_CADA3>;
}  // namespace Limiters

// make_muscl_flux (spatial/muscl.h:10-87): the second-order flux descriptor
struct MusclFlux {
  int limiter;
  int flux;
  int vscale = HC_SCALING_CONVECTIVE, pscale = HC_SCALING_CONVECTIVE;  // AUSM+up's scalings
};
template <class Limiter, class Flux> MusclFlux make_muscl_flux(const Limiter&, const Flux&) {
  if constexpr (requires { Flux::vscale; }) return MusclFlux{Limiter::id, Flux::id, Flux::vscale, Flux::pscale};
  else return MusclFlux{Limiter::id, Flux::id};
}

// ODE::Explicit::RungeKutta tables (ode.h:85-197); the id selects the device table
namespace ODE::Explicit {
template <class Real> struct RungeKutta {
  unsigned order, nstages;
  Real maxCFL;
  int id;
};
template <class Real> RungeKutta<Real> ssp11() { return {1, 1, Real(1), HC_RK_SSP11}; }
template <class Real> RungeKutta<Real> ssp22() { return {2, 2, Real(1), HC_RK_SSP22}; }
template <class Real> RungeKutta<Real> ssp33() { return {3, 3, Real(1), HC_RK_SSP33}; }
template <class Real> RungeKutta<Real> ssp34() { return {3, 4, Real(2), HC_RK_SSP34}; }
}  // namespace ODE::Explicit

// UnsteadyTimeControls (controls.h:11-19)
template <class Real> struct UnsteadyTimeControls {
  std::size_t nTimesteps;
  Real cfl;
};

// SteadyTimeControls (controls.h:31-48)
template <class Real> struct SteadyTimeControls {
  std::size_t nTimesteps;
  Real cfl;
  Real residual_drop;
  bool use_residual_smoothing = false;
  Real smoothing_factor = 0;
};

// execution policies: the GPU path in global or local timestepping
namespace execution {
struct gpu_policy { int dt_mode = HC_DT_GLOBAL; int precision = HC_FP64; };
inline constexpr gpu_policy gpu{HC_DT_GLOBAL, HC_FP64};
inline constexpr gpu_policy gpu_local_dt{HC_DT_LOCAL, HC_FP64};
inline constexpr gpu_policy gpu_fp32{HC_DT_GLOBAL, HC_FP32};
inline constexpr gpu_policy gpu_fp32_local_dt{HC_DT_LOCAL, HC_FP32};
// FP64 state and update, stage arithmetic in double-float
inline constexpr gpu_policy gpu_df{HC_DT_GLOBAL, HC_FP64_DF};
inline constexpr gpu_policy gpu_df_local_dt{HC_DT_LOCAL, HC_FP64_DF};
}  // namespace execution

// Mesh<2,Real> nodes (mesh/mesh.h:19-57)
template <class Real> struct Mesh {
  int ni = 0, nj = 0;
  std::vector<double> nodes;  // (ni+1)*(nj+1) x,y pairs
};
template <class Real>
Mesh<Real> make_cylinder_mesh(const std::array<Real, 2> lengths, const std::array<std::size_t, 2> ncells,
                              double stretch = 1.0) {
  Mesh<Real> m;
  m.ni = int(ncells[0]); m.nj = int(ncells[1]);
  m.nodes.resize(std::size_t(m.ni + 1) * (m.nj + 1) * 2);
  check(hc_mesh_cylinder_nodes(m.ni, m.nj, lengths[0], lengths[1], stretch, m.nodes.data()));
  return m;
}
template <class Real>
Mesh<Real> make_linspace_mesh(const std::array<std::size_t, 2> cellDims, Real lox, Real hix, Real loy, Real hiy) {
  Mesh<Real> m;
  m.ni = int(cellDims[0]); m.nj = int(cellDims[1]);
  m.nodes.resize(std::size_t(m.ni + 1) * (m.nj + 1) * 2);
  check(hc_mesh_linspace_nodes(m.ni, m.nj, lox, hix, loy, hiy, m.nodes.data()));
  return m;
}

// EulerBCs (conservationLaws/euler/euler.h:31-41)
enum class BC { Periodic = HC_BC_PERIODIC, Riemann = HC_BC_RIEMANN, Entropy = HC_BC_ENTROPY,
                Fixed = HC_BC_FIXED, InviscidWall = HC_BC_WALL };

// Boundary conditions of the reference's BC tuple (spatial/boundary/boundaryCondition.h:49-136):
// each names the boundary type it implements; the sides' types are q.bcTypes, and the
// device applies the type's ghost update or flux.
template <BC T> struct BoundaryCondition {
  static constexpr BC type = T;
};
template <LawType Law, BC T> BoundaryCondition<T> make_ghostCell_BCond() {
  static_assert(T == BC::Riemann || T == BC::Entropy, "ghost-cell conditions: Riemann or Entropy");
  return {};
}
template <LawType Law, BC T> BoundaryCondition<T> make_flux_BCond() {
  static_assert(T == BC::InviscidWall, "flux conditions: InviscidWall");
  return {};
}
template <LawType Law> BoundaryCondition<BC::Fixed> make_fixed_BCond() { return {}; }
template <LawType Law> BoundaryCondition<BC::Periodic> make_periodic_BCond() { return {}; }

namespace detail {
// the reference dispatches each side to the tuple's condition of the side's type; a side
// whose type the tuple does not hold has no condition
template <class... BCs> void check_bc_tuple(const std::tuple<BCs...>& bcs, const std::array<BC, 4>& types) {
  for (int s = 0; s < 4; ++s) {
    const bool found = std::apply([&](const auto&... b) { return ((b.type == types[s]) || ...); }, bcs);
    if (!found) throw Error(HC_ERR_ARG, "side " + std::to_string(s) + ": the boundary-condition tuple holds no "
                                        "condition of the side's type");
  }
}
}  // namespace detail

// SolutionField (solutionField/solutionField.h:56-91) in the primitive basis:
// interior as 4 planes {u, v, rho, p}; boundary[side] the reference layer,
// 4 planes per side face (nj faces on sides 0/1, ni on 2/3).
// the basis of a SolutionField<SolVarT,2>: its SolVarT (primitive or conserved set)
enum class Basis { Primitive = HC_BASIS_PRIMITIVE, Conserved = HC_BASIS_CONSERVED };

template <class Real> struct SolutionField {
  int ni, nj;
  Basis basis = Basis::Primitive;  // of interior and boundary
  std::vector<double> interior;
  std::array<std::vector<double>, 4> boundary;
  std::array<BC, 4> bcTypes{BC::Periodic, BC::Periodic, BC::Periodic, BC::Periodic};
  SolutionField(int ni_, int nj_) : ni(ni_), nj(nj_), interior(std::size_t(4) * ni_ * nj_) {
    for (int s = 0; s < 4; ++s) boundary[s].assign(std::size_t(4) * (s < 2 ? nj_ : ni_), 0.0);
  }
  double& operator()(int var, int i, int j) { return interior[(std::size_t(var) * ni + i) * nj + j]; }
  void fill_boundary(int side, const std::array<double, 4>& prim) {
    const std::size_t n = boundary[side].size() / 4;
    for (int v = 0; v < 4; ++v)
      for (std::size_t k = 0; k < n; ++k) boundary[side][v * n + k] = prim[v];
  }
};

// RAII context over the C ABI
class Context {
 public:
  Context(const hc_config& cfg) { check(hc_context_create(&cfg, &ctx_)); }
  ~Context() { hc_context_destroy(ctx_); }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  hc_ctx* get() const { return ctx_; }

 private:
  hc_ctx* ctx_ = nullptr;
};

// integrate (timestepping/rungeKutta.h:37-167): advances q by nTimesteps RK
// steps on the GPU and returns the last step's statistics.
template <class Real>
hc_step_stats integrate(const execution::gpu_policy policy, const UnsteadyTimeControls<Real>& timeControls,
                        const ODE::Explicit::RungeKutta<Real>& rungeKutta, const MusclFlux& flux2,
                        const Species<Real>& species, const Mesh<Real>& mesh, SolutionField<Real>& q) {
  if (q.ni != mesh.ni || q.nj != mesh.nj) throw Error(HC_ERR_ARG, "solution field and mesh shapes differ");
  hc_config cfg{flux2.flux, flux2.limiter, rungeKutta.id, policy.precision, policy.dt_mode,
                double(timeControls.cfl), HC_LAW_EULER, int(q.basis)};
  Context ctx(cfg);
  check(hc_mesh_upload(ctx.get(), mesh.ni, mesh.nj, mesh.nodes.data()));
  check(hc_set_species(ctx.get(), species.gamma, species.R, species.minf));
  check(hc_set_low_mach(ctx.get(), flux2.vscale, flux2.pscale, double(species.lref), double(species.dt)));
  int bct[4];
  const double* refs[4];
  for (int s = 0; s < 4; ++s) {
    bct[s] = int(q.bcTypes[s]);
    refs[s] = q.boundary[s].data();
  }
  check(hc_set_bcs(ctx.get(), bct, refs));
  // the caller's field advanced in place: upload, steps, download, one wait
  hc_step_stats st{};
  check(hc_step_host(ctx.get(), int(timeControls.nTimesteps), q.interior.data(), q.interior.data(), &st));
  return st;
}

// Steady-state integrate: the convergence loop SteadyTimeControls describes, on the
// GPU; returns the residual history (read every check_every steps) and the stats.
template <class Real>
hc_steady_stats integrate(const execution::gpu_policy policy, const SteadyTimeControls<Real>& timeControls,
                          const ODE::Explicit::RungeKutta<Real>& rungeKutta, const MusclFlux& flux2,
                          const Species<Real>& species, const Mesh<Real>& mesh, SolutionField<Real>& q,
                          std::vector<double>* history = nullptr, int check_every = 100) {
  if (q.ni != mesh.ni || q.nj != mesh.nj) throw Error(HC_ERR_ARG, "solution field and mesh shapes differ");
  hc_config cfg{flux2.flux, flux2.limiter, rungeKutta.id, policy.precision, policy.dt_mode,
                double(timeControls.cfl), HC_LAW_EULER, int(q.basis)};
  Context ctx(cfg);
  check(hc_mesh_upload(ctx.get(), mesh.ni, mesh.nj, mesh.nodes.data()));
  check(hc_set_species(ctx.get(), species.gamma, species.R, species.minf));
  check(hc_set_low_mach(ctx.get(), flux2.vscale, flux2.pscale, double(species.lref), double(species.dt)));
  int bct[4];
  const double* refs[4];
  for (int s = 0; s < 4; ++s) {
    bct[s] = int(q.bcTypes[s]);
    refs[s] = q.boundary[s].data();
  }
  check(hc_set_bcs(ctx.get(), bct, refs));
  check(hc_state_upload(ctx.get(), q.interior.data()));
  const hc_steady_controls ctl{(long long)timeControls.nTimesteps, double(timeControls.residual_drop), check_every,
                               timeControls.use_residual_smoothing ? 1 : 0, double(timeControls.smoothing_factor)};
  std::vector<double> h(timeControls.nTimesteps / std::size_t(check_every) + 2);
  hc_steady_stats st{};
  check(hc_steady_run(ctx.get(), &ctl, h.data(), (long long)h.size(), &st));
  check(hc_state_download(ctx.get(), q.interior.data()));
  if (history) history->assign(h.begin(), h.begin() + st.history_len);
  return st;
}

// integrate with the reference's argument list (timestepping/rungeKutta.h:37-51): the BC
// tuple between the high-order flux and the species
template <class Real, class... BCs>
hc_step_stats integrate(const execution::gpu_policy policy, const UnsteadyTimeControls<Real>& timeControls,
                        const ODE::Explicit::RungeKutta<Real>& rungeKutta, const MusclFlux& flux2,
                        const std::tuple<BCs...>& boundaryConditions, const Species<Real>& species,
                        const Mesh<Real>& mesh, SolutionField<Real>& q) {
  detail::check_bc_tuple(boundaryConditions, q.bcTypes);
  return integrate(policy, timeControls, rungeKutta, flux2, species, mesh, q);
}
template <class Real, class... BCs>
hc_steady_stats integrate(const execution::gpu_policy policy, const SteadyTimeControls<Real>& timeControls,
                          const ODE::Explicit::RungeKutta<Real>& rungeKutta, const MusclFlux& flux2,
                          const std::tuple<BCs...>& boundaryConditions, const Species<Real>& species,
                          const Mesh<Real>& mesh, SolutionField<Real>& q, std::vector<double>* history = nullptr,
                          int check_every = 100) {
  detail::check_bc_tuple(boundaryConditions, q.bcTypes);
  return integrate(policy, timeControls, rungeKutta, flux2, species, mesh, q, history, check_every);
}

}  // namespace hcgpu
