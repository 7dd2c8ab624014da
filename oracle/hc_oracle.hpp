// hc_oracle.hpp -- CPU oracle for the residual-and-timestep path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA path is
// compared against; it is never linked into the product library.  Only the
// tests, the smoke check and the CPU-baseline leg of the benchmark load it.
//
// It restates, in plain scalar C++, the algorithm of the reference solver
// (lacrymose/hyperboliConvergence, cpp/inc) for 2D structured meshes:
// pointwise Euler physics, limiters, least-squares gradients, MUSCL faces,
// residual accumulation, boundary conditions, spectral radius and the
// alpha/beta Runge-Kutta integrator.  Operation order follows the reference
// expression by expression so that, built without contraction or fast-math,
// the pointwise functions reproduce the reference bit for bit (pinned by the
// golden vectors generated from the reference's own headers).
//
// Variable order everywhere (reference conservationLaws/euler/euler.h:19-25):
//   primitive  = { u, v, rho, p }
//   conserved  = { rho*u, rho*v, rho, rho*E }
// Storage order of 2D arrays: cell (i,j) at i*nj + j (j fastest), as
// par::Array (parallalg/array.h:46-59).
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

namespace hco {

// unqualified math calls: double resolves to <cmath>, other arithmetic types
// (the forward-mode Dual of hc_dual.hpp) to their own overloads
using std::abs;
using std::fabs;
using std::fmax;
using std::fmin;
using std::pow;
using std::sqrt;

// the per-step timestep is held fixed when differentiating (identity here)
template <class R> R freeze(const R& x) { return x; }

// ---------------------------------------------------------------- enums
enum Flux { FLUX_ROE = 0, FLUX_SLAU = 1, FLUX_SLAU_REF = 2, FLUX_AUSMPUP = 3,
            FLUX_RUSANOV = 4, FLUX_CENTRAL = 5, FLUX_ROE_WS = 6, FLUX_ROE_FACE = 7 };
// LowMachScaling (conservationLaws/euler/euler.h:331-339)
enum Scaling { SCALING_CONVECTIVE = 0, SCALING_ACOUSTIC = 1, SCALING_ADAPTIVE = 2 };
enum Limiter { LIM_NOLIMIT1 = 0, LIM_NOLIMIT2 = 1, LIM_NOLIMIT3 = 2, LIM_VANALBADA = 3,
               LIM_MINMOD = 4, LIM_SUPERBEE = 5, LIM_MC = 6, LIM_VANLEER = 7,
               LIM_VANLEER_REF = 8, LIM_CADA3 = 9 };
enum BC { BC_PERIODIC = 0, BC_FIXED = 1, BC_RIEMANN = 2, BC_ENTROPY = 3, BC_WALL = 4 };
enum RK { RK_SSP11 = 0, RK_SSP22 = 1, RK_SSP33 = 2, RK_SSP34 = 3 };
enum DtMode { DT_GLOBAL = 0, DT_LOCAL = 1 };

// ---------------------------------------------------------------- types
// Species<Euler> (conservationLaws/euler/euler.h:48-60)
template <class R> struct Species {
  R gamma, minf, lref, nu, pr, dt, Rgas, gamma1;
  // corrections of two defects of the reference (FIX_*), 0 = as the reference computes
  unsigned fixes;
};
// FIX_MACH_SPLIT_P1: MachSplit_P1 as M1/M, the 1/0 split it is meant to be, instead of the
// (M1 + eps)/(|M| + eps) with the largest eps that it is (machSplittings.ipp:26-31);
// FIX_FARFIELD_TRANSVERSE: the
// far fields' transverse-flow test on |u_n|/|u| (conservationLaws/euler/boundary/riemann.ipp:48-50, entropy.ipp:47-49), so
// outflow faces get the characteristic update instead of an interior copy
enum : unsigned { FIX_MACH_SPLIT_P1 = 1u, FIX_FARFIELD_TRANSVERSE = 2u };

// get_air_species (conservationLaws/euler/species.ipp:1-17)
template <class R> Species<R> air_species() {
  Species<R> s;
  s.gamma = 1.4; s.minf = 0.0001; s.lref = 1.; s.pr = 0.7; s.nu = 1.81e-5;
  s.dt = std::numeric_limits<R>::max(); s.Rgas = 287.058;
  s.gamma1 = 1. / (s.gamma - 1.);
  s.fixes = 0u;
  return s;
}

// State<Euler,2> (conservationLaws/euler/euler.h:62-83)
template <class R> struct State { R p, r, t, h, u2, a2, u[2]; };

// geom::Surface / geom::Volume (geometry/geometry.h:64-81)
template <class R> struct Face { R area; R c[2]; R n[2]; R t[2]; };
template <class R> struct Cell { R vol; R c[2]; };

// FluxResult (conservationLaws/base/base.h:57-83)
template <class R> struct FluxRes { R f[4]; R lam; };

// ---------------------------------------------------------------- geometry
// geom::surface(p0,p1) (geometry/surface.ipp:12-29)
template <class R> Face<R> surface(const R* p0, const R* p1) {
  Face<R> s;
  const R t0x = p1[0] - p0[0], t0y = p1[1] - p0[1];
  const R t1x = p0[0] - p1[0], t1y = p0[1] - p1[1];
  R d = 0; d += t0x * t0x; d += t0y * t0y;
  const R l = sqrt(d);
  const R l1 = 1. / l;
  s.area = l;
  s.c[0] = p0[0] + 0.5 * t0x;
  s.c[1] = p0[1] + 0.5 * t0y;
  const R ux = l1 * t1x, uy = l1 * t1y;  // l1*tangent1
  s.n[0] = -uy; s.n[1] = ux;               // orthog (geometry/operations.ipp:43-47)
  s.t[0] = l1 * t0x; s.t[1] = l1 * t0y;
  return s;
}

// geom::volume(p0..p3) (geometry/volume.ipp:25-66): bilinear shape functions
// at the element centre (fem/fem.h:14-77).  The value is |J(0,0)|, which is a
// quarter of the quad's area; it is kept as the reference defines it.
template <class R> Cell<R> volume(const R* p0, const R* p1, const R* p2, const R* p3) {
  // shape functions n2 and derivatives dn2 evaluated at (0,0): exact binary fractions
  const R u[4] = {0.25, 0.25, 0.25, 0.25};
  const R du[4][2] = {{-0.25, -0.25}, {0.25, -0.25}, {-0.25, 0.25}, {0.25, 0.25}};
  const R* p[4] = {p0, p1, p2, p3};
  Cell<R> c;
  for (int i = 0; i < 2; ++i) {
    R com = 0;
    for (int k = 0; k < 4; ++k) com += u[k] * p[k][i];
    c.c[i] = com;
  }
  R tg[2][2] = {{0, 0}, {0, 0}};
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j)
      for (int k = 0; k < 4; ++k) tg[i][j] += du[k][i] * p[k][j];
  c.vol = fabs(tg[0][0] * tg[1][1] - tg[0][1] * tg[1][0]);
  return c;
}

// ---------------------------------------------------------------- transforms
// set2State(primitive) (conservationLaws/euler/transforms/primitive.ipp:24-60)
template <class R> State<R> prim2state(const Species<R>& sp, const R* q) {
  State<R> s;
  s.u2 = 0;
  for (int i = 0; i < 2; ++i) { s.u[i] = q[i]; s.u2 += q[i] * q[i]; }
  const R k = 0.5 * s.u2;
  const R r = q[2], p = q[3];
  const R t = p / (r * sp.Rgas);
  const R a2 = sp.gamma * sp.Rgas * t;
  const R h = a2 * sp.gamma1 + k;
  s.h = h; s.p = p; s.r = r; s.t = t; s.a2 = a2;
  return s;
}

// set2State(conserved) (conservationLaws/euler/transforms/conserved.ipp:31-76)
template <class R> State<R> cons2state(const Species<R>& sp, const R* qc) {
  State<R> s;
  const R r = qc[2], re = qc[3];
  const R r1 = 1. / r;
  s.u2 = 0;
  for (int i = 0; i < 2; ++i) s.u[i] = qc[i] * r1;
  for (int i = 0; i < 2; ++i) s.u2 += s.u[i] * s.u[i];
  const R k = 0.5 * s.u2;
  const R p = (sp.gamma - 1.) * (re - r * k);
  const R t = p / (sp.Rgas * r);
  const R a2 = sp.gamma * sp.Rgas * t;
  const R h = a2 * sp.gamma1 + k;
  s.p = p; s.r = r; s.t = t; s.h = h; s.a2 = a2;
  return s;
}

// state2Set<conserved> (conservationLaws/euler/transforms/conserved.ipp:2-29)
template <class R> void state2cons(const State<R>& s, R* qc) {
  const R re = s.r * s.h - s.p;
  for (int i = 0; i < 2; ++i) qc[i] = s.r * s.u[i];
  qc[2] = s.r; qc[3] = re;
}

// state2Set<primitive> (conservationLaws/euler/transforms/primitive.ipp:82-98)
template <class R> void state2prim(const State<R>& s, R* qp) {
  qp[0] = s.u[0]; qp[1] = s.u[1]; qp[2] = s.r; qp[3] = s.p;
}

template <class R> void prim2cons(const Species<R>& sp, const R* qp, R* qc) {
  state2cons(prim2state(sp, qp), qc);
}
template <class R> void cons2prim(const Species<R>& sp, const R* qc, R* qp) {
  state2prim(cons2state(sp, qc), qp);
}

// projectedVelocity (conservationLaws/base/base.h:148-158)
template <class R> R proj_vel(const R* n, const State<R>& s) {
  R un = 0;
  for (int i = 0; i < 2; ++i) un += n[i] * s.u[i];
  return un;
}

// spectralRadius (conservationLaws/euler/euler.h:161-166)
template <class R> R spec_rad(const R* n, const State<R>& s) {
  return abs(proj_vel(n, s)) + sqrt(s.a2);
}

// wavespeeds (conservationLaws/euler/euler.h:168-181)
template <class R> void wavespeeds(const R* n, const State<R>& s, R* w) {
  const R u = proj_vel(n, s);
  const R a = sqrt(s.a2);
  w[0] = u; w[1] = u - a; w[2] = u + a; w[3] = u;
}

// rotateToFace / rotateFromFace of the vector part (conservationLaws/base/base.h:171-232)
template <class R> void rotate_to(const Face<R>& f, const R* q0, R* q1) {
  const R* m[2] = {f.n, f.t};
  for (int k = 2; k < 4; ++k) q1[k] = q0[k];
  for (int i = 0; i < 2; ++i) {
    R a = 0;
    for (int j = 0; j < 2; ++j) a += m[i][j] * q0[j];
    q1[i] = a;
  }
}
template <class R> void rotate_from(const Face<R>& f, const R* q0, R* q1) {
  const R* m[2] = {f.n, f.t};
  for (int k = 2; k < 4; ++k) q1[k] = q0[k];
  for (int i = 0; i < 2; ++i) {
    R a = 0;
    for (int j = 0; j < 2; ++j) a += m[j][i] * q0[j];
    q1[i] = a;
  }
}

// delta2Delta conserved -> primitive (primitive.ipp:65-107)
template <class R> void dcons2dprim(const Species<R>& sp, const State<R>& s, const R* dqc, R* dqp) {
  const R dr = dqc[2], dre = dqc[3];
  const R rho1 = 1. / s.r;
  const R k = 0.5 * s.u2;
  R c = k * dr + dre;
  for (int i = 0; i < 2; ++i) {
    const R u = s.u[i], dru = dqc[i];
    const R du = (dru - u * dr) * rho1;
    dqp[i] = du;
    c -= u * dru;
  }
  const R dp = c * (sp.gamma - 1.);
  dqp[2] = dr; dqp[3] = dp;
}

// delta2Delta primitive -> conserved (primitive.ipp:110-156)
template <class R> void dprim2dcons(const Species<R>& sp, const State<R>& s, const R* dqp, R* dqc) {
  const R dr = dqp[2], dp = dqp[3];
  const R r = s.r;
  R dk = 0;
  for (int i = 0; i < 2; ++i) {
    const R u = s.u[i], du = dqp[i];
    const R dru = r * du + u * dr;
    dqc[i] = dru;
    dk += u * du;
  }
  const R k = 0.5 * s.u2;
  const R dre = dp * sp.gamma1 + r * dk + k * dr;
  dqc[2] = dr; dqc[3] = dre;
}

// delta2Delta characteristic -> primitive (characteristic.ipp:5-41)
template <class R> void dchar2dprim(const Species<R>& sp, const State<R>& s, const R* dqw, R* dqp) {
  const R r = s.r;
  const R a = sqrt(s.a2);
  const R dp = 0.5 * r * a * (dqw[2] - dqw[1]);
  const R dr = dp / (a * a) - r * dqw[0] / sp.gamma;
  dqp[0] = 0.5 * (dqw[1] + dqw[2]);
  dqp[1] = dqw[3];
  dqp[2] = dr; dqp[3] = dp;
}

// delta2Delta primitive -> characteristic (characteristic.ipp:44-79)
template <class R> void dprim2dchar(const Species<R>& sp, const State<R>& s, const R* dqp, R* dqw) {
  const R r1 = 1. / s.r;
  const R a1 = 1. / sqrt(s.a2);
  const R du = dqp[0], dr = dqp[2], dp = dqp[3];
  dqw[0] = sp.gamma * (dp * a1 * a1 - dr) * r1;
  dqw[1] = du - dp * r1 * a1;
  dqw[2] = du + dp * r1 * a1;
  dqw[3] = dqp[1];
}

// ---------------------------------------------------------------- fluxes
// exactFlux (conservationLaws/euler/fluxes/exactFlux.ipp:4-36)
template <class R> FluxRes<R> exact_flux(const R* n, const State<R>& s) {
  const R r = s.r, p = s.p, h = s.h;
  const R a = sqrt(s.a2);
  const R un = proj_vel(n, s);
  const R mn = r * un;
  FluxRes<R> fr;
  for (int i = 0; i < 2; ++i) fr.f[i] = mn * s.u[i] + p * n[i];
  fr.f[2] = mn; fr.f[3] = mn * h;
  fr.lam = abs(un) + a;
  return fr;
}

// CentralFlux (conservationLaws/base/fluxes/centralFlux.ipp:2-14)
template <class R> FluxRes<R> central_flux(const Face<R>& f, const State<R>& sl, const State<R>& sr) {
  const FluxRes<R> fl = exact_flux(f.n, sl), fr = exact_flux(f.n, sr);
  FluxRes<R> o;
  for (int i = 0; i < 4; ++i) o.f[i] = (R)(0.5 * (fl.f[i] + fr.f[i])) * f.area;
  o.lam = std::max(fl.lam, fr.lam) * f.area;
  return o;
}

// roeAverage (conservationLaws/euler/fluxes/roe.ipp:2-48)
template <class R> State<R> roe_average(const Species<R>& sp, const State<R>& sl, const State<R>& sr) {
  State<R> a;
  const R cr = sqrt(sr.r / sl.r);
  const R wl = 1. / (1. + cr);
  const R wr = 1. - wl;
  const R ra = cr * sl.r;
  R ka = 0;
  for (int i = 0; i < 2; ++i) {
    const R ua = wl * sl.u[i] + wr * sr.u[i];
    ka += ua * ua;
    a.u[i] = ua;
  }
  ka *= 0.5;
  const R ha = wl * sl.h + wr * sr.h;
  const R a2a = (sp.gamma - 1.) * (ha - ka);
  const R ta = a2a / (sp.Rgas * sp.gamma);
  const R pa = ra * sp.Rgas * ta;
  a.p = pa; a.r = ra; a.t = ta; a.h = ha; a.u2 = 2. * ka; a.a2 = a2a;
  return a;
}

// entropyfix, Harten eps=0.05 (conservationLaws/euler/fluxes/roe.ipp:50-78)
template <class R> void entropy_fix(const R* la, const R* ll, const R* lr, R* sp) {
  const R ua = fabs(la[0]);
  sp[0] = ua; sp[3] = ua;
  sp[1] = fabs(la[1]); sp[2] = fabs(la[2]);
  constexpr R eps = 0.05;
  for (int i = 1; i < 3; ++i) {
    const R le = eps * fmax((R)0., fmax(la[i] - ll[i], lr[i] - la[i]));
    const R laa = fabs(la[i]);
    sp[i] = (laa > le) ? laa : (R)(0.5 * (le + laa * laa / le));
  }
}

// RoeDissipation (conservationLaws/base/fluxes/roeFlux.ipp:22-58)
// face_frame = false is RoeDissipation as written: the jump is rotated to the face frame
// while the Roe-averaged state keeps its global-frame velocity, which is the Roe matrix's
// dissipation only for the face normal (1, 0).  face_frame = true (FLUX_ROE_FACE, not in
// the reference) takes the averaged velocity into the face frame too, which makes the flux
// invariant under rotation and equal to the literal one for the normal (1, 0).
template <class R> FluxRes<R> roe_dissipation(const Species<R>& sp, const Face<R>& f,
                                              const State<R>& sl, const State<R>& sr,
                                              bool face_frame = false) {
  const State<R> ra = roe_average(sp, sl, sr);
  R wa[4], wl[4], wr[4], lam[4];
  wavespeeds(f.n, ra, wa); wavespeeds(f.n, sl, wl); wavespeeds(f.n, sr, wr);
  entropy_fix(wa, wl, wr, lam);
  R cl[4], cr[4], dq[4], dqc[4];
  state2cons(sr, cr); state2cons(sl, cl);
  for (int i = 0; i < 4; ++i) dq[i] = cr[i] - cl[i];
  rotate_to(f, dq, dqc);
  R dqp[4], dqw[4];
  // face_frame: the averaged state's velocity in the frame of the jump, {n.u, t.u}
  State<R> rf = ra;
  if (face_frame) {
    R u[4] = {ra.u[0], ra.u[1], 0, 0}, uf[4];
    rotate_to(f, u, uf);
    rf.u[0] = uf[0]; rf.u[1] = uf[1];
  }
  dcons2dprim(sp, rf, dqc, dqp);
  dprim2dchar(sp, rf, dqp, dqw);
  for (int i = 0; i < 4; ++i) dqw[i] = lam[i] * dqw[i];
  R dp2[4], dc2[4], fd[4];
  dchar2dprim(sp, rf, dqw, dp2);
  dprim2dcons(sp, rf, dp2, dc2);
  rotate_from(f, dc2, fd);
  FluxRes<R> o;
  const R s = -0.5 * f.area;
  for (int i = 0; i < 4; ++i) o.f[i] = s * fd[i];
  o.lam = spec_rad(f.n, ra) * f.area;
  return o;
}

// RoeFlux = Central + RoeDissipation (conservationLaws/base/fluxes/roeFlux.ipp:2-19)
template <class R> FluxRes<R> roe_flux(const Species<R>& sp, const Face<R>& f,
                                       const State<R>& sl, const State<R>& sr, bool face_frame = false) {
  const FluxRes<R> c = central_flux(f, sl, sr);
  const FluxRes<R> d = roe_dissipation(sp, f, sl, sr, face_frame);
  FluxRes<R> o;
  for (int i = 0; i < 4; ++i) o.f[i] = c.f[i] + d.f[i];
  o.lam = fmax(c.lam, d.lam);
  return o;
}

// RusanovFlux (conservationLaws/base/fluxes/rusanovFlux.ipp:2-50)
template <class R> FluxRes<R> rusanov_flux(const Species<R>& sp, const Face<R>& f,
                                           const State<R>& sl, const State<R>& sr) {
  FluxRes<R> o = central_flux(f, sl, sr);
  const R lambda = std::max(spec_rad(f.n, sl), spec_rad(f.n, sr));
  R cl[4], cr[4];
  state2cons(sr, cr); state2cons(sl, cl);
  const R la = lambda * f.area;
  const R s = -0.5 * la;
  for (int i = 0; i < 4; ++i) o.f[i] += s * (cr[i] - cl[i]);
  (void)sp;
  return o;
}

// Mach-number splittings (conservationLaws/euler/fluxes/machSplittings.ipp:8-43)
template <class R> R msplit_m1(int s, R M) { return 0.5 * (M + s * fabs(M)); }
template <class R> R msplit_m2(int s, R M) { return s * 0.25 * (M + s) * (M + s); }
template <class R> R msplit_m4(int s, R M, R beta) {
  return msplit_m2(s, M) * (1. - s * 16. * beta * msplit_m2(-s, M));
}
// as written: (M1 + eps)/(|M| + eps), eps the largest value (1 for both signs); with
// FIX_MACH_SPLIT_P1: (s M1 + eps)/(|M| + eps), eps the smallest normal value, i.e. M1/M
template <class R> R msplit_p1(int s, R M, unsigned fixes) {
  const bool fix = (fixes & FIX_MACH_SPLIT_P1) != 0u;
  const R eps = fix ? std::numeric_limits<R>::min() : std::numeric_limits<R>::max();
  const R m1 = msplit_m1(s, M);
  return ((fix ? R(s * m1) : m1) + eps) / (fabs(M) + eps);
}
template <class R> R msplit_p3(int s, R M) { return msplit_m2(s, M) * (s * 2. - M); }
template <class R> R msplit_p5(int s, R M, R alpha) {
  return msplit_p3(s, M) - s * 16. * alpha * M * msplit_m2(s, M) * msplit_m2(-s, M);
}

// SLAU2 with (Convective, Acoustic) low-Mach tags
// (conservationLaws/euler/fluxes/slau.ipp:4-161).  upwind_by_mdot=false is the
// literal reference form that selects the convected state by the sign of
// ua = sqrt(0.5(|u_l|^2+|u_r|^2)) (slau.ipp:124-125), which is never negative;
// upwind_by_mdot=true selects it by the sign of the interface mass flux.
template <class R> FluxRes<R> slau_flux(const Species<R>& sp, const Face<R>& f,
                                        const State<R>& sl, const State<R>& sr, bool upwind_by_mdot) {
  const R ua = sqrt(0.5 * (sl.u2 + sr.u2));
  const R aa = 0.5 * (sqrt(sl.a2) + sqrt(sr.a2));
  const R aa1 = 1.0 / aa;
  const R ma = ua * aa1;
  const R ma_hat = fmin((R)1.0, ma);
  const R unl = proj_vel(f.n, sl), unr = proj_vel(f.n, sr);
  const R ml = unl * aa1, mr = unr * aa1;
  const R una = (sl.r * fabs(unl) + sr.r * fabs(unr)) / (sl.r + sr.r);
  const R chi = (1. - ma_hat) * (1. - ma_hat);
  const R g = -fmax(fmin(ml, (R)0.), (R)-1.) * fmin(fmax(mr, (R)0.), (R)1.);
  const R dr = sr.r - sl.r;
  const R dp = sr.p - sl.p;
  const R mdot_c = sl.r * unl + sr.r * unr;
  const R mdot_dr = una * dr;
  const R mdot_dp = chi * dp * aa1;
  const R mdot = 0.5 * ((mdot_c - mdot_dr) * (1. - g) - mdot_dp) * f.area;
  const unsigned mlsup = fabs(ml) > 1 ? 1 : 0, mlsub = 1 - mlsup;
  const unsigned mrsup = fabs(mr) > 1 ? 1 : 0, mrsub = 1 - mrsup;
  const R betal = mlsub * msplit_p3(1, ml) + mlsup * msplit_p1(1, ml, sp.fixes);
  const R betar = mrsub * msplit_p3(-1, mr) + mrsup * msplit_p1(-1, mr, sp.fixes);
  const R p_c = sl.p + sr.p;
  const R p_dp = (betal - betar) * dp;
  const R p_du = -ma * (betal + betar - 1.) * (p_c);
  const R pa = 0.5 * (p_c - p_dp - p_du) * f.area;
  const bool left = upwind_by_mdot ? (mdot > 0) : (ua > 0);
  const int m1l = left ? 1 : 0, m1r = left ? 0 : 1;
  FluxRes<R> o;
  for (int i = 0; i < 2; ++i) o.f[i] = mdot * (m1l * sl.u[i] + m1r * sr.u[i]) + pa * f.n[i];
  o.f[2] = mdot;
  o.f[3] = mdot * (m1l * sl.h + m1r * sr.h);
  const R lmax = sqrt(fmax(sl.a2, sr.a2)) + fmax(fabs(unl), fabs(unr));
  o.lam = lmax * f.area;
  return o;
}

// AUSM+up, Liou 2006: AusmPlusUP<VFluxScaling, PFluxScaling>
// (conservationLaws/euler/fluxes/ausmPlusUP.ipp:6-171); vscale / pscale select the template
// arguments (SCALING_*).  The acoustic-to-step time-scale ratio lref / (as dt) of the adaptive
// scaling reads the species' dt, which the reference leaves at its largest value
// (conservationLaws/euler/species.ipp:12) unless a caller sets it.
template <class R> FluxRes<R> ausmpup_flux(const Species<R>& sp, const Face<R>& f,
                                           const State<R>& sl, const State<R>& sr,
                                           int vscale = SCALING_CONVECTIVE, int pscale = SCALING_CONVECTIVE) {
  const R alpha0 = 0.1875, beta = 0.125, Ku = 0.75 * 2., Kp = 0.25, sigma = 1.0;
  const R ascoeff = 2. * (sp.gamma - 1.) / (sp.gamma + 1.);
  const R unl = proj_vel(f.n, sl), unr = proj_vel(f.n, sr);
  const R als2 = ascoeff * sl.h, ars2 = ascoeff * sr.h;
  const R als = als2 / fmax(unl, sqrt(als2));
  const R ars = ars2 / fmax(-unr, sqrt(ars2));
  const R ra = 0.5 * (sl.r + sr.r);
  const R as = fmin(ars, als);
  const R ml = unl / as, mr = unr / as;
  const R minf = sp.minf;
  const R m0 = sqrt(0.5 * (ml * ml + mr * mr));
  const R mu = sp.lref / (as * sp.dt);
  const R m0_c = std::clamp<R>(m0, minf, 1.);
  const R m0_a = std::clamp<R>(fmax(m0, mu), minf, 1.);
  auto pick = [&](int k) -> R { return k == SCALING_CONVECTIVE ? m0_c : (k == SCALING_ACOUSTIC ? R(1.0) : m0_a); };
  const R m0_p = pick(pscale), m0_u = pick(vscale);
  const R fa_p = m0_p * (2. - m0_p);
  const R fa_u = m0_u * (2. - m0_u);
  const unsigned mlsup = fabs(ml) > 1 ? 1 : 0, mlsub = 1 - mlsup;
  const unsigned mrsup = fabs(mr) > 1 ? 1 : 0, mrsub = 1 - mrsup;
  const R mlp = mlsub * msplit_m4(1, ml, beta) + mlsup * msplit_m1(1, ml);
  const R mrm = mrsub * msplit_m4(-1, mr, beta) + mrsup * msplit_m1(-1, mr);
  const R delp = sr.p - sl.p;
  const R mp = Kp * fmax(1. - sigma * m0 * m0, (R)0.) * delp / (fa_p * ra * as * as);
  const R uaf = as * (mlp + mrm - mp) * f.area;
  const R alpha = alpha0 * (5. * fa_u * fa_u - 4.);
  const R plp = mlsub * msplit_p5(1, ml, alpha) + mlsup * msplit_p1(1, ml, sp.fixes);
  const R prm = mrsub * msplit_p5(-1, mr, alpha) + mrsup * msplit_p1(-1, mr, sp.fixes);
  const R delu = unr - unl;
  const R pu = Ku * plp * prm * ra * (fa_u * as) * delu;
  const R pa = (plp * sl.p + prm * sr.p - pu) * f.area;
  const int m1l = (uaf > 0) ? 1 : 0, m1r = (uaf > 0) ? 0 : 1;
  const R mdot = uaf * (m1l * sl.r + m1r * sr.r);
  FluxRes<R> o;
  for (int i = 0; i < 2; ++i) o.f[i] = mdot * (m1l * sl.u[i] + m1r * sr.u[i]) + pa * f.n[i];
  o.f[2] = mdot;
  o.f[3] = mdot * (m1l * sl.h + m1r * sr.h);
  const R lmd = 0.5 * (m0_p + 1) / fa_p;
  const R amax = sqrt(fmax(as * as, fmax(sl.a2, sr.a2)));
  const R lmax = lmd * amax + fmax(fabs(uaf), fmax(fabs(unl), fabs(unr)));
  o.lam = lmax * f.area;
  return o;
}

// RoeUnprecWS (conservationLaws/euler/fluxes/roeUnprecWS.ipp:2-109): central flux minus a
// Weiss & Smith / Li & Gu scalar dissipation scaled by the cut-off Mach number
template <class R> FluxRes<R> roe_ws_flux(const Species<R>& sp, const Face<R>& f,
                                          const State<R>& sl, const State<R>& sr) {
  const State<R> ravg = roe_average(sp, sl, sr);
  const FluxRes<R> central = central_flux(f, sl, sr);
  const R dp = sr.p - sl.p;
  const R du = proj_vel(f.n, sr) - proj_vel(f.n, sl);
  const R una = proj_vel(f.n, ravg);
  const R ra = ravg.r;
  const R aa = sqrt(ravg.a2);
  const R minf = sp.minf;
  const R uinf = minf * aa;
  R ql[4], qr[4], dqc[4];
  state2cons(sl, ql);
  state2cons(sr, qr);
  for (int v = 0; v < 4; ++v) dqc[v] = qr[v] - ql[v];
  const int A11 = 1, A12 = 0, A21 = 1, A22 = 1;
  const R nu_p = 1.00 * (1. / (ra * uinf * uinf)) * pow(minf, R(A11));
  const R nu_u = 0.05 * pow(minf, R(A12));
  const R mu_p = 0.02 * pow(minf, R(A21));
  const R mu_u = 0.10 * (ra * uinf) * pow(minf, R(A22));
  const R deltaU = nu_p * dp + nu_u * du;
  const R ruvh[4] = {ra * ravg.u[0], ra * ravg.u[1], ra, ra * ravg.h};
  const R deltaP = mu_p * dp + mu_u * du;
  const R onu[4] = {f.n[0], f.n[1], R(0.), una};
  FluxRes<R> o;
  for (int v = 0; v < 4; ++v) {
    const R d = 0.5 * ((fabs(una) * dqc[v] + deltaU * ruvh[v]) + deltaP * onu[v]) * f.area;
    o.f[v] = central.f[v] - d;
  }
  const R dlam = spec_rad(f.n, ravg) * f.area * pow(minf, R(A11 - 1));
  o.lam = fmax(central.lam, dlam);
  return o;
}

template <class R> FluxRes<R> face_flux(int kind, const Species<R>& sp, const Face<R>& f,
                                        const State<R>& sl, const State<R>& sr,
                                        int vscale = SCALING_CONVECTIVE, int pscale = SCALING_CONVECTIVE) {
  switch (kind) {
    case FLUX_ROE: return roe_flux(sp, f, sl, sr);
    case FLUX_ROE_FACE: return roe_flux(sp, f, sl, sr, true);
    case FLUX_SLAU: return slau_flux(sp, f, sl, sr, true);
    case FLUX_SLAU_REF: return slau_flux(sp, f, sl, sr, false);
    case FLUX_AUSMPUP: return ausmpup_flux(sp, f, sl, sr, vscale, pscale);
    case FLUX_RUSANOV: return rusanov_flux(sp, f, sl, sr);
    case FLUX_ROE_WS: return roe_ws_flux(sp, f, sl, sr);
    default: return central_flux(f, sl, sr);
  }
}

// ---------------------------------------------------------------- limiters
// limiters/limiter.ipp:8-161.  VANLEER is the textbook harmonic-mean slope
// (a|b|+|a|b)/(|a|+|b|+eps) with the reference's eps convention; VANLEER_REF
// is the literal reference expression (b+|b|)/(a+|b|+eps) (limiter.ipp:81-89).
template <class R> R limit(int kind, R a, R b) {
  switch (kind) {
    case LIM_NOLIMIT1: return 0;
    case LIM_NOLIMIT2: return 0.5 * (a + b);
    case LIM_NOLIMIT3: return 0.33333333333333333 * (2. * a + b);
    case LIM_VANALBADA: {
      const R eps = std::numeric_limits<R>::min();
      return a * b < 0 ? (R)0 : (b * (a * a) + a * (b * b)) / (a * a + b * b + eps);
    }
    case LIM_MINMOD:
      return a > 0 ? (R)fmin(a, (R)fmax(b, (R)0.)) : (R)fmax(a, (R)fmin(b, (R)0.));
    case LIM_SUPERBEE:
      return a > 0 ? (R)fmax((R)0., fmax(fmin(2 * a, b), fmin(2 * b, a)))
                   : (R)fmin((R)0., fmin(fmax(2 * a, b), fmax(2 * b, a)));
    case LIM_MC:
      return a > 0 ? (R)fmax((R)0., fmin((R)(0.5 * (a + b)), fmin(2 * b, 2 * a)))
                   : (R)fmin((R)0., fmax((R)(0.5 * (a + b)), fmax(2 * b, 2 * a)));
    case LIM_VANLEER: {
      const R eps = std::numeric_limits<R>::min();
      return (a * fabs(b) + fabs(a) * b) / (fabs(a) + fabs(b) + eps);
    }
    case LIM_VANLEER_REF: {
      const R eps = std::numeric_limits<R>::min();
      return (b + fabs(b)) / (a + fabs(b) + eps);
    }
    case LIM_CADA3: {
      const R t = 0.0, gam = 1.5, c1 = -2. / 7., c2 = 0.4, c3 = 3 * gam - 2;
      R u, v, w, p, q;
      if (a > 0) { u = a; v = b; } else { u = -a; v = -b; }
      p = (v + 2. * u) / 3.;
      q = fabs(a) + fabs(b);
      if (q > t) {
        if (v < -2 * u) w = 0;
        else if (v < c1 * u) w = (v + 2. * u) / 3.;
        else if (v < 0) w = -2. * v;
        else if (v < c2 * u) w = 2. * v;
        else if (v < c3 * u) w = (v + 2. * u) / 3.;
        else w = gam * u;
      } else {
        w = p;
      }
      if (a <= 0) w = -w;
      return w;
    }
    default: return 0;
  }
}

// ---------------------------------------------------------------- LSQ
// lsq::xmetric (lsq/xmetric.ipp:53-69), lsq::qmetric (lsq/qmetric.ipp:48-70),
// lsq::factor (lsq/factor_solve.ipp:13-22), lsq::solve (lsq/factor_solve.ipp:47-69).
// QMetric index is q[2*var+dim] (the intent of lsq/lsq.h:72).
template <class R> struct XM { R x[3]; };
template <class R> struct QM { R q[8]; };

template <class R> XM<R> xmetric(R dx, R dy) { return XM<R>{{dx * dx, dx * dy, dy * dy}}; }
template <class R> QM<R> qmetric(R dx, R dy, const R* dq) {
  QM<R> m;
  for (int i = 0; i < 4; ++i) { m.q[2 * i] = dq[i] * dx; m.q[2 * i + 1] = dq[i] * dy; }
  return m;
}
template <class R> XM<R> factor(const XM<R>& xm) {
  const R d = 1. / (xm.x[0] * xm.x[2] - xm.x[1] * xm.x[1]);
  return XM<R>{{d * xm.x[2], -d * xm.x[1], d * xm.x[0]}};
}
template <class R> void solve(const XM<R>& xf, const QM<R>& qm, const R* dir, R* g) {
  for (int i = 0; i < 4; ++i)
    g[i] = (xf.x[0] * qm.q[2 * i] + xf.x[1] * qm.q[2 * i + 1]) * dir[0] +
           (xf.x[1] * qm.q[2 * i] + xf.x[2] * qm.q[2 * i + 1]) * dir[1];
}

// ---------------------------------------------------------------- RK tables
// ODE::Explicit ssp11/ssp22/ssp33/ssp34 (ode.h:107-197)
template <class R> struct RKTable { int nstages; R maxcfl; R alpha[4][4]; R beta[4]; };
template <class R> RKTable<R> rk_table(int kind) {
  RKTable<R> t{};
  if (kind == RK_SSP11) { t.nstages = 1; t.maxcfl = 1.; t.beta[0] = 1.0; t.alpha[0][0] = 1.0; }
  else if (kind == RK_SSP22) {
    t.nstages = 2; t.maxcfl = 1.; t.beta[0] = 1.0; t.beta[1] = 1.0;
    t.alpha[0][0] = 1.0; t.alpha[1][0] = 0.5; t.alpha[1][1] = 0.5;
  } else if (kind == RK_SSP33) {
    t.nstages = 3; t.maxcfl = 1.; t.beta[0] = 1.0; t.beta[1] = 0.5; t.beta[2] = 1.0;
    t.alpha[0][0] = 1.; t.alpha[1][0] = 0.5; t.alpha[1][1] = 0.5;
    t.alpha[2][0] = 1. / 6.; t.alpha[2][1] = 1. / 6.; t.alpha[2][2] = 2. / 3.;
  } else {
    t.nstages = 4; t.maxcfl = 2.; t.beta[0] = 0.5; t.beta[1] = 1.0; t.beta[2] = 0.5; t.beta[3] = 1.0;
    t.alpha[0][0] = 1.0; t.alpha[1][0] = 0.5; t.alpha[1][1] = 0.5;
    t.alpha[2][0] = 1. / 3.; t.alpha[2][1] = 1. / 3.; t.alpha[2][2] = 1. / 3.;
    t.alpha[3][0] = 1. / 6.; t.alpha[3][1] = 1. / 6.; t.alpha[3][2] = 1. / 6.; t.alpha[3][3] = 1. / 2.;
  }
  return t;
}

// ---------------------------------------------------------------- branch signatures
// Which branches one face's evaluation takes, with the same codes as the CUDA path's
// recording kernels (limit_piece, flux_bits there): the parity report compares the two
// per face.  limit_piece: bit 3 = (a > 0), bits 0-2 the interval of b/a (by
// multiplication, u = |a|, v = b signed like a) that selects the limiter's expression.
template <class R> unsigned limit_piece(int kind, R a, R b) {
  const bool pos = a > 0;
  const R u = pos ? a : -a, v = pos ? b : -b;
  unsigned p = 0;
  switch (kind) {
    case LIM_VANALBADA: p = (a * b < 0) ? 0u : 1u; break;
    case LIM_VANLEER: p = (a * b > 0) ? 1u : 0u; break;
    case LIM_MINMOD: p = (v <= 0) ? 0u : (v < u ? 1u : 2u); break;
    case LIM_SUPERBEE: p = (v <= 0) ? 0u : (2 * v < u ? 1u : (v < u ? 2u : (v < 2 * u ? 3u : 4u))); break;
    case LIM_MC: p = (v <= 0) ? 0u : (3 * v < u ? 1u : (v < 3 * u ? 2u : 3u)); break;
    case LIM_CADA3: {
      const R c1 = -2. / 7., c2 = 0.4, c3 = 3 * 1.5 - 2;
      if (!(fabs(a) + fabs(b) > 0)) p = 7u;
      else if (v < -2 * u) p = 1u;
      else if (v < c1 * u) p = 2u;
      else if (v < 0) p = 3u;
      else if (v < c2 * u) p = 4u;
      else if (v < c3 * u) p = 5u;
      else p = 6u;
      break;
    }
    default: return 0u;
  }
  return p | (pos ? 8u : 0u);
}

// flux branches of two face states, with the reference's expressions: Roe -- Harten's
// fix on waves 1 and 2 (roe.ipp:50-78); SLAU -- |M_L| > 1, |M_R| > 1, mean-speed Mach
// > 1 (slau.ipp:18-31); AUSM+up -- |M_L| > 1, |M_R| > 1, left critical speed below the
// right (ausmPlusUP.ipp:30-55); others -- right spectral radius larger
template <class R> unsigned flux_bits(int kind, const Species<R>& sp, const Face<R>& f, const State<R>& sl,
                                      const State<R>& sr) {
  const R unl = proj_vel(f.n, sl), unr = proj_vel(f.n, sr);
  if (kind == FLUX_ROE || kind == FLUX_ROE_FACE) {
    const State<R> ra = roe_average(sp, sl, sr);
    R wa[4], wl[4], wr[4];
    wavespeeds(f.n, ra, wa); wavespeeds(f.n, sl, wl); wavespeeds(f.n, sr, wr);
    unsigned b = 0;
    for (int i = 1; i < 3; ++i) {
      const R le = 0.05 * fmax((R)0., fmax(wa[i] - wl[i], wr[i] - wa[i]));
      if (!(fabs(wa[i]) > le)) b |= 1u << (i - 1);
    }
    return b;
  }
  if (kind == FLUX_SLAU || kind == FLUX_SLAU_REF) {
    const R ua = sqrt(0.5 * (sl.u2 + sr.u2));
    const R aa = 0.5 * (sqrt(sl.a2) + sqrt(sr.a2));
    const R aa1 = 1.0 / aa;
    const R ml = unl * aa1, mr = unr * aa1;
    return (fabs(ml) > 1 ? 1u : 0u) | (fabs(mr) > 1 ? 2u : 0u) | (ua * aa1 > 1 ? 4u : 0u);
  }
  if (kind == FLUX_AUSMPUP) {
    const R ascoeff = 2. * (sp.gamma - 1.) / (sp.gamma + 1.);
    const R als2 = ascoeff * sl.h, ars2 = ascoeff * sr.h;
    const R als = als2 / fmax(unl, sqrt(als2));
    const R ars = ars2 / fmax(-unr, sqrt(ars2));
    const R as = fmin(ars, als);
    const R ml = unl / as, mr = unr / as;
    return (fabs(ml) > 1 ? 1u : 0u) | (fabs(mr) > 1 ? 2u : 0u) | (als < ars ? 4u : 0u);
  }
  return spec_rad(f.n, sr) > spec_rad(f.n, sl) ? 1u : 0u;
}
enum : unsigned { SIG_FLUX_SHIFT = 32, SIG_BC_SHIFT = 36, SIG_VALID_SHIFT = 63 };

// ---------------------------------------------------------------- solution basis
// The basis of the solution field (the SolVarT of SolutionField<SolVarT,2>): primitive
// {u, v, rho, p}, as in the reference drivers (cylinder2D.cpp:110, gresho2D.cpp:112), or
// conserved {rho u, rho v, rho, rho E}; the residual glue, boundary updates and fluxes are
// generic over it and reach the State through set2State of the basis.
enum Basis { BASIS_PRIMITIVE = 0, BASIS_CONSERVED = 1 };
template <class R> State<R> basis2state(const Species<R>& sp, const R* q, int basis) {
  return basis == BASIS_CONSERVED ? cons2state(sp, q) : prim2state(sp, q);
}

// ---------------------------------------------------------------- boundary physics
// boundaryUpdate for Riemann invariants (conservationLaws/euler/boundary/riemann.ipp:18-113),
// entropy/pressure (entropy.ipp:18-88); qi/qf/qb in the solution basis, face normal into the domain.
// The subsonic result is built as a primitive set in the face frame, converted to the
// basis (set2Set) and rotated back, as the reference composes it.
template <class R> void basis_from_face(const Species<R>& sp, const Face<R>& f, const R* qbr, R* qb, int basis) {
  if (basis == BASIS_CONSERVED) {
    R c[4];
    prim2cons(sp, qbr, c);
    rotate_from(f, c, qb);
  } else {
    rotate_from(f, qbr, qb);
  }
}
template <class R>
void bc_riemann(const Species<R>& sp, const Face<R>& f, const R* qi, const R* qf, R* qb, int basis = BASIS_PRIMITIVE,
                unsigned* path = nullptr) {
  const R gam = sp.gamma, gam1 = sp.gamma1;
  R ri[4], rf[4];
  rotate_to(f, qi, ri); rotate_to(f, qf, rf);
  const State<R> sA = roe_average(sp, basis2state(sp, ri, basis), basis2state(sp, rf, basis));
  const R cosn = sA.u[0] / sqrt(sA.u2);
  if (((sp.fixes & FIX_FARFIELD_TRANSVERSE) ? R(fabs(cosn)) : cosn) < 0.001) {
    for (int k = 0; k < 4; ++k) qb[k] = qi[k];
    if (path) *path = 1u;
    return;
  }
  const R ma = sA.u[0] / sqrt(sA.a2);
  const bool inflow = ma > 0;
  const R* quw = inflow ? qf : qi;
  if (abs(ma) > 1.) { for (int k = 0; k < 4; ++k) qb[k] = quw[k]; if (path) *path = 2u; return; }
  if (path) *path = 3u;
  const State<R> sI = basis2state(sp, ri, basis), sF = basis2state(sp, rf, basis);
  const R ai = sqrt(sI.a2), af = sqrt(sF.a2);
  const R uni = sI.u[0], unf = sF.u[0];
  const R rim = uni - 2. * ai * gam1;
  const R rip = unf + 2. * af * gam1;
  const R ub = 0.5 * (rim + rip);
  const R ab = 0.25 * (gam - 1.) * (rip - rim);
  R ru[4];
  rotate_to(f, quw, ru);
  const State<R> sU = basis2state(sp, ru, basis);
  const R sb = sU.a2 / (gam * pow(sU.r, gam - 1.));
  const R vb = sU.u[1];
  const R rb = pow(ab * ab / (gam * sb), gam1);
  const R pb = rb * ab * ab / gam;
  const R qbr[4] = {ub, vb, rb, pb};
  basis_from_face(sp, f, qbr, qb, basis);
}

template <class R>
void bc_entropy(const Species<R>& sp, const Face<R>& f, const R* qi, const R* qf, R* qb, int basis = BASIS_PRIMITIVE,
                unsigned* path = nullptr) {
  const R gam = sp.gamma;
  R ri[4], rf[4];
  rotate_to(f, qi, ri); rotate_to(f, qf, rf);
  const State<R> sA = roe_average(sp, basis2state(sp, ri, basis), basis2state(sp, rf, basis));
  const R cosn = sA.u[0] / sqrt(sA.u2);
  if (((sp.fixes & FIX_FARFIELD_TRANSVERSE) ? R(fabs(cosn)) : cosn) < 0.0001) {
    for (int k = 0; k < 4; ++k) qb[k] = qi[k];
    if (path) *path = 1u;
    return;
  }
  const R ma = sA.u[0] / sqrt(sA.a2);
  const bool inflow = ma > 0;
  const R* quw = inflow ? qf : qi;
  const R* qdw = inflow ? qi : qf;
  if (abs(ma) > 1.) { for (int k = 0; k < 4; ++k) qb[k] = quw[k]; if (path) *path = 2u; return; }
  if (path) *path = 3u;
  R ru[4], rd[4];
  rotate_to(f, quw, ru); rotate_to(f, qdw, rd);
  const State<R> sU = basis2state(sp, ru, basis), sD = basis2state(sp, rd, basis);
  const R pb = sD.p;
  const R sb = sU.a2 / (gam * pow(sU.r, gam - 1.));
  const R rb = pow(pb / sb, 1. / gam);
  const R qbr[4] = {sU.u[0], sU.u[1], rb, pb};
  basis_from_face(sp, f, qbr, qb, basis);
}

// boundaryFlux for an inviscid wall (conservationLaws/euler/boundary/inviscidWall.ipp:33-72):
// pressure-only flux from q_wall = q_interior - dq, dq the gradient increment
// from the face to the cell centre.
template <class R>
FluxRes<R> wall_flux(const Species<R>& sp, const Face<R>& f, const R* qi, const R* dq, int basis = BASIS_PRIMITIVE) {
  const int direction = -1;
  R qw[4];
  for (int k = 0; k < 4; ++k) qw[k] = qi[k] + direction * dq[k];
  const State<R> sw = basis2state(sp, qw, basis);
  const R pw = sw.p;
  FluxRes<R> o;
  for (int i = 0; i < 2; ++i) o.f[i] = f.area * pw * f.n[i];
  o.f[2] = 0.; o.f[3] = 0.;
  o.lam = f.area * spec_rad(f.n, sw);
  return o;
}

}  // namespace hco
