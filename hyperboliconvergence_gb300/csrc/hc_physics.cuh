// hc_physics.cuh -- device pointwise physics for the 2D Euler residual path.
//
// Every function is templated on the arithmetic type R (double or float) and
// keeps all constants in R, so the FP32 path never touches the FP64 pipe.
// Formulas follow the reference solver (lacrymose/hyperboliConvergence,
// cpp/inc); each function names the file:line it follows.  Variable order:
// primitive {u, v, rho, p}, conserved {rho u, rho v, rho, rho E}
// (conservationLaws/euler/euler.h:19-25).
#pragma once

#include <cuda_runtime.h>
#include <cfloat>
#include <cstring>
#include <type_traits>

#include "hc_df64.cuh"

namespace hc {

enum FluxKind { FLUX_ROE = 0, FLUX_SLAU = 1, FLUX_SLAU_REF = 2, FLUX_AUSMPUP = 3,
                FLUX_RUSANOV = 4, FLUX_CENTRAL = 5, FLUX_ROE_WS = 6, FLUX_ROE_FACE = 7, FLUX_COUNT = 8 };
// LowMachScaling (conservationLaws/euler/euler.h:331-339) of AUSM+up's two diffusion terms
enum LowMachScaling { SCALING_CONVECTIVE = 0, SCALING_ACOUSTIC = 1, SCALING_ADAPTIVE = 2 };
enum LimiterKind { LIM_NOLIMIT1 = 0, LIM_NOLIMIT2 = 1, LIM_NOLIMIT3 = 2, LIM_VANALBADA = 3,
                   LIM_MINMOD = 4, LIM_SUPERBEE = 5, LIM_MC = 6, LIM_VANLEER = 7,
                   LIM_VANLEER_REF = 8, LIM_CADA3 = 9, LIM_COUNT = 10 };
enum BcKind { BC_PERIODIC = 0, BC_FIXED = 1, BC_RIEMANN = 2, BC_ENTROPY = 3, BC_WALL = 4 };

// a / b in the stage arithmetic.  FP32 on the device: the approximate quotient
// (__fdividef: within 2 ulp for |b| in [2^-126, 2^126]); the FP32 stage kernels are
// bound by instruction issue, and the correctly rounded division costs a sequence of
// instructions with a slow path (measured: 19% of the FP32 stage).  Used where the
// divisor is a density, a limiter denominator (at least the smallest normal value), an
// averaged sound speed or a volume.  FP64 and double-float keep exact division, so the
// FP64 results are unchanged.
template <class R> __host__ __device__ __forceinline__ R qdiv(R a, R b) { return a / b; }
template <> __host__ __device__ __forceinline__ float qdiv<float>(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fdividef(a, b);
#else
  return a / b;
#endif
}

template <class R> struct Lim;
template <> struct Lim<double> {
  __host__ __device__ static constexpr double tiny() { return DBL_MIN; }
  __host__ __device__ static constexpr double huge() { return DBL_MAX; }
};
template <> struct Lim<float> {
  __host__ __device__ static constexpr float tiny() { return FLT_MIN; }
  __host__ __device__ static constexpr float huge() { return FLT_MAX; }
};
// double-float has FP32's exponent range
template <> struct Lim<df64> {
  __host__ __device__ static constexpr df64 tiny() { return df64(FLT_MIN, 0.f); }
  __host__ __device__ static constexpr df64 huge() { return df64(FLT_MAX, 0.f); }
};

// Species<Euler> subset used on the path (conservationLaws/euler/euler.h:48-60)
template <class R> struct Gas {
  R gamma;      // ratio of specific heats
  R gm1;        // gamma - 1
  R gamma1;     // 1/(gamma-1)
  R Rgas;       // gas constant
  R minf;       // cut-off Mach number (AUSM+up, RoeUnprecWS)
  R inv_gamma;  // 1/gamma
  R lref_dt;    // lref / dt of the species: AUSM+up's adaptive scaling mu = lref / (as dt)
  int vscale;   // AUSM+up velocity-diffusion scaling (LowMachScaling)
  int pscale;   // AUSM+up pressure-diffusion scaling (LowMachScaling)
  unsigned fixes;  // FIX_* corrections of the reference's defects (0: as the reference computes)
};

// Corrections of two defects of the reference, off by default (the reference's results are
// reproduced as written):
//  FIX_MACH_SPLIT_P1 -- MachSplit_P1 (machSplittings.ipp:26-31) is (M1 + eps)/(|M| + eps)
//    with eps the largest finite value, which rounds to 1 for both signs, so SLAU and
//    AUSM+up add both sides' pressure on supersonic faces (F(q, q) is not the exact flux);
//    corrected, P1 is M1/M, the 1/0 split it is meant to be: (s M1 + eps)/(|M| + eps) with
//    eps the smallest normal value (dividing by |M| alone would give -1 for s = -1, M < -1).
//  FIX_FARFIELD_TRANSVERSE -- the Riemann and entropy far fields (conservationLaws/euler/boundary/riemann.ipp:48-50,
//    entropy.ipp:47-49) return the interior state when u_n/|u| < threshold, a test without
//    the absolute value, so every outflow face copies the interior (subsonic outflow then
//    takes no far-field information); corrected, the test is |u_n|/|u| < threshold and
//    outflow faces get the characteristic treatment the rest of the function has.
enum : unsigned { FIX_MACH_SPLIT_P1 = 1u, FIX_FARFIELD_TRANSVERSE = 2u, FIX_ALL = 3u };

// lref and dt default to the reference's air species (1 and the largest double,
// conservationLaws/euler/species.ipp:12), where the adaptive ratio vanishes
template <class R>
__host__ __device__ inline Gas<R> make_gas(double gamma, double Rgas, double minf, double lref = 1.,
                                           double dt = 1.7976931348623157e308, int vscale = 0, int pscale = 0) {
  Gas<R> g;
  g.gamma = R(gamma);
  g.gm1 = R(gamma - 1.);
  g.gamma1 = R(1. / (gamma - 1.));
  g.Rgas = R(Rgas);
  g.minf = R(minf);
  g.inv_gamma = R(1. / gamma);
  g.lref_dt = R(lref / dt);
  g.vscale = vscale;
  g.pscale = pscale;
  g.fixes = 0u;
  return g;
}
template <class R> __host__ __device__ inline Gas<R> with_fixes(Gas<R> g, unsigned fixes) {
  g.fixes = fixes;
  return g;
}

// State<Euler,2> without the unused temperature (conservationLaws/euler/euler.h:62-83)
template <class R> struct St { R p, r, h, u2, a2, u, v, ir; };  // ir = 1/r

template <class R> struct Flux5 { R f[4]; R lam; };

// set2State(primitive) (conservationLaws/euler/transforms/primitive.ipp:24-60)
// (ir = 1/r given)
template <class R>
__host__ __device__ __forceinline__ St<R> prim_state_ir(const Gas<R>& g, R u, R v, R r, R p, R ir) {
  St<R> s;
  s.u = u; s.v = v;
  s.u2 = u * u;
  s.u2 += v * v;
  const R k = R(0.5) * s.u2;
  // a2 = gamma R T with T = p/(r R): gamma p / r, through 1/r (kept for the flux)
  s.ir = ir;
  s.a2 = g.gamma * (p * s.ir);
  s.h = s.a2 * g.gamma1 + k;
  s.p = p; s.r = r;
  return s;
}
template <class R> __host__ __device__ __forceinline__ St<R> prim_state(const Gas<R>& g, R u, R v, R r, R p) {
  return prim_state_ir(g, u, v, r, p, R(1) / r);
}

// set2State(conserved) (conservationLaws/euler/transforms/conserved.ipp:31-76)
template <class R> __host__ __device__ __forceinline__ St<R> cons_state_ir(const Gas<R>& g, const R* qc, R r1) {
  St<R> s;
  const R r = qc[2], re = qc[3];
  s.u = qc[0] * r1; s.v = qc[1] * r1;
  s.u2 = s.u * s.u;
  s.u2 += s.v * s.v;
  const R k = R(0.5) * s.u2;
  const R p = g.gm1 * (re - r * k);
  s.ir = r1;
  s.a2 = g.gamma * (p * r1);
  s.h = s.a2 * g.gamma1 + k;
  s.p = p; s.r = r;
  return s;
}

// set2State of the solution basis: primitive {u, v, rho, p} or conserved
// {rho u, rho v, rho, rho E} (cons = true); the choice is uniform across a launch
template <class R> __host__ __device__ __forceinline__ St<R> cons_state(const Gas<R>& g, const R* qc) {
  return cons_state_ir(g, qc, qdiv(R(1), qc[2]));
}

template <class R> __host__ __device__ __forceinline__ St<R> basis_state(const Gas<R>& g, const R* q, bool cons) {
  return cons ? cons_state(g, q) : prim_state(g, q[0], q[1], q[2], q[3]);
}

// Bits of an FP64 value, for sign and range tests on the integer pipe (the FP64 pipe
// bounds the FP64 stage kernels).
__host__ __device__ __forceinline__ long long f64_bits(double x) {
#ifdef __CUDA_ARCH__
  return __double_as_longlong(x);
#else
  long long b;
  memcpy(&b, &x, sizeof b);
  return b;
#endif
}
// biased exponent of x >= 0 within [1023 - e, 1023 + e] (false for negative, zero,
// subnormal, infinite and NaN x beyond that window)
__host__ __device__ __forceinline__ bool f64_exp_within(double x, unsigned e) {
  const unsigned be = unsigned((unsigned long long)f64_bits(x) >> 52);  // sign bit included
  return be - (1023u - e) <= 2u * e;
}

// s = sqrt(x) and r = 1/s.  FP64 on the device, for positive finite x: r = rsqrt(x)
// (within 1 ulp), s = x r, one multi-instruction sequence instead of two.  Zero,
// infinity, NaN and negative x take sqrt and a division there too, so they give what
// the host gives (x = 0: s = 0, r = inf; x*rsqrt(x) would make s = 0*inf = NaN).
template <class R> __host__ __device__ __forceinline__ void sqrt_rcp(R x, R& s, R& r) {
#ifdef __CUDA_ARCH__
  if constexpr (std::is_same<R, double>::value) {
    const long long b = f64_bits(x);
    if (b > 0 && b < 0x7ff0000000000000LL) {
      r = rsqrt(x);
      s = x * r;
      return;
    }
  }
#endif
  s = sqrt(x);
  r = R(1) / s;
}

// s = sqrt(x); FP64 on the device as x rsqrt(x) for positive x (within 1.5 ulp, fewer
// instructions than the correctly rounded square root), sqrt otherwise (zero stays zero)
template <class R> __host__ __device__ __forceinline__ void sqrt_fast(R x, R& s) {
#ifdef __CUDA_ARCH__
  if constexpr (std::is_same<R, double>::value) {
    const long long b = f64_bits(x);
    s = (b > 0 && b < 0x7ff0000000000000LL) ? x * rsqrt(x) : sqrt(x);
    return;
  }
#endif
  s = sqrt(x);
}

// set2State of the two states of one face.  FP64: both densities' inverses from one
// division, 1/(rL rR) times the other density, when both densities lie in
// [2^-500, 2^500] (the product stays normal); otherwise, and for the other types, one
// division each.
template <class R>
__host__ __device__ __forceinline__ void basis_state2(const Gas<R>& g, const R* ql, const R* qr, bool cons, St<R>& sl,
                                                      St<R>& sr) {
  R il, ir;
  if constexpr (std::is_same<R, double>::value) {
    if (f64_exp_within(ql[2], 500u) && f64_exp_within(qr[2], 500u)) {
      const double inv = 1.0 / (ql[2] * qr[2]);
      il = inv * qr[2];
      ir = inv * ql[2];
    } else {
      il = 1.0 / ql[2];
      ir = 1.0 / qr[2];
    }
  } else {
    il = qdiv(R(1), ql[2]);
    ir = qdiv(R(1), qr[2]);
  }
  if (cons) {
    sl = cons_state_ir(g, ql, il);
    sr = cons_state_ir(g, qr, ir);
  } else {
    sl = prim_state_ir(g, ql[0], ql[1], ql[2], ql[3], il);
    sr = prim_state_ir(g, qr[0], qr[1], qr[2], qr[3], ir);
  }
}

// state2Set<conserved> (conservationLaws/euler/transforms/conserved.ipp:2-29)
template <class R> __host__ __device__ __forceinline__ void state_cons(const St<R>& s, R* qc) {
  qc[0] = s.r * s.u; qc[1] = s.r * s.v; qc[2] = s.r; qc[3] = s.r * s.h - s.p;
}

// projectedVelocity (conservationLaws/base/base.h:148-158)
template <class R> __host__ __device__ __forceinline__ R proj(R nx, R ny, const St<R>& s) { return nx * s.u + ny * s.v; }

// exactFlux (conservationLaws/euler/fluxes/exactFlux.ipp:4-36); a = sqrt(a2)
template <class R> __host__ __device__ __forceinline__ Flux5<R> exact_flux_a(R nx, R ny, const St<R>& s, R a) {
  Flux5<R> o;
  const R un = proj(nx, ny, s);
  const R mn = s.r * un;
  o.f[0] = mn * s.u + s.p * nx;
  o.f[1] = mn * s.v + s.p * ny;
  o.f[2] = mn;
  o.f[3] = mn * s.h;
  o.lam = fabs(un) + a;
  return o;
}
template <class R> __host__ __device__ __forceinline__ Flux5<R> exact_flux(R nx, R ny, const St<R>& s) {
  return exact_flux_a(nx, ny, s, sqrt(s.a2));
}

// CentralFlux (conservationLaws/base/fluxes/centralFlux.ipp:2-14), sound speeds given;
// lam left unscaled by A (the caller's max of unscaled speeds times A equals the max of
// the scaled speeds: rounding is monotone)
template <class R>
__host__ __device__ __forceinline__ Flux5<R> central_flux_u(R nx, R ny, R A, const St<R>& l, const St<R>& r, R al,
                                                            R ar) {
  const Flux5<R> fl = exact_flux_a(nx, ny, l, al), fr = exact_flux_a(nx, ny, r, ar);
  Flux5<R> o;
  const R hA = R(0.5) * A;  // (0.5 s) A == s (0.5 A) in binary arithmetic, one product fewer per component
#pragma unroll
  for (int i = 0; i < 4; ++i) o.f[i] = (fl.f[i] + fr.f[i]) * hA;
  o.lam = fmax(fl.lam, fr.lam);
  return o;
}
template <class R>
__host__ __device__ __forceinline__ Flux5<R> central_flux_a(R nx, R ny, R A, const St<R>& l, const St<R>& r, R al,
                                                            R ar) {
  Flux5<R> o = central_flux_u(nx, ny, A, l, r, al, ar);
  o.lam *= A;
  return o;
}
template <class R> __host__ __device__ __forceinline__ Flux5<R> central_flux(R nx, R ny, R A, const St<R>& l, const St<R>& r) {
  return central_flux_a(nx, ny, A, l, r, sqrt(l.a2), sqrt(r.a2));
}

// Roe flux = central + matrix dissipation (conservationLaws/base/fluxes/roeFlux.ipp:2-58),
// with roeAverage and Harten's entropy fix (conservationLaws/euler/fluxes/roe.ipp:2-78)
// and the characteristic transforms (conservationLaws/euler/transforms/characteristic.ipp).
// FACE = false (RoeFlux as written): the Roe-averaged state keeps its velocity in the
// global frame while the jump is rotated to the face frame (roeFlux.ipp:40-54), exactly as
// the reference composes them; the dissipation is then the Roe matrix's only for a face
// normal (1, 0).  FACE = true: the averaged velocity enters the characteristic transforms
// by its face-normal and tangential components, the frame of the jump, so the flux is
// invariant under rotation; for the normal (1, 0) both are the same bit for bit.
template <class R, bool FACE = false>
__host__ __device__ __forceinline__ Flux5<R> roe_flux(const Gas<R>& g, R nx, R ny, R A, const St<R>& l,
                                                      const St<R>& r) {
  R al, ar;
  sqrt_fast(l.a2, al);
  sqrt_fast(r.a2, ar);
  const Flux5<R> c = central_flux_u(nx, ny, A, l, r, al, ar);
  // roe average: cr = sqrt(rR/rL), ra = cr rL, 1/ra = cr/rR
  const R cr = sqrt(r.r * l.ir);
  const R wl = qdiv(R(1), R(1) + cr);
  const R wr = R(1) - wl;
  const R ra = cr * l.r;
  const R ua = wl * l.u + wr * r.u;
  const R va = wl * l.v + wr * r.v;
  R ka = ua * ua;
  ka += va * va;
  ka *= R(0.5);
  const R ha = wl * l.h + wr * r.h;
  const R a2a = g.gm1 * (ha - ka);
  // the averaged sound speed and its inverse: FP64 from one reciprocal square root
  R aa, a1;
  if constexpr (std::is_same<R, double>::value) sqrt_rcp(a2a, aa, a1);
  else aa = sqrt(a2a);
  // wave speeds and entropy fix
  const R una = nx * ua + ny * va;
  const R unl = proj(nx, ny, l), unr = proj(nx, ny, r);
  R lam[4];
  const R la0 = fabs(una);
  lam[0] = la0; lam[3] = la0;
  {
    const R la1 = una - aa, ll1 = unl - al, lr1 = unr - ar;
    const R le = R(0.05) * fmax(R(0), fmax(la1 - ll1, lr1 - la1));
    const R laa = fabs(la1);
    lam[1] = (laa > le) ? laa : R(0.5) * (le + laa * laa / le);
  }
  {
    const R la2 = una + aa, ll2 = unl + al, lr2 = unr + ar;
    const R le = R(0.05) * fmax(R(0), fmax(la2 - ll2, lr2 - la2));
    const R laa = fabs(la2);
    lam[2] = (laa > le) ? laa : R(0.5) * (le + laa * laa / le);
  }
  // face-aligned jump of conserved variables
  const R tx = -ny, ty = nx;
  const R d0 = r.r * r.u - l.r * l.u;
  const R d1 = r.r * r.v - l.r * l.v;
  const R d2 = r.r - l.r;
  const R d3 = (r.r * r.h - r.p) - (l.r * l.h - l.p);
  const R c0 = nx * d0 + ny * d1;
  const R c1 = tx * d0 + ty * d1;
  // the averaged velocity the transforms see: global components as written, or the
  // face-normal and tangential ones
  const R xa = FACE ? una : ua;
  const R ya = FACE ? tx * ua + ty * va : va;
  // conserved -> primitive about the average state
  const R rho1 = cr * r.ir;
  R cc = ka * d2 + d3;
  const R du0 = (c0 - xa * d2) * rho1;
  cc -= xa * c0;
  const R du1 = (c1 - ya * d2) * rho1;
  cc -= ya * c1;
  const R dp = cc * g.gm1;
  // primitive -> characteristic, scaled by the wave speeds
  if constexpr (!std::is_same<R, double>::value) a1 = qdiv(R(1), aa);
  const R w0 = lam[0] * ((g.gamma * (dp * a1 * a1 - d2)) * rho1);
  const R w1 = lam[1] * (du0 - dp * rho1 * a1);
  const R w2 = lam[2] * (du0 + dp * rho1 * a1);
  const R w3 = lam[3] * du1;
  // characteristic -> primitive -> conserved
  const R dpp = R(0.5) * ra * aa * (w2 - w1);
  const R drr = dpp * (a1 * a1) - ra * w0 * g.inv_gamma;
  const R du = R(0.5) * (w1 + w2);
  const R dv = w3;
  const R e0 = ra * du + xa * drr;
  const R e1 = ra * dv + ya * drr;
  R dk = xa * du;
  dk += ya * dv;
  const R e3 = dpp * g.gamma1 + ra * dk + ka * drr;
  // rotate back
  const R f0 = nx * e0 + tx * e1;
  const R f1 = ny * e0 + ty * e1;
  const R s = R(-0.5) * A;
  Flux5<R> o;
  o.f[0] = c.f[0] + s * f0;
  o.f[1] = c.f[1] + s * f1;
  o.f[2] = c.f[2] + s * drr;
  o.f[3] = c.f[3] + s * e3;
  o.lam = fmax(c.lam, fabs(una) + aa) * A;
  return o;
}

// RusanovFlux (conservationLaws/base/fluxes/rusanovFlux.ipp:2-50)
template <class R> __host__ __device__ __forceinline__ Flux5<R> rusanov_flux(R nx, R ny, R A, const St<R>& l, const St<R>& r) {
  Flux5<R> o = central_flux(nx, ny, A, l, r);
  const R lambda = fmax(fabs(proj(nx, ny, l)) + sqrt(l.a2), fabs(proj(nx, ny, r)) + sqrt(r.a2));
  const R s = R(-0.5) * (lambda * A);
  o.f[0] += s * (r.r * r.u - l.r * l.u);
  o.f[1] += s * (r.r * r.v - l.r * l.v);
  o.f[2] += s * (r.r - l.r);
  o.f[3] += s * ((r.r * r.h - r.p) - (l.r * l.h - l.p));
  return o;
}

// Mach splittings (conservationLaws/euler/fluxes/machSplittings.ipp:8-43)
template <class R> __host__ __device__ __forceinline__ R ms_m1(R s, R M) { return R(0.5) * (M + s * fabs(M)); }
template <class R> __host__ __device__ __forceinline__ R ms_m2(R s, R M) { return s * R(0.25) * (M + s) * (M + s); }
template <class R> __host__ __device__ __forceinline__ R ms_m4(R s, R M, R beta) {
  return ms_m2(s, M) * (R(1) - s * R(16) * beta * ms_m2(-s, M));
}
// (M1 + eps)/(|M| + eps) with eps the largest finite value, as the reference computes it
// (1 for both signs); with FIX_MACH_SPLIT_P1 (s M1 + eps)/(|M| + eps), eps the smallest
// normal value: M1/M, 1 on the side the flow comes from and 0 on the other
template <class R> __host__ __device__ __forceinline__ R ms_p1(R s, R M, unsigned fixes) {
  const bool fix = (fixes & FIX_MACH_SPLIT_P1) != 0u;
  const R eps = fix ? Lim<R>::tiny() : Lim<R>::huge();
  const R m1 = ms_m1(s, M);
  return ((fix ? s * m1 : m1) + eps) / (fabs(M) + eps);
}
template <class R> __host__ __device__ __forceinline__ R ms_p3(R s, R M) { return ms_m2(s, M) * (s * R(2) - M); }
template <class R> __host__ __device__ __forceinline__ R ms_p5(R s, R M, R alpha) {
  return ms_p3(s, M) - s * R(16) * alpha * M * ms_m2(s, M) * ms_m2(-s, M);
}

// SLAU2 with (Convective, Acoustic) tags (conservationLaws/euler/fluxes/slau.ipp:4-161).
// by_mdot=false: literal reference upwinding by the sign of ua (slau.ipp:124-125);
// by_mdot=true: upwinding by the sign of the interface mass flux.
template <class R, bool by_mdot>
__host__ __device__ __forceinline__ Flux5<R> slau_flux(R nx, R ny, R A, const St<R>& l, const St<R>& r,
                                                       unsigned fixes = 0u) {
  const R ua = sqrt(R(0.5) * (l.u2 + r.u2));
  R al, ar;
  sqrt_fast(l.a2, al);
  sqrt_fast(r.a2, ar);
  const R aa = R(0.5) * (al + ar);
  const R aa1 = qdiv(R(1), aa);
  const R ma = ua * aa1;
  const R ma_hat = fmin(R(1), ma);
  const R unl = proj(nx, ny, l), unr = proj(nx, ny, r);
  const R ml = unl * aa1, mr = unr * aa1;
  const R una = (l.r * fabs(unl) + r.r * fabs(unr)) / (l.r + r.r);
  const R chi = (R(1) - ma_hat) * (R(1) - ma_hat);
  const R gs = -fmax(fmin(ml, R(0)), R(-1)) * fmin(fmax(mr, R(0)), R(1));
  const R dr = r.r - l.r, dp = r.p - l.p;
  const R mdot_c = l.r * unl + r.r * unr;
  const R mdot = R(0.5) * ((mdot_c - una * dr) * (R(1) - gs) - chi * dp * aa1) * A;
  const R betal = (fabs(ml) > R(1)) ? ms_p1(R(1), ml, fixes) : ms_p3(R(1), ml);
  const R betar = (fabs(mr) > R(1)) ? ms_p1(R(-1), mr, fixes) : ms_p3(R(-1), mr);
  const R p_c = l.p + r.p;
  const R p_dp = (betal - betar) * dp;
  const R p_du = -ma * (betal + betar - R(1)) * (p_c);
  const R pa = R(0.5) * (p_c - p_dp - p_du) * A;
  const bool left = by_mdot ? (mdot > R(0)) : (ua > R(0));
  const St<R>& w = left ? l : r;
  Flux5<R> o;
  o.f[0] = mdot * w.u + pa * nx;
  o.f[1] = mdot * w.v + pa * ny;
  o.f[2] = mdot;
  o.f[3] = mdot * w.h;
  o.lam = (fmax(al, ar) + fmax(fabs(unl), fabs(unr))) * A;  // sqrt of the larger a2
  return o;
}

// AusmPlusUP<VFluxScaling, PFluxScaling> (conservationLaws/euler/fluxes/ausmPlusUP.ipp:6-171), the
// two scalings chosen at run time (g.vscale, g.pscale; uniform across a launch)
template <class R> __host__ __device__ __forceinline__ Flux5<R> ausmpup_flux(const Gas<R>& g, R nx, R ny, R A,
                                                                   const St<R>& l, const St<R>& r) {
  const R alpha0 = R(0.1875), beta = R(0.125), Ku = R(0.75 * 2.), Kp = R(0.25), sigma = R(1.0);
  const R ascoeff = R(2) * g.gm1 / (g.gamma + R(1));
  const R unl = proj(nx, ny, l), unr = proj(nx, ny, r);
  const R als2 = ascoeff * l.h, ars2 = ascoeff * r.h;
  R sls, srs;
  sqrt_fast(als2, sls);
  sqrt_fast(ars2, srs);
  const R als = als2 / fmax(unl, sls);
  const R ars = ars2 / fmax(-unr, srs);
  const R ra = R(0.5) * (l.r + r.r);
  const R as = fmin(ars, als);
  const R ml = unl / as, mr = unr / as;
  const R m0 = sqrt(R(0.5) * (ml * ml + mr * mr));
  // std::clamp(m0, minf, 1) as libstdc++ evaluates it: min(max(m0, minf), 1)
  const R mlo = (m0 < g.minf) ? g.minf : m0;
  const R m0c = (R(1) < mlo) ? R(1) : mlo;
  R m0p = m0c, m0u = m0c;
  if (g.vscale != SCALING_CONVECTIVE || g.pscale != SCALING_CONVECTIVE) {
    // adaptive: clamp(max(m0, mu), minf, 1), mu = lref / (as dt) the ratio of the acoustic
    // time scale to the step
    const R mu = g.lref_dt / as;
    const R mx = fmax(m0, mu);
    const R alo = (mx < g.minf) ? g.minf : mx;
    const R m0a = (R(1) < alo) ? R(1) : alo;
    m0p = g.pscale == SCALING_CONVECTIVE ? m0c : (g.pscale == SCALING_ACOUSTIC ? R(1) : m0a);
    m0u = g.vscale == SCALING_CONVECTIVE ? m0c : (g.vscale == SCALING_ACOUSTIC ? R(1) : m0a);
  }
  const R fa = m0p * (R(2) - m0p);
  const R fu = (g.vscale == g.pscale) ? fa : m0u * (R(2) - m0u);
  const bool lsup = fabs(ml) > R(1), rsup = fabs(mr) > R(1);
  const R mlp = lsup ? ms_m1(R(1), ml) : ms_m4(R(1), ml, beta);
  const R mrm = rsup ? ms_m1(R(-1), mr) : ms_m4(R(-1), mr, beta);
  const R delp = r.p - l.p;
  const R mp = Kp * fmax(R(1) - sigma * m0 * m0, R(0)) * delp / (fa * ra * as * as);
  const R uaf = as * (mlp + mrm - mp) * A;
  const R alpha = alpha0 * (R(5) * fu * fu - R(4));
  const R plp = lsup ? ms_p1(R(1), ml, g.fixes) : ms_p5(R(1), ml, alpha);
  const R prm = rsup ? ms_p1(R(-1), mr, g.fixes) : ms_p5(R(-1), mr, alpha);
  const R pu = Ku * plp * prm * ra * (fu * as) * (unr - unl);
  const R pa = (plp * l.p + prm * r.p - pu) * A;
  const St<R>& w = (uaf > R(0)) ? l : r;
  const R mdot = uaf * w.r;
  Flux5<R> o;
  o.f[0] = mdot * w.u + pa * nx;
  o.f[1] = mdot * w.v + pa * ny;
  o.f[2] = mdot;
  o.f[3] = mdot * w.h;
  const R lmd = R(0.5) * (m0p + R(1)) / fa;
  const R amax = sqrt(fmax(as * as, fmax(l.a2, r.a2)));
  o.lam = (lmd * amax + fmax(fabs(uaf), fmax(fabs(unl), fabs(unr)))) * A;
  return o;
}

// RoeUnprecWS (conservationLaws/euler/fluxes/roeUnprecWS.ipp:2-109): the central flux minus a
// scalar dissipation, |un| times the conserved jump plus velocity and pressure perturbations
// scaled by the cut-off Mach number (Weiss & Smith's low-Mach form with fixed coefficients)
template <class R> __host__ __device__ __forceinline__ Flux5<R> roe_ws_flux(const Gas<R>& g, R nx, R ny, R A,
                                                                  const St<R>& l, const St<R>& r) {
  R al, ar;
  sqrt_fast(l.a2, al);
  sqrt_fast(r.a2, ar);
  const Flux5<R> c = central_flux_u(nx, ny, A, l, r, al, ar);
  // roe average (conservationLaws/euler/fluxes/roe.ipp:2-48)
  const R cr = sqrt(r.r * l.ir);
  const R wl = qdiv(R(1), R(1) + cr);
  const R wr = R(1) - wl;
  const R ra = cr * l.r;
  const R ua = wl * l.u + wr * r.u;
  const R va = wl * l.v + wr * r.v;
  R ka = ua * ua;
  ka += va * va;
  ka *= R(0.5);
  const R ha = wl * l.h + wr * r.h;
  const R aa = sqrt(g.gm1 * (ha - ka));
  const R una = nx * ua + ny * va;
  const R dp = r.p - l.p;
  const R du = proj(nx, ny, r) - proj(nx, ny, l);
  const R uinf = g.minf * aa;
  // nu_p = minf / (ra uinf^2), nu_u = 0.05, mu_p = 0.02 minf, mu_u = 0.1 ra uinf minf
  const R nu_p = (R(1) / (ra * uinf * uinf)) * g.minf;
  const R mu_u = (R(0.10) * (ra * uinf)) * g.minf;
  const R dU = nu_p * dp + R(0.05) * du;
  const R dP = (R(0.02) * g.minf) * dp + mu_u * du;
  const R aun = fabs(una);
  const R d0 = r.r * r.u - l.r * l.u;
  const R d1 = r.r * r.v - l.r * l.v;
  const R d2 = r.r - l.r;
  const R d3 = (r.r * r.h - r.p) - (l.r * l.h - l.p);
  const R s = R(0.5) * A;
  Flux5<R> o;
  o.f[0] = c.f[0] - s * ((aun * d0 + dU * (ra * ua)) + dP * nx);
  o.f[1] = c.f[1] - s * ((aun * d1 + dU * (ra * va)) + dP * ny);
  o.f[2] = c.f[2] - s * (aun * d2 + dU * ra);
  o.f[3] = c.f[3] - s * ((aun * d3 + dU * (ra * ha)) + dP * una);
  o.lam = fmax(c.lam, aun + aa) * A;
  return o;
}

template <class R, int FK>
__host__ __device__ __forceinline__ Flux5<R> face_flux(const Gas<R>& g, R nx, R ny, R A, const St<R>& l, const St<R>& r) {
  if constexpr (FK == FLUX_ROE) return roe_flux(g, nx, ny, A, l, r);
  else if constexpr (FK == FLUX_ROE_FACE) return roe_flux<R, true>(g, nx, ny, A, l, r);
  else if constexpr (FK == FLUX_SLAU) return slau_flux<R, true>(nx, ny, A, l, r, g.fixes);
  else if constexpr (FK == FLUX_SLAU_REF) return slau_flux<R, false>(nx, ny, A, l, r, g.fixes);
  else if constexpr (FK == FLUX_AUSMPUP) return ausmpup_flux(g, nx, ny, A, l, r);
  else if constexpr (FK == FLUX_RUSANOV) return rusanov_flux(nx, ny, A, l, r);
  else if constexpr (FK == FLUX_ROE_WS) return roe_ws_flux(g, nx, ny, A, l, r);
  else return central_flux(nx, ny, A, l, r);
}

template <class R> __host__ __device__ __forceinline__ R limit(int kind, R a, R b);

// van Albada's slopes a b (a + b) / (a^2 + b^2) of the four variables of one face side
// (0 exactly where a b <= 0), a2 = a^2 given, FP64.  The four quotients come from one
// division (batched inversion: 1/d_v from the inverse of the product of the
// denominators and the partial products) when every denominator lies in
// [2^-240, 2^240], so that all products stay normal and finite; otherwise one division
// per variable, with the reference's tiny added to the denominator.  The sign and range
// tests read the bits on the integer pipe.
__host__ __device__ __forceinline__ void vanalbada4(const double* a, const double* a2, const double* b, double* out) {
  double num[4], den[4], pre[4];
  double acc = 1.0;
  bool ok = true, any = false;
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const double ab = a[v] * b[v];
    const long long bits = f64_bits(ab);
    // a b > 0, or NaN (which propagates)
    const bool on = bits > 0 || (bits & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
    // explicit contraction: the same rounding in every kernel that inlines this
    num[v] = on ? ab * (a[v] + b[v]) : 0.0;
    den[v] = on ? fma(b[v], b[v], a2[v]) : 1.0;
    any = any || on;
    pre[v] = acc;
    acc = acc * den[v];
    ok = ok && f64_exp_within(den[v], 240u);
  }
  if (!any) {
#pragma unroll
    for (int v = 0; v < 4; ++v) out[v] = 0.0;
  } else if (ok) {
    double inv = 1.0 / acc;
#pragma unroll
    for (int v = 3; v >= 0; --v) {
      out[v] = num[v] * (inv * pre[v]);
      inv = inv * den[v];
    }
  } else {
#pragma unroll
    for (int v = 0; v < 4; ++v) out[v] = num[v] / (den[v] + Lim<double>::tiny());
  }
}

// The limited slopes of both sides of one face, FP64: outl[v] = limit(a[v], bl[v]),
// outr[v] = limit(a[v], br[v]) (the central slope a is common to both sides).
__host__ __device__ __forceinline__ void limit4x2(int kind, const double* a, const double* bl, const double* br,
                                                  double* outl, double* outr) {
  if (kind == LIM_VANALBADA) {
    double a2[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) a2[v] = a[v] * a[v];
    vanalbada4(a, a2, bl, outl);
    vanalbada4(a, a2, br, outr);
    return;
  }
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    outl[v] = limit<double>(kind, a[v], bl[v]);
    outr[v] = limit<double>(kind, a[v], br[v]);
  }
}

// Slope limiters (limiters/limiter.ipp:8-161), called as limit(central, biased).
// LIM_VANLEER is the harmonic-mean slope (a|b|+|a|b)/(|a|+|b|+eps);
// LIM_VANLEER_REF the literal reference expression (limiter.ipp:81-89).
template <class R> __host__ __device__ __forceinline__ R limit(int kind, R a, R b) {
  const R tiny = Lim<R>::tiny();
  switch (kind) {
    case LIM_NOLIMIT1: return R(0);
    case LIM_NOLIMIT2: return R(0.5) * (a + b);
    case LIM_NOLIMIT3: return R(0.33333333333333333) * (R(2) * a + b);
    case LIM_VANALBADA: return (a * b < R(0)) ? R(0) : qdiv(b * (a * a) + a * (b * b), a * a + b * b + tiny);
    case LIM_MINMOD: return (a > R(0)) ? fmin(a, fmax(b, R(0))) : fmax(a, fmin(b, R(0)));
    case LIM_SUPERBEE:
      return (a > R(0)) ? fmax(R(0), fmax(fmin(R(2) * a, b), fmin(R(2) * b, a)))
                        : fmin(R(0), fmin(fmax(R(2) * a, b), fmax(R(2) * b, a)));
    case LIM_MC:
      return (a > R(0)) ? fmax(R(0), fmin(R(0.5) * (a + b), fmin(R(2) * b, R(2) * a)))
                        : fmin(R(0), fmax(R(0.5) * (a + b), fmax(R(2) * b, R(2) * a)));
    case LIM_VANLEER: return qdiv(a * fabs(b) + fabs(a) * b, fabs(a) + fabs(b) + tiny);
    case LIM_VANLEER_REF: return (b + fabs(b)) / (a + fabs(b) + tiny);
    case LIM_CADA3: {
      const R gam = R(1.5), c1 = R(-2. / 7.), c2 = R(0.4), c3 = R(3) * gam - R(2);
      const R u = (a > R(0)) ? a : -a;
      const R v = (a > R(0)) ? b : -b;
      R w;
      if (fabs(a) + fabs(b) > R(0)) {
        if (v < R(-2) * u) w = R(0);
        else if (v < c1 * u) w = (v + R(2) * u) / R(3);
        else if (v < R(0)) w = R(-2) * v;
        else if (v < c2 * u) w = R(2) * v;
        else if (v < c3 * u) w = (v + R(2) * u) / R(3);
        else w = gam * u;
      } else {
        w = (v + R(2) * u) / R(3);
      }
      return (a <= R(0)) ? -w : w;
    }
    default: return R(0);
  }
}

// ---------------------------------------------------------------- branch signatures
// The parity report counts the faces (and cells) where the GPU and the oracle take a
// different branch.  limit_piece: which piece of the limiter's piecewise definition
// limit(a, b) evaluates, as 4 bits: bit 3 = (a > 0); bits 0-2 = the interval of the
// ratio b/a (compared by multiplication, with u = |a| and v = b signed like a) that
// selects the expression.  The oracle (oracle/hc_oracle.hpp) defines the same codes.
template <class R> __host__ __device__ __forceinline__ unsigned limit_piece(int kind, R a, R b) {
  const bool pos = a > R(0);
  const R u = pos ? a : -a, v = pos ? b : -b;
  unsigned p = 0;
  switch (kind) {
    case LIM_VANALBADA: p = (a * b < R(0)) ? 0u : 1u; break;
    case LIM_VANLEER: p = (a * b > R(0)) ? 1u : 0u; break;
    case LIM_MINMOD: p = (v <= R(0)) ? 0u : (v < u ? 1u : 2u); break;
    case LIM_SUPERBEE:
      p = (v <= R(0)) ? 0u : (R(2) * v < u ? 1u : (v < u ? 2u : (v < R(2) * u ? 3u : 4u)));
      break;
    case LIM_MC: p = (v <= R(0)) ? 0u : (R(3) * v < u ? 1u : (v < R(3) * u ? 2u : 3u)); break;
    case LIM_CADA3: {
      const R c1 = R(-2. / 7.), c2 = R(0.4), c3 = R(3) * R(1.5) - R(2);
      if (!(fabs(a) + fabs(b) > R(0))) p = 7u;
      else if (v < R(-2) * u) p = 1u;
      else if (v < c1 * u) p = 2u;
      else if (v < R(0)) p = 3u;
      else if (v < c2 * u) p = 4u;
      else if (v < c3 * u) p = 5u;
      else p = 6u;
      break;
    }
    default: return 0u;  // the unlimited and the literal van Leer expressions have one piece
  }
  return p | (pos ? 8u : 0u);
}

// Branches taken inside the interface flux of two face states (4 bits), with the
// flux's own intermediate expressions: Roe -- Harten's fix active on the u-a and u+a
// waves; SLAU -- |M_L| > 1, |M_R| > 1, Mach of the mean speed above 1; AUSM+up --
// |M_L| > 1, |M_R| > 1, which side's critical speed is the interface sound speed;
// Rusanov / central / RoeUnprecWS -- which side's spectral radius is the larger.
template <class R, int FK>
__host__ __device__ __forceinline__ unsigned flux_bits(const Gas<R>& g, R nx, R ny, const St<R>& l, const St<R>& r) {
  const R unl = proj(nx, ny, l), unr = proj(nx, ny, r);
  if constexpr (FK == FLUX_ROE || FK == FLUX_ROE_FACE) {
    R al, ar;
    sqrt_fast(l.a2, al);
    sqrt_fast(r.a2, ar);
    const R cr = sqrt(r.r * l.ir);
    const R wl = R(1) / (R(1) + cr);
    const R wr = R(1) - wl;
    const R ua = wl * l.u + wr * r.u;
    const R va = wl * l.v + wr * r.v;
    R ka = ua * ua;
    ka += va * va;
    ka *= R(0.5);
    const R ha = wl * l.h + wr * r.h;
    R aa, a1;
    if constexpr (std::is_same<R, double>::value) sqrt_rcp(g.gm1 * (ha - ka), aa, a1);
    else aa = sqrt(g.gm1 * (ha - ka));
    (void)a1;
    const R una = nx * ua + ny * va;
    unsigned b = 0;
    {
      const R la1 = una - aa, ll1 = unl - al, lr1 = unr - ar;
      const R le = R(0.05) * fmax(R(0), fmax(la1 - ll1, lr1 - la1));
      if (!(fabs(la1) > le)) b |= 1u;
    }
    {
      const R la2 = una + aa, ll2 = unl + al, lr2 = unr + ar;
      const R le = R(0.05) * fmax(R(0), fmax(la2 - ll2, lr2 - la2));
      if (!(fabs(la2) > le)) b |= 2u;
    }
    return b;
  } else if constexpr (FK == FLUX_SLAU || FK == FLUX_SLAU_REF) {
    const R ua = sqrt(R(0.5) * (l.u2 + r.u2));
    R al, ar;
    sqrt_fast(l.a2, al);
    sqrt_fast(r.a2, ar);
    const R aa = R(0.5) * (al + ar);
    const R aa1 = qdiv(R(1), aa);
    const R ml = unl * aa1, mr = unr * aa1;
    return (fabs(ml) > R(1) ? 1u : 0u) | (fabs(mr) > R(1) ? 2u : 0u) | (ua * aa1 > R(1) ? 4u : 0u);
  } else if constexpr (FK == FLUX_AUSMPUP) {
    const R ascoeff = R(2) * g.gm1 / (g.gamma + R(1));
    const R als2 = ascoeff * l.h, ars2 = ascoeff * r.h;
    R sls, srs;
    sqrt_fast(als2, sls);
    sqrt_fast(ars2, srs);
    const R als = als2 / fmax(unl, sls);
    const R ars = ars2 / fmax(-unr, srs);
    const R as = fmin(ars, als);
    const R ml = unl / as, mr = unr / as;
    return (fabs(ml) > R(1) ? 1u : 0u) | (fabs(mr) > R(1) ? 2u : 0u) | (als < ars ? 4u : 0u);
  } else {
    const R lamL = fabs(unl) + sqrt(l.a2), lamR = fabs(unr) + sqrt(r.a2);
    return lamR > lamL ? 1u : 0u;
  }
}

// Roe average of two primitive states in the face frame, used by the far-field
// boundary updates (conservationLaws/euler/fluxes/roe.ipp:2-48).
template <class R> __host__ __device__ __forceinline__ void roe_avg_vel(const St<R>& l, const St<R>& r, R* uav, R* u2,
                                                              R* a2, const Gas<R>& g) {
  const R cr = sqrt(r.r / l.r);
  const R wl = R(1) / (R(1) + cr);
  const R wr = R(1) - wl;
  const R ua = wl * l.u + wr * r.u;
  const R va = wl * l.v + wr * r.v;
  R ka = ua * ua;
  ka += va * va;
  ka *= R(0.5);
  const R ha = wl * l.h + wr * r.h;
  *a2 = g.gm1 * (ha - ka);
  uav[0] = ua; uav[1] = va;
  *u2 = R(2) * ka;
}

// Riemann-invariant far field (conservationLaws/euler/boundary/riemann.ipp:18-113)
// and entropy/pressure far field (entropy.ipp:18-88).  (nx,ny) points into the
// domain; qi, qf, qb are primitive.
template <class R, int BK>
__host__ __device__ __forceinline__ void farfield_update(const Gas<R>& g, R nx, R ny, const R* qi, const R* qf, R* qb,
                                                         bool cons = false, unsigned* path = nullptr) {
  // path (when asked for): 1 interior copy (transverse flow), 2 upwind copy (supersonic), 3 subsonic
  const R tx = -ny, ty = nx;
  const R ri[4] = {nx * qi[0] + ny * qi[1], tx * qi[0] + ty * qi[1], qi[2], qi[3]};
  const R rf[4] = {nx * qf[0] + ny * qf[1], tx * qf[0] + ty * qf[1], qf[2], qf[3]};
  const St<R> sI = basis_state(g, ri, cons);
  const St<R> sF = basis_state(g, rf, cons);
  R uav[2], u2a, a2a;
  roe_avg_vel(sI, sF, uav, &u2a, &a2a, g);
  const R thr = (BK == BC_RIEMANN) ? R(0.001) : R(0.0001);
  const R cosn = uav[0] / sqrt(u2a);
  if (((g.fixes & FIX_FARFIELD_TRANSVERSE) ? fabs(cosn) : cosn) < thr) {
#pragma unroll
    for (int k = 0; k < 4; ++k) qb[k] = qi[k];
    if (path) *path = 1u;
    return;
  }
  const R ma = uav[0] / sqrt(a2a);
  const bool inflow = ma > R(0);
  const R* quw = inflow ? qf : qi;
  if (fabs(ma) > R(1)) {
#pragma unroll
    for (int k = 0; k < 4; ++k) qb[k] = quw[k];
    if (path) *path = 2u;
    return;
  }
  if (path) *path = 3u;
  const St<R>& sU = inflow ? sF : sI;
  R b[4];
  if constexpr (BK == BC_RIEMANN) {
    const R ai = sqrt(sI.a2), af = sqrt(sF.a2);
    const R rim = sI.u - R(2) * ai * g.gamma1;
    const R rip = sF.u + R(2) * af * g.gamma1;
    const R ub = R(0.5) * (rim + rip);
    const R ab = R(0.25) * g.gm1 * (rip - rim);
    const R sb = sU.a2 / (g.gamma * pow(sU.r, g.gm1));
    const R rb = pow(ab * ab / (g.gamma * sb), g.gamma1);
    const R pb = rb * ab * ab / g.gamma;
    b[0] = ub; b[1] = sU.v; b[2] = rb; b[3] = pb;
  } else {
    const St<R>& sD = inflow ? sI : sF;
    const R pb = sD.p;
    const R sb = sU.a2 / (g.gamma * pow(sU.r, g.gm1));
    const R rb = pow(pb / sb, R(1) / g.gamma);
    b[0] = sU.u; b[1] = sU.v; b[2] = rb; b[3] = pb;
  }
  if (cons) {  // set2Set to the conserved basis in the face frame, then rotate back
    const St<R> sb = prim_state(g, b[0], b[1], b[2], b[3]);
    state_cons(sb, b);
  }
  qb[0] = nx * b[0] + tx * b[1];
  qb[1] = ny * b[0] + ty * b[1];
  qb[2] = b[2]; qb[3] = b[3];
}

// Inviscid wall (conservationLaws/euler/boundary/inviscidWall.ipp:33-72): pressure
// flux only, from the interior state moved to the face (qw primitive).
template <class R>
__host__ __device__ __forceinline__ Flux5<R> wall_flux(const Gas<R>& g, R nx, R ny, R A, const R* qw, bool cons = false) {
  const St<R> s = basis_state(g, qw, cons);
  Flux5<R> o;
  o.f[0] = A * s.p * nx;
  o.f[1] = A * s.p * ny;
  o.f[2] = R(0);
  o.f[3] = R(0);
  o.lam = A * (fabs(proj(nx, ny, s)) + sqrt(s.a2));
  return o;
}

}  // namespace hc
