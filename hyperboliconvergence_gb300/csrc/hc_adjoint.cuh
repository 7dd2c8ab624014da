// hc_adjoint.cuh -- hand-written reverse-mode (discrete adjoint) versions of
// the pointwise functions of the residual path.  Each *_adj function takes the
// primal inputs, recomputes what it needs, and accumulates input adjoints from
// output adjoints (x_bar += (dy/dx)^T y_bar).  Branches (limiters, entropy fix,
// upwind switches) are differentiated along the branch the primal takes.
// The spectral-radius outputs are not differentiated: the adjoint treats the
// timestep of every step as a constant (frozen-timestep adjoint).
#pragma once

#include "hc_physics.cuh"

namespace hc {

template <class R> __host__ __device__ __forceinline__ R sgn(R x) { return x > R(0) ? R(1) : (x < R(0) ? R(-1) : R(0)); }

// primitive state adjoint: (u2, a2, h) -> (u, v, r, p); p and r also pass through
template <class R> struct StBar { R u, v, r, p, u2, a2, h; };

// (ir = 1/r given)
template <class R> __host__ __device__ __forceinline__ void prim_state_adj_ir(const Gas<R>& g, const R* q, R ir,
                                                                              StBar<R>& sb, R* qbar) {
  // h = a2*gamma1 + 0.5*u2
  sb.a2 += g.gamma1 * sb.h;
  sb.u2 += R(0.5) * sb.h;
  // u2 = u*u + v*v
  sb.u += R(2) * q[0] * sb.u2;
  sb.v += R(2) * q[1] * sb.u2;
  // a2 = gamma*R*t, t = p/(r*R): d a2/dp = gamma/r, d a2/dr = -gamma p/r^2
  const R gb = g.gamma * ir * sb.a2;
  sb.p += gb;
  sb.r -= gb * (q[3] * ir);
  qbar[0] += sb.u;
  qbar[1] += sb.v;
  qbar[2] += sb.r;
  qbar[3] += sb.p;
}
template <class R> __host__ __device__ __forceinline__ void prim_state_adj(const Gas<R>& g, const R* q, StBar<R>& sb,
                                                                  R* qbar) {
  prim_state_adj_ir(g, q, R(1) / q[2], sb, qbar);
}

// exact flux adjoint, accumulating into the state adjoint of one side
template <class R> __host__ __device__ __forceinline__ void exact_flux_adj(R nx, R ny, const St<R>& s, const R* fbar,
                                                                  StBar<R>& sb) {
  const R un = nx * s.u + ny * s.v;
  const R mn = s.r * un;
  const R mnbar = s.u * fbar[0] + s.v * fbar[1] + fbar[2] + s.h * fbar[3];
  sb.u += mn * fbar[0];
  sb.v += mn * fbar[1];
  sb.p += nx * fbar[0] + ny * fbar[1];
  sb.h += mn * fbar[3];
  sb.r += un * mnbar;
  const R unbar = s.r * mnbar;
  sb.u += nx * unbar;
  sb.v += ny * unbar;
}

// Harten entropy fix of one nonlinear wave (roe.ipp:66-75) reversed
template <class R> __host__ __device__ __forceinline__ void entropy_fix_adj(R la, R ll, R lr, R lbar, R* labar, R* llbar,
                                                                   R* lrbar) {
  const R d1 = la - ll, d2 = lr - la;
  const R mx = fmax(d1, d2);
  const R le = R(0.05) * fmax(R(0), mx);
  const R laa = fabs(la);
  R laabar, lebar = R(0);
  if (laa > le) {
    laabar = lbar;
  } else {
    lebar = R(0.5) * (R(1) - laa * laa / (le * le)) * lbar;
    laabar = (laa / le) * lbar;
  }
  *labar += sgn(la) * laabar;
  if (mx > R(0)) {
    const R mbar = R(0.05) * lebar;
    if (d1 >= d2) { *labar += mbar; *llbar -= mbar; }
    else { *lrbar += mbar; *labar -= mbar; }
  }
}

// Reverse of roe_flux (hc_physics.cuh) for the four conserved flux components,
// with respect to the two primitive face states.
template <class R>
__host__ __device__ __forceinline__ void roe_flux_adj(const Gas<R>& g, R nx, R ny, R A, const R* ql, const R* qr,
                                             const R* Fbar, R* qlbar, R* qrbar) {
  // FP64: the two inverse densities from one division, the sound speeds and their
  // inverses from reciprocal square roots (as the forward stage computes them)
  St<R> l, r;
  basis_state2(g, ql, qr, false, l, r);
  // ---- forward recomputation (reciprocals: l.ir = 1/rL, r.ir = 1/rR, a1 = 1/aa)
  const R z = r.r * l.ir;
  const R cr = sqrt(z);
  const R icr = cr * l.r * r.ir;  // 1/cr
  const R wl = R(1) / (R(1) + cr);
  const R wr = R(1) - wl;
  const R ra = cr * l.r;
  const R ua = wl * l.u + wr * r.u;
  const R va = wl * l.v + wr * r.v;
  const R ka = R(0.5) * (ua * ua + va * va);
  const R ha = wl * l.h + wr * r.h;
  const R a2a = g.gm1 * (ha - ka);
  R aa, a1, al, ial, ar, iar;
  sqrt_rcp(a2a, aa, a1);
  sqrt_rcp(l.a2, al, ial);
  sqrt_rcp(r.a2, ar, iar);
  const R una = nx * ua + ny * va;
  const R unl = nx * l.u + ny * l.v, unr = nx * r.u + ny * r.v;
  const R la1 = una - aa, ll1 = unl - al, lr1 = unr - ar;
  const R la2 = una + aa, ll2 = unl + al, lr2 = unr + ar;
  auto fix = [](R la, R ll, R lr) {
    const R le = R(0.05) * fmax(R(0), fmax(la - ll, lr - la));
    const R laa = fabs(la);
    return (laa > le) ? laa : R(0.5) * (le + laa * laa / le);
  };
  const R lam0 = fabs(una), lam1 = fix(la1, ll1, lr1), lam2 = fix(la2, ll2, lr2), lam3 = lam0;
  const R tx = -ny, ty = nx;
  const R d0 = r.r * r.u - l.r * l.u;
  const R d1 = r.r * r.v - l.r * l.v;
  const R d2 = r.r - l.r;
  const R d3 = (r.r * r.h - r.p) - (l.r * l.h - l.p);
  const R c0 = nx * d0 + ny * d1;
  const R c1 = tx * d0 + ty * d1;
  const R rho1 = cr * r.ir;  // 1/ra
  const R cc = ka * d2 + d3 - ua * c0 - va * c1;
  const R du0 = (c0 - ua * d2) * rho1;
  const R du1 = (c1 - va * d2) * rho1;
  const R dp = cc * g.gm1;
  const R X0 = g.gamma * (dp * a1 * a1 - d2) * rho1;
  const R X1 = du0 - dp * rho1 * a1;
  const R X2 = du0 + dp * rho1 * a1;
  const R w0 = lam0 * X0, w1 = lam1 * X1, w2 = lam2 * X2, w3 = lam3 * du1;
  const R dpp = R(0.5) * ra * aa * (w2 - w1);
  const R drr = dpp * (a1 * a1) - ra * w0 * g.inv_gamma;
  const R du = R(0.5) * (w1 + w2);
  const R dv = w3;
  const R dk = ua * du + va * dv;
  // ---- reverse
  const R s = R(-0.5) * A;
  const R f0b = s * Fbar[0], f1b = s * Fbar[1];
  R drrb = s * Fbar[2];
  const R e3b = s * Fbar[3];
  const R e0b = nx * f0b + ny * f1b;
  const R e1b = tx * f0b + ty * f1b;
  R dppb = g.gamma1 * e3b;
  R rab = dk * e3b;
  const R dkb = ra * e3b;
  R kab = drr * e3b;
  drrb += ka * e3b;
  R uab = du * dkb, vab = dv * dkb;
  R dub = ua * dkb, dvb = va * dkb;
  rab += dv * e1b; dvb += ra * e1b; vab += drr * e1b; drrb += va * e1b;
  rab += du * e0b; dub += ra * e0b; uab += drr * e0b; drrb += ua * e0b;
  R w3b = dvb;
  R w1b = R(0.5) * dub, w2b = R(0.5) * dub;
  dppb += drrb * (a1 * a1);
  R aab = R(-2) * dpp * (a1 * a1 * a1) * drrb;
  rab += -w0 * g.inv_gamma * drrb;
  R w0b = -ra * g.inv_gamma * drrb;
  rab += R(0.5) * aa * (w2 - w1) * dppb;
  aab += R(0.5) * ra * (w2 - w1) * dppb;
  w2b += R(0.5) * ra * aa * dppb;
  w1b -= R(0.5) * ra * aa * dppb;
  R lam0b = X0 * w0b, lam1b = X1 * w1b, lam2b = X2 * w2b, lam3b = du1 * w3b;
  const R X0b = lam0 * w0b, X1b = lam1 * w1b, X2b = lam2 * w2b;
  R du1b = lam3 * w3b;
  R du0b = X1b + X2b;
  R dpb = rho1 * a1 * (X2b - X1b);
  R rho1b = dp * a1 * (X2b - X1b);
  R a1b = dp * rho1 * (X2b - X1b);
  dpb += g.gamma * a1 * a1 * rho1 * X0b;
  a1b += g.gamma * R(2) * dp * a1 * rho1 * X0b;
  R d2b = -g.gamma * rho1 * X0b;
  rho1b += g.gamma * (dp * a1 * a1 - d2) * X0b;
  aab += -a1 * a1 * a1b;
  const R ccb = g.gm1 * dpb;
  R c1b = rho1 * du1b;
  vab -= d2 * rho1 * du1b;
  d2b -= va * rho1 * du1b;
  rho1b += (c1 - va * d2) * du1b;
  R c0b = rho1 * du0b;
  uab -= d2 * rho1 * du0b;
  d2b -= ua * rho1 * du0b;
  rho1b += (c0 - ua * d2) * du0b;
  kab += d2 * ccb; d2b += ka * ccb;
  const R d3b = ccb;
  uab -= c0 * ccb; c0b -= ua * ccb;
  vab -= c1 * ccb; c1b -= va * ccb;
  rab += -rho1 * rho1 * rho1b;
  const R d0b = nx * c0b + tx * c1b;
  const R d1b = ny * c0b + ty * c1b;
  StBar<R> lb{}, rb{};
  rb.r += r.u * d0b; rb.u += r.r * d0b; lb.r -= l.u * d0b; lb.u -= l.r * d0b;
  rb.r += r.v * d1b; rb.v += r.r * d1b; lb.r -= l.v * d1b; lb.v -= l.r * d1b;
  rb.r += d2b; lb.r -= d2b;
  rb.r += r.h * d3b; rb.h += r.r * d3b; rb.p -= d3b;
  lb.r -= l.h * d3b; lb.h -= l.r * d3b; lb.p += d3b;
  // wave speeds
  R unab = sgn(una) * (lam0b + lam3b);
  R la1b = R(0), ll1b = R(0), lr1b = R(0), la2b = R(0), ll2b = R(0), lr2b = R(0);
  entropy_fix_adj(la1, ll1, lr1, lam1b, &la1b, &ll1b, &lr1b);
  entropy_fix_adj(la2, ll2, lr2, lam2b, &la2b, &ll2b, &lr2b);
  unab += la1b + la2b;
  aab += la2b - la1b;
  const R unlb = ll1b + ll2b, unrb = lr1b + lr2b;
  const R alb = ll2b - ll1b, arb = lr2b - lr1b;
  lb.a2 += alb * (R(0.5) * ial);
  rb.a2 += arb * (R(0.5) * iar);
  lb.u += nx * unlb; lb.v += ny * unlb;
  rb.u += nx * unrb; rb.v += ny * unrb;
  uab += nx * unab; vab += ny * unab;
  const R a2ab = aab * (R(0.5) * a1);
  const R hab = g.gm1 * a2ab;
  kab -= g.gm1 * a2ab;
  uab += ua * kab; vab += va * kab;
  R wlb = l.h * hab + l.u * uab + l.v * vab;
  const R wrb = r.h * hab + r.u * uab + r.v * vab;
  lb.h += wl * hab; rb.h += wr * hab;
  lb.u += wl * uab; rb.u += wr * uab;
  lb.v += wl * vab; rb.v += wr * vab;
  R crb = l.r * rab;
  lb.r += cr * rab;
  wlb -= wrb;
  crb += -wl * wl * wlb;
  const R zb = crb * (R(0.5) * icr);
  rb.r += zb * l.ir;
  lb.r -= zb * z * l.ir;
  // central part: c.f[i] = 0.5*(fl[i]+fr[i])*A
  R fe[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) fe[i] = R(0.5) * A * Fbar[i];
  exact_flux_adj(nx, ny, l, fe, lb);
  exact_flux_adj(nx, ny, r, fe, rb);
  prim_state_adj_ir(g, ql, l.ir, lb, qlbar);
  prim_state_adj_ir(g, qr, r.ir, rb, qrbar);
}

// Reverse of rusanov_flux (conservationLaws/base/fluxes/rusanovFlux.ipp:2-50)
template <class R>
__host__ __device__ __forceinline__ void rusanov_flux_adj(const Gas<R>& g, R nx, R ny, R A, const R* ql, const R* qr,
                                                 const R* Fbar, R* qlbar, R* qrbar) {
  const St<R> l = prim_state(g, ql[0], ql[1], ql[2], ql[3]);
  const St<R> r = prim_state(g, qr[0], qr[1], qr[2], qr[3]);
  const R unl = nx * l.u + ny * l.v, unr = nx * r.u + ny * r.v;
  const R al = sqrt(l.a2), ar = sqrt(r.a2);
  const R srl = fabs(unl) + al, srr = fabs(unr) + ar;
  const R lambda = fmax(srl, srr);
  const R s = R(-0.5) * (lambda * A);
  const R dc[4] = {r.r * r.u - l.r * l.u, r.r * r.v - l.r * l.v, r.r - l.r, (r.r * r.h - r.p) - (l.r * l.h - l.p)};
  StBar<R> lb{}, rb{};
  // dissipation s*dc
  R sb = R(0);
#pragma unroll
  for (int i = 0; i < 4; ++i) sb += dc[i] * Fbar[i];
  const R lamb = R(-0.5) * A * sb;
  rb.r += r.u * s * Fbar[0]; rb.u += r.r * s * Fbar[0]; lb.r -= l.u * s * Fbar[0]; lb.u -= l.r * s * Fbar[0];
  rb.r += r.v * s * Fbar[1]; rb.v += r.r * s * Fbar[1]; lb.r -= l.v * s * Fbar[1]; lb.v -= l.r * s * Fbar[1];
  rb.r += s * Fbar[2]; lb.r -= s * Fbar[2];
  rb.r += r.h * s * Fbar[3]; rb.h += r.r * s * Fbar[3]; rb.p -= s * Fbar[3];
  lb.r -= l.h * s * Fbar[3]; lb.h -= l.r * s * Fbar[3]; lb.p += s * Fbar[3];
  if (srl >= srr) {
    lb.u += nx * sgn(unl) * lamb; lb.v += ny * sgn(unl) * lamb; lb.a2 += lamb / (R(2) * al);
  } else {
    rb.u += nx * sgn(unr) * lamb; rb.v += ny * sgn(unr) * lamb; rb.a2 += lamb / (R(2) * ar);
  }
  R fe[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) fe[i] = R(0.5) * A * Fbar[i];
  exact_flux_adj(nx, ny, l, fe, lb);
  exact_flux_adj(nx, ny, r, fe, rb);
  prim_state_adj(g, ql, lb, qlbar);
  prim_state_adj(g, qr, rb, qrbar);
}

// van Albada's value z = ab(a+b)/(a^2+b^2+tiny) and its derivatives along the taken branch
// for four (a, b) pairs, FP64: 0 with zero derivatives where a b < 0 or a = b = 0 (the
// formula's own derivatives there); otherwise the four inverse denominators from one
// division (batched inversion) when every denominator lies in [2^-240, 2^240], one
// division each when not.  The sign and range tests read the bits on the integer pipe.
__host__ __device__ __forceinline__ void vanalbada_vg4(const double* a, const double* b, double* z, double* da,
                                                       double* db) {
  double den[4], pre[4], iden[4];
  double acc = 1.0;
  bool ok = true, any = false;
  bool on[4];
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const long long bits = f64_bits(a[v] * b[v]);
    const unsigned long long mag = (unsigned long long)bits << 1;  // magnitude bits
    // not (a b < 0): a b is +0, -0, positive or NaN (which propagates); and not a = b = 0
    const bool both_zero = ((unsigned long long)f64_bits(a[v]) << 1) == 0 && ((unsigned long long)f64_bits(b[v]) << 1) == 0;
    on[v] = (bits >= 0 || mag == 0 || mag > (0x7ff0000000000000ULL << 1)) && !both_zero;
    den[v] = on[v] ? fma(a[v], a[v], b[v] * b[v]) : 1.0;
    any = any || on[v];
    pre[v] = acc;
    acc = acc * den[v];
    ok = ok && f64_exp_within(den[v], 240u);
  }
  if (!any) {
#pragma unroll
    for (int v = 0; v < 4; ++v) z[v] = da[v] = db[v] = 0.0;
    return;
  }
  if (ok) {
    double inv = 1.0 / acc;
#pragma unroll
    for (int v = 3; v >= 0; --v) {
      iden[v] = inv * pre[v];
      inv = inv * den[v];
    }
  } else {
#pragma unroll
    for (int v = 0; v < 4; ++v) iden[v] = 1.0 / (den[v] + Lim<double>::tiny());
  }
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    if (!on[v]) { z[v] = da[v] = db[v] = 0.0; continue; }
    const double a2 = a[v] * a[v], b2 = b[v] * b[v], ab2 = 2.0 * a[v] * b[v];
    const double zz = (b[v] * a2 + a[v] * b2) * iden[v];
    z[v] = zz;
    da[v] = ((ab2 + b2) - zz * 2.0 * a[v]) * iden[v];
    db[v] = ((a2 + ab2) - zz * 2.0 * b[v]) * iden[v];
  }
}

// derivative of limit(kind, a, b) along the taken branch: *da, *db
template <class R> __host__ __device__ __forceinline__ void limit_grad(int kind, R a, R b, R* da, R* db) {
  const R tiny = Lim<R>::tiny();
  *da = R(0); *db = R(0);
  switch (kind) {
    case LIM_NOLIMIT1: return;
    case LIM_NOLIMIT2: *da = R(0.5); *db = R(0.5); return;
    case LIM_NOLIMIT3: *da = R(0.33333333333333333) * R(2); *db = R(0.33333333333333333); return;
    case LIM_VANALBADA: {
      if (a * b < R(0)) return;
      // z = num/den; dz = (dnum - z*dden)/den (no den^2: it underflows at a = b = 0)
      const R num = b * (a * a) + a * (b * b), den = a * a + b * b + tiny;
      const R iden = R(1) / den;
      const R z = num * iden;
      *da = ((R(2) * a * b + b * b) - z * R(2) * a) * iden;
      *db = ((a * a + R(2) * a * b) - z * R(2) * b) * iden;
      return;
    }
    case LIM_MINMOD:
      if (a > R(0)) { if (a <= fmax(b, R(0))) *da = R(1); else if (b > R(0)) *db = R(1); }
      else { if (a >= fmin(b, R(0))) *da = R(1); else if (b < R(0)) *db = R(1); }
      return;
    case LIM_VANLEER: {
      const R num = a * fabs(b) + fabs(a) * b, den = fabs(a) + fabs(b) + tiny;
      const R iden = R(1) / den;
      const R z = num * iden;
      *da = ((fabs(b) + sgn(a) * b) - z * sgn(a)) * iden;
      *db = ((a * sgn(b) + fabs(a)) - z * sgn(b)) * iden;
      return;
    }
    default: return;  // other limiters are not differentiated
  }
}

// Jacobian transposes of the primitive <-> conserved maps (the RK update
// cons(q0) + R*f -> prim): prim adjoint at state q -> conserved adjoint, and
// conserved adjoint at state q0 -> prim adjoint.
// (one reciprocal of the density and the gas's 1/(gamma-1) instead of four divisions: the
// reverse passes are bound by the FP64 pipe)
template <class R> __host__ __device__ __forceinline__ void cons2prim_adj(const Gas<R>& g, const R* q, const R* pb, R* cb) {
  const R u = q[0], v = q[1], ir = R(1) / q[2];
  cb[0] = pb[0] * ir - g.gm1 * u * pb[3];
  cb[1] = pb[1] * ir - g.gm1 * v * pb[3];
  cb[2] = pb[2] - (u * pb[0] + v * pb[1]) * ir + R(0.5) * g.gm1 * (u * u + v * v) * pb[3];
  cb[3] = g.gm1 * pb[3];
}
template <class R> __host__ __device__ __forceinline__ void prim2cons_adj(const Gas<R>& g, const R* q, const R* cb, R* pb) {
  const R u = q[0], v = q[1], r = q[2];
  pb[0] += r * cb[0] + r * u * cb[3];
  pb[1] += r * cb[1] + r * v * cb[3];
  pb[2] += u * cb[0] + v * cb[1] + cb[2] + R(0.5) * (u * u + v * v) * cb[3];
  pb[3] += cb[3] * g.gamma1;
}

}  // namespace hc
