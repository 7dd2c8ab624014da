// hc_tangent.cuh -- forward-mode tangents on the device: Tan<T>{v, d} carries a value and
// its derivative along one input direction through the same templated physics code
// (hc_physics.cuh) that the stage kernels run.  Comparisons look at values only, so
// every switch of a flux takes the branch of the plain evaluation and the derivative is
// that branch's: max/min return the operand the plain code picks (the left one on a
// tie), |x| has derivative sign(x) and 0 at 0, sqrt has derivative 0 at 0.
//
// The discrete adjoint of the fluxes without a hand-written reverse (SLAU, AUSM+up,
// RoeUnprecWS) and of the Riemann and entropy far-field ghosts is built on it: eight
// tangent evaluations give the Jacobian's columns, F_bar . dF/dq_k the adjoint of each
// input.
#pragma once

#include "hc_physics.cuh"

namespace hc {
// its own namespace: the overloads below are found by argument-dependent lookup and do
// not hide the global ones for plain types inside namespace hc
namespace tg {

template <class T> struct Tan {
  T v, d;
  __host__ __device__ constexpr Tan() : v(T(0)), d(T(0)) {}
  __host__ __device__ constexpr Tan(double x) : v(T(x)), d(T(0)) {}
  __host__ __device__ constexpr Tan(T x, T dx) : v(x), d(dx) {}
};

template <class T> __host__ __device__ __forceinline__ Tan<T> operator+(Tan<T> a, Tan<T> b) {
  return {a.v + b.v, a.d + b.d};
}
template <class T> __host__ __device__ __forceinline__ Tan<T> operator-(Tan<T> a) { return {-a.v, -a.d}; }
template <class T> __host__ __device__ __forceinline__ Tan<T> operator-(Tan<T> a, Tan<T> b) {
  return {a.v - b.v, a.d - b.d};
}
template <class T> __host__ __device__ __forceinline__ Tan<T> operator*(Tan<T> a, Tan<T> b) {
  return {a.v * b.v, a.d * b.v + a.v * b.d};
}
template <class T> __host__ __device__ __forceinline__ Tan<T> operator/(Tan<T> a, Tan<T> b) {
  const T q = a.v / b.v;
  return {q, (a.d - q * b.d) / b.v};
}
template <class T> __host__ __device__ __forceinline__ Tan<T>& operator+=(Tan<T>& a, Tan<T> b) { return a = a + b; }
template <class T> __host__ __device__ __forceinline__ Tan<T>& operator-=(Tan<T>& a, Tan<T> b) { return a = a - b; }
template <class T> __host__ __device__ __forceinline__ Tan<T>& operator*=(Tan<T>& a, Tan<T> b) { return a = a * b; }
template <class T> __host__ __device__ __forceinline__ Tan<T>& operator/=(Tan<T>& a, Tan<T> b) { return a = a / b; }

template <class T> __host__ __device__ __forceinline__ bool operator<(Tan<T> a, Tan<T> b) { return a.v < b.v; }
template <class T> __host__ __device__ __forceinline__ bool operator>(Tan<T> a, Tan<T> b) { return a.v > b.v; }
template <class T> __host__ __device__ __forceinline__ bool operator<=(Tan<T> a, Tan<T> b) { return a.v <= b.v; }
template <class T> __host__ __device__ __forceinline__ bool operator>=(Tan<T> a, Tan<T> b) { return a.v >= b.v; }
template <class T> __host__ __device__ __forceinline__ bool operator==(Tan<T> a, Tan<T> b) { return a.v == b.v; }
template <class T> __host__ __device__ __forceinline__ bool operator!=(Tan<T> a, Tan<T> b) { return a.v != b.v; }

template <class T> __host__ __device__ __forceinline__ Tan<T> fabs(Tan<T> x) {
  return x.v < T(0) ? -x : (x.v > T(0) ? x : Tan<T>(T(0), T(0)));
}
template <class T> __host__ __device__ __forceinline__ Tan<T> fmax(Tan<T> a, Tan<T> b) { return (a.v < b.v) ? b : a; }
template <class T> __host__ __device__ __forceinline__ Tan<T> fmin(Tan<T> a, Tan<T> b) { return (b.v < a.v) ? b : a; }
template <class T> __host__ __device__ __forceinline__ Tan<T> sqrt(Tan<T> x) {
  using ::sqrt;
  const T s = sqrt(x.v);
  return {s, s > T(0) ? T(0.5) * x.d / s : T(0)};
}
// d(a^b) = b a^(b-1) da + a^b ln(a) db; the terms with a zero tangent are skipped
template <class T> __host__ __device__ __forceinline__ Tan<T> pow(Tan<T> a, Tan<T> b) {
  using ::log;
  using ::pow;
  const T p = pow(a.v, b.v);
  T d = T(0);
  if (a.d != T(0) && a.v != T(0)) d += b.v * (p / a.v) * a.d;
  if (b.d != T(0) && a.v > T(0)) d += p * log(a.v) * b.d;
  return {p, d};
}
template <class T> __host__ __device__ __forceinline__ bool isfinite(Tan<T> x) {
  using ::isfinite;
  return isfinite(x.v);
}

}  // namespace tg
using tg::Tan;

template <class T> struct Lim<Tan<T>> {
  __host__ __device__ static constexpr Tan<T> tiny() { return Tan<T>(Lim<T>::tiny(), T(0)); }
  __host__ __device__ static constexpr Tan<T> huge() { return Tan<T>(Lim<T>::huge(), T(0)); }
};

// Reverse of face_flux<R, FK> on two primitive states by eight tangent evaluations:
// qlb[k] += Fb . dF/dql[k], qrb[k] += Fb . dF/dqr[k] for the four conserved flux
// components (the spectral radius feeds only the frozen timestep).
template <class R> __host__ __device__ __forceinline__ Gas<Tan<R>> tan_gas(const Gas<R>& g) {
  using T = Tan<R>;
  Gas<T> gt;
  gt.gamma = T(g.gamma, R(0)); gt.gm1 = T(g.gm1, R(0)); gt.gamma1 = T(g.gamma1, R(0));
  gt.Rgas = T(g.Rgas, R(0)); gt.minf = T(g.minf, R(0)); gt.inv_gamma = T(g.inv_gamma, R(0));
  gt.lref_dt = T(g.lref_dt, R(0)); gt.vscale = g.vscale; gt.pscale = g.pscale; gt.fixes = g.fixes;
  return gt;
}

template <class R, int FK>
__host__ __device__ __forceinline__ void tangent_flux_adj(const Gas<R>& g, R nx, R ny, R A, const R* ql,
                                                          const R* qr, const R* Fb, R* qlb, R* qrb) {
  using T = Tan<R>;
  const Gas<T> gt = tan_gas(g);
  const T tnx(nx, R(0)), tny(ny, R(0)), tA(A, R(0));
#pragma unroll 1
  for (int k = 0; k < 8; ++k) {
    T l[4], r[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      l[v] = T(ql[v], k == v ? R(1) : R(0));
      r[v] = T(qr[v], k == 4 + v ? R(1) : R(0));
    }
    const St<T> sl = prim_state(gt, l[0], l[1], l[2], l[3]);
    const St<T> sr = prim_state(gt, r[0], r[1], r[2], r[3]);
    const Flux5<T> F = face_flux<T, FK>(gt, tnx, tny, tA, sl, sr);
    R s = R(0);
#pragma unroll
    for (int v = 0; v < 4; ++v) s += Fb[v] * F.f[v].d;
    if (k < 4) qlb[k] += s;
    else qrb[k - 4] += s;
  }
}

// Reverse of farfield_update<R, BK> (Riemann or entropy far-field ghost of the primitive
// basis; (nx, ny) into the domain) by eight tangent evaluations: given gb, the adjoint of
// the ghost state, qib += gb . dG/dqi and qfb += gb . dG/dqf.
template <class R, int BK>
__host__ __device__ __forceinline__ void farfield_adj(const Gas<R>& g, R nx, R ny, const R* qi, const R* qf,
                                                      const R* gb, R* qib, R* qfb) {
  using T = Tan<R>;
  const Gas<T> gt = tan_gas(g);
  const T tnx(nx, R(0)), tny(ny, R(0));
#pragma unroll 1
  for (int k = 0; k < 8; ++k) {
    T ti[4], tf[4], qb[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      ti[v] = T(qi[v], k == v ? R(1) : R(0));
      tf[v] = T(qf[v], k == 4 + v ? R(1) : R(0));
    }
    farfield_update<T, BK>(gt, tnx, tny, ti, tf, qb);
    R s = R(0);
#pragma unroll
    for (int v = 0; v < 4; ++v) s += gb[v] * qb[v].d;
    if (k < 4) qib[k] += s;
    else qfb[k - 4] += s;
  }
}

}  // namespace hc
