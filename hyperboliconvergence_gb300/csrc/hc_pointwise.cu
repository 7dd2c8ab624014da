// hc_pointwise.cu -- host evaluation of one interface flux and one slope limiter with the
// pointwise functions the stage kernels compile (hc_physics.cuh, its host path), for the
// C++ adapter's flux and limiter tags (the reference's FluxFunctor and
// VariableLimiterInterface plug-in points) and for checks.  No device work.
#include "hc_host.h"

using namespace hc;

namespace {

template <int FK> Flux5<double> flux_of(const Gas<double>& g, const double* f, const St<double>& l, const St<double>& r) {
  return face_flux<double, FK>(g, f[3], f[4], f[0], l, r);
}

}  // namespace

extern "C" {

int hc_flux_eval(int flux, int vscale, int pscale, const double species[5], const double face[7], const double ql[4],
                 const double qr[4], double out5[5]) {
  if (!species || !face || !ql || !qr || !out5) return fail(HC_ERR_ARG, "null pointer");
  if (flux < 0 || flux >= FLUX_COUNT) return fail(HC_ERR_ARG, "unknown flux");
  if (!(species[0] > 1.0) || !(species[1] > 0.0) || !(species[3] > 0.0) || !(species[4] > 0.0))
    return fail(HC_ERR_ARG, "invalid species");
  auto ok = [](int k) { return k >= SCALING_CONVECTIVE && k <= SCALING_ADAPTIVE; };
  if (!ok(vscale) || !ok(pscale)) return fail(HC_ERR_ARG, "unknown low-Mach scaling");
  const Gas<double> g = make_gas<double>(species[0], species[1], species[2], species[3], species[4], vscale, pscale);
  const St<double> l = prim_state(g, ql[0], ql[1], ql[2], ql[3]);
  const St<double> r = prim_state(g, qr[0], qr[1], qr[2], qr[3]);
  Flux5<double> o;
  switch (flux) {
    case FLUX_ROE: o = flux_of<FLUX_ROE>(g, face, l, r); break;
    case FLUX_SLAU: o = flux_of<FLUX_SLAU>(g, face, l, r); break;
    case FLUX_SLAU_REF: o = flux_of<FLUX_SLAU_REF>(g, face, l, r); break;
    case FLUX_AUSMPUP: o = flux_of<FLUX_AUSMPUP>(g, face, l, r); break;
    case FLUX_RUSANOV: o = flux_of<FLUX_RUSANOV>(g, face, l, r); break;
    case FLUX_ROE_WS: o = flux_of<FLUX_ROE_WS>(g, face, l, r); break;
    case FLUX_ROE_FACE: o = flux_of<FLUX_ROE_FACE>(g, face, l, r); break;
    default: o = flux_of<FLUX_CENTRAL>(g, face, l, r); break;
  }
  for (int v = 0; v < 4; ++v) out5[v] = o.f[v];
  out5[4] = o.lam;
  return HC_OK;
}

int hc_limit_eval(int limiter, double a, double b, double* out) {
  if (!out) return fail(HC_ERR_ARG, "null pointer");
  if (limiter < 0 || limiter >= LIM_COUNT) return fail(HC_ERR_ARG, "unknown limiter");
  *out = limit<double>(limiter, a, b);
  return HC_OK;
}

}  // extern "C"
