// hc_oned.cu -- launchers of the one-dimensional stage kernels (FP64 and FP32, every
// flux) and the host-side 1D geometry: cells, face records and LSQ weights.
#include "hc_oned.cuh"
#include "hc_launch.h"

#include <vector>

namespace hc {

template <class R, int FK> static cudaError_t go1(const Stage1DArgs<R>& a, cudaStream_t s) {
  const unsigned grid = unsigned((a.nc + kTile1D - 1) / kTile1D);
  stage1d_kernel<R, FK><<<grid, kTile1D, 0, s>>>(a);
  return cudaGetLastError();
}

template <class R> static cudaError_t dispatch1(const Stage1DArgs<R>& a, int flux, cudaStream_t s) {
  switch (flux) {
    case FLUX_ROE: return go1<R, FLUX_ROE>(a, s);
    case FLUX_SLAU: return go1<R, FLUX_SLAU>(a, s);
    case FLUX_SLAU_REF: return go1<R, FLUX_SLAU_REF>(a, s);
    case FLUX_AUSMPUP: return go1<R, FLUX_AUSMPUP>(a, s);
    case FLUX_RUSANOV: return go1<R, FLUX_RUSANOV>(a, s);
    case FLUX_ROE_WS: return go1<R, FLUX_ROE_WS>(a, s);
    case FLUX_ROE_FACE: return go1<R, FLUX_ROE_FACE>(a, s);
    default: return go1<R, FLUX_CENTRAL>(a, s);
  }
}

template <> cudaError_t launch_stage1d<double>(const Stage1DArgs<double>& a, int flux, cudaStream_t s) {
  return dispatch1(a, flux, s);
}
template <> cudaError_t launch_stage1d<float>(const Stage1DArgs<float>& a, int flux, cudaStream_t s) {
  return dispatch1(a, flux, s);
}

// Cells (centre, length) and face records of a 1D mesh (nodes x[0..nc]); the LSQ metric of
// a cell sums the squared centre distances to its neighbours (the periodic pair across
// x[0] = x[nc] shifted by the period), plus the mirrored point at a non-periodic end
// (spatial/lsqMetrics.h:66-101); rec holds F1REC planes of nc + 1 faces.
void oned_geometry(const double* x, int nc, const int bc[2], std::vector<double>& rec, std::vector<double>& vol) {
  const bool per = bc[0] == BC_PERIODIC;
  const double L = x[nc] - x[0];
  std::vector<double> cx(nc), xm(nc, 0.0);
  vol.resize(nc);
  for (int i = 0; i < nc; ++i) { cx[i] = 0.5 * (x[i] + x[i + 1]); vol[i] = x[i + 1] - x[i]; }
  for (int i = 0; i < nc - 1; ++i) { const double d = cx[i + 1] - cx[i]; xm[i] += d * d; xm[i + 1] += d * d; }
  const double dper = cx[0] - (cx[nc - 1] - L);
  if (per) { xm[nc - 1] += dper * dper; xm[0] += dper * dper; }
  auto mirror = [&](int side) {
    const int c0 = side == 0 ? 0 : nc - 1, c1 = side == 0 ? 1 : nc - 2;
    const double disp = cx[c0] - cx[c1];
    const double bp = cx[c0] + disp;
    return bp - cx[c0];
  };
  if (!per)
    for (int side = 0; side < 2; ++side) { const double m = mirror(side); xm[side == 0 ? 0 : nc - 1] += m * m; }
  const size_t nf = size_t(nc) + 1;
  rec.assign(size_t(F1REC) * nf, 0.0);
  auto put = [&](int fld, int f, double v) { rec[size_t(fld) * nf + f] = v; };
  for (int f = 0; f <= nc; ++f) {
    const double xf = x[f];
    const bool bnd = (f == 0 || f == nc);
    if (!bnd || per) {
      const int l = (f == 0) ? nc - 1 : f - 1, r = (f == nc) ? 0 : f;
      double cl = cx[l], cr = cx[r];
      if (f == 0) cl -= L;
      if (f == nc) cr += L;
      const double dxc = (f == 0 || f == nc) ? dper : cr - cl;
      const double dl = std::sqrt((xf - cl) * (xf - cl)), dr = std::sqrt((cr - xf) * (cr - xf));
      put(F1_DL, f, dl);
      put(F1_DR, f, dr);
      put(F1_IDLR, f, 1. / (dl + dr));
      const double wl = 1. / (xm[l] - dxc * dxc), wr = 1. / (xm[r] - dxc * dxc);
      put(F1_WL, f, wl);
      put(F1_SL, f, dxc * wl);
      put(F1_WR, f, wr);
      put(F1_SR, f, dxc * wr);
      put(F1_DX, f, dxc);
    } else {
      const int side = f == 0 ? 0 : 1;
      const int c = side == 0 ? 0 : nc - 1;
      const double dd = std::sqrt((xf - cx[c]) * (xf - cx[c]));
      const double m = mirror(side);
      const double w = 1. / (xm[c] - m * m);
      put(F1_DL, f, dd);
      put(F1_IDLR, f, 1. / (dd + dd));
      put(side == 0 ? F1_WR : F1_WL, f, w);
      put(F1_WW, f, (1. / xm[c]) * (cx[c] - xf));
    }
  }
}

}  // namespace hc
