// hc_geometry.cuh -- once-per-mesh geometry kernels (always FP64): cell
// volumes and centres, face normals and areas, and the least-squares metrics
// folded into per-face gradient weights.  Included by hc_api.cu only.
#pragma once

#include "hc_kernels.cuh"

namespace hc {

// ---------------------------------------------------------------- geometry (FP64)
__device__ __forceinline__ void node_at(const double* nodes, int nj, int i, int j, double* p) {
  const size_t k = (size_t(i) * (nj + 1) + j) * 2;
  p[0] = nodes[k]; p[1] = nodes[k + 1];
}

// geom::surface (geometry/surface.ipp:12-29)
__device__ __forceinline__ void surface_dev(const double* p0, const double* p1, double* n, double* A, double* c) {
  const double t0x = p1[0] - p0[0], t0y = p1[1] - p0[1];
  const double t1x = p0[0] - p1[0], t1y = p0[1] - p1[1];
  double d = t0x * t0x;
  d += t0y * t0y;
  const double l = sqrt(d);
  const double l1 = 1. / l;
  *A = l;
  c[0] = p0[0] + 0.5 * t0x;
  c[1] = p0[1] + 0.5 * t0y;
  n[0] = -(l1 * t1y);
  n[1] = l1 * t1x;
}

// cell volume |J(0,0)| of the bilinear map and the vertex centroid (geometry/volume.ipp:25-66)
__global__ void geom_cells_kernel(const double* __restrict__ nodes, int ni, int nj, double* __restrict__ vol,
                                  double* __restrict__ cx, double* __restrict__ cy) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ni * nj) return;
  const int i = c / nj, j = c % nj;
  double p[4][2];
  node_at(nodes, nj, i, j, p[0]);
  node_at(nodes, nj, i + 1, j, p[1]);
  node_at(nodes, nj, i, j + 1, p[2]);
  node_at(nodes, nj, i + 1, j + 1, p[3]);
  const double du[4][2] = {{-0.25, -0.25}, {0.25, -0.25}, {-0.25, 0.25}, {0.25, 0.25}};
  double com[2], tg[2][2] = {{0, 0}, {0, 0}};
  for (int d = 0; d < 2; ++d) {
    double s = 0;
    for (int k = 0; k < 4; ++k) s += 0.25 * p[k][d];
    com[d] = s;
  }
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b)
      for (int k = 0; k < 4; ++k) tg[a][b] += du[k][a] * p[k][b];
  vol[c] = fabs(tg[0][0] * tg[1][1] - tg[0][1] * tg[1][0]);
  cx[c] = com[0];
  cy[c] = com[1];
}

struct GeomArgs {
  const double* nodes;
  int ni, nj;
  int bc[4];
  const double* cx;
  const double* cy;
  double* fi;   // (ni+1)*nj records
  double* fj;   // ni*(nj+1) records
  double* xm;   // 3 planes per cell
};

// Face pass 1: normal, area, and the centre distances of the two cells (with
// the periodic image of the far cell on wrap faces, D2; the mirrored ghost
// centre on the other boundary faces, D4).
__global__ void geom_faces1_kernel(GeomArgs g, int dir) {
  const int ni = g.ni, nj = g.nj;
  const int nf = dir == 0 ? (ni + 1) * nj : ni * (nj + 1);
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  double* rec = dir == 0 ? g.fi : g.fj;
  int i, j;
  if (dir == 0) { i = f / nj; j = f % nj; } else { i = f / (nj + 1); j = f % (nj + 1); }
  const int lo = dir == 0 ? i : j;
  const int n_along = dir == 0 ? ni : nj;
  const int side_lo = dir == 0 ? 0 : 2;
  const bool periodic = g.bc[side_lo] == BC_PERIODIC;
  const bool at_lo = lo == 0, at_hi = lo == n_along;
  // face nodes (residualCalc.h:211-213, 239-241; periodic faces use the low node line)
  double p0[2], p1[2];
  const int lo_use = (periodic && at_hi) ? 0 : lo;
  if (dir == 0) { node_at(g.nodes, nj, lo_use, j, p0); node_at(g.nodes, nj, lo_use, j + 1, p1); }
  else { node_at(g.nodes, nj, i + 1, lo_use, p0); node_at(g.nodes, nj, i, lo_use, p1); }
  double n[2], A, fc[2];
  surface_dev(p0, p1, n, &A, fc);
  double r[FREC];
  for (int k = 0; k < FREC; ++k) r[k] = 0;
  r[F_NX] = n[0]; r[F_NY] = n[1]; r[F_A] = A;
  auto cidx = [&](int a, int b) { return size_t(a) * nj + b; };
  if (!at_lo && !at_hi) {
    const size_t L = dir == 0 ? cidx(i - 1, j) : cidx(i, j - 1);
    const size_t Rr = cidx(i, j);
    const double cl[2] = {g.cx[L], g.cy[L]}, cr[2] = {g.cx[Rr], g.cy[Rr]};
    double d = (fc[0] - cl[0]) * (fc[0] - cl[0]);
    d += (fc[1] - cl[1]) * (fc[1] - cl[1]);
    r[F_DL] = sqrt(d);
    d = (cr[0] - fc[0]) * (cr[0] - fc[0]);
    d += (cr[1] - fc[1]) * (cr[1] - fc[1]);
    r[F_DR] = sqrt(d);
    r[F_DXX] = cr[0] - cl[0];
    r[F_DXY] = cr[1] - cl[1];
  } else if (periodic) {
    // wrap face between the last cell (image) and the first cell
    size_t L, Rr;
    double s[2], a0[2], a1[2], b0[2], b1[2];
    if (dir == 0) {
      L = cidx(ni - 1, j); Rr = cidx(0, j);
      node_at(g.nodes, nj, ni, j, a0); node_at(g.nodes, nj, 0, j, b0);
      node_at(g.nodes, nj, ni, j + 1, a1); node_at(g.nodes, nj, 0, j + 1, b1);
    } else {
      L = cidx(i, nj - 1); Rr = cidx(i, 0);
      node_at(g.nodes, nj, i, nj, a0); node_at(g.nodes, nj, i, 0, b0);
      node_at(g.nodes, nj, i + 1, nj, a1); node_at(g.nodes, nj, i + 1, 0, b1);
    }
    for (int k = 0; k < 2; ++k) s[k] = 0.5 * ((a0[k] - b0[k]) + (a1[k] - b1[k]));
    const double cl[2] = {g.cx[L] - s[0], g.cy[L] - s[1]}, cr[2] = {g.cx[Rr], g.cy[Rr]};
    double d = (fc[0] - cl[0]) * (fc[0] - cl[0]);
    d += (fc[1] - cl[1]) * (fc[1] - cl[1]);
    r[F_DL] = sqrt(d);
    d = (cr[0] - fc[0]) * (cr[0] - fc[0]);
    d += (cr[1] - fc[1]) * (cr[1] - fc[1]);
    r[F_DR] = sqrt(d);
    r[F_DXX] = cr[0] - cl[0];
    r[F_DXY] = cr[1] - cl[1];
  } else {
    // ghost/wall face: distance from the interior centre; no pair contribution
    const size_t c = at_lo ? cidx(i, j) : (dir == 0 ? cidx(ni - 1, j) : cidx(i, nj - 1));
    double d = (fc[0] - g.cx[c]) * (fc[0] - g.cx[c]);
    d += (fc[1] - g.cy[c]) * (fc[1] - g.cy[c]);
    const double dd = sqrt(d);
    r[F_DL] = dd; r[F_DR] = dd;
  }
  r[F_IDLR] = 1. / (r[F_DL] + r[F_DR]);
  for (int k = 0; k < FREC; ++k) rec[size_t(k) * nf + f] = r[k];
}

__device__ __forceinline__ void xm_add(double* x, double dx, double dy) {
  x[0] += dx * dx; x[1] += dx * dy; x[2] += dy * dy;
}

// mirrored-point displacement of boundary cell (a,b) away from its neighbour
// (na,nb) (spatial/lsqMetrics.h:119-123)
__device__ __forceinline__ void mirror_disp(const GeomArgs& g, size_t c0, size_t c1, double* m) {
  const double x0[2] = {g.cx[c0], g.cy[c0]}, x1[2] = {g.cx[c1], g.cy[c1]};
  for (int k = 0; k < 2; ++k) {
    const double disp = x0[k] - x1[k];
    const double bp = x0[k] + disp;
    m[k] = bp - x0[k];
  }
}

// Cell pass: full xmetric = pair terms of the 4 faces + mirror terms on
// non-periodic sides (spatial/lsqMetrics.h:31-163, D2).
__global__ void geom_xm_kernel(GeomArgs g) {
  const int ni = g.ni, nj = g.nj;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ni * nj) return;
  const int i = c / nj, j = c % nj;
  const int nfi = (ni + 1) * nj, nfj = ni * (nj + 1);
  double x[3] = {0, 0, 0};
  const int fis[2] = {i * nj + j, (i + 1) * nj + j};
  const int fjs[2] = {i * (nj + 1) + j, i * (nj + 1) + j + 1};
  const bool per_i = g.bc[0] == BC_PERIODIC, per_j = g.bc[2] == BC_PERIODIC;
  for (int k = 0; k < 2; ++k) {
    const int fi = fis[k];
    const int il = fi / nj;
    if ((il > 0 && il < ni) || per_i) xm_add(x, g.fi[size_t(F_DXX) * nfi + fi], g.fi[size_t(F_DXY) * nfi + fi]);
  }
  for (int k = 0; k < 2; ++k) {
    const int fj = fjs[k];
    const int jl = fj % (nj + 1);
    if ((jl > 0 && jl < nj) || per_j) xm_add(x, g.fj[size_t(F_DXX) * nfj + fj], g.fj[size_t(F_DXY) * nfj + fj]);
  }
  double m[2];
  if (!per_i) {
    if (i == 0) { mirror_disp(g, c, size_t(1) * nj + j, m); xm_add(x, m[0], m[1]); }
    if (i == ni - 1) { mirror_disp(g, c, size_t(ni - 2) * nj + j, m); xm_add(x, m[0], m[1]); }
  }
  if (g.bc[2] != BC_PERIODIC) {
    if (j == 0) { mirror_disp(g, c, size_t(i) * nj + 1, m); xm_add(x, m[0], m[1]); }
    if (j == nj - 1) { mirror_disp(g, c, size_t(i) * nj + nj - 2, m); xm_add(x, m[0], m[1]); }
  }
  const size_t n = size_t(ni) * nj;
  g.xm[c] = x[0]; g.xm[n + c] = x[1]; g.xm[2 * n + c] = x[2];
}

// factor the 2x2 metric and project on direction d: w = X^-1 d (lsq/factor_solve.ipp:13-22, 47-69)
__device__ __forceinline__ void weights(const double* x, const double* d, double* w) {
  const double det = 1. / (x[0] * x[2] - x[1] * x[1]);
  const double f0 = det * x[2], f1 = -det * x[1], f2 = det * x[0];
  w[0] = f0 * d[0] + f1 * d[1];
  w[1] = f1 * d[0] + f2 * d[1];
}

// Face pass 2: biased-gradient weights of both cells (lsq::bias_solves,
// lsq/factor_solve.ipp:71-100) and, on wall faces, the extrapolation weights of the
// interior cell's full gradient (D4).
__global__ void geom_faces2_kernel(GeomArgs g, int dir) {
  const int ni = g.ni, nj = g.nj;
  const int nf = dir == 0 ? (ni + 1) * nj : ni * (nj + 1);
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  double* rec = dir == 0 ? g.fi : g.fj;
  int i, j;
  if (dir == 0) { i = f / nj; j = f % nj; } else { i = f / (nj + 1); j = f % (nj + 1); }
  const int lo = dir == 0 ? i : j;
  const int n_along = dir == 0 ? ni : nj;
  const int side_lo = dir == 0 ? 0 : 2;
  const bool periodic = g.bc[side_lo] == BC_PERIODIC;
  const bool at_lo = lo == 0, at_hi = lo == n_along;
  const size_t n = size_t(ni) * nj;
  auto R = [&](int k) -> double& { return rec[size_t(k) * nf + f]; };
  auto cidx = [&](int a, int b) { return size_t(a) * nj + b; };
  const double nn[2] = {R(F_NX), R(F_NY)};
  if ((!at_lo && !at_hi) || periodic) {
    size_t L, Rr;
    if (!at_lo && !at_hi) {
      L = dir == 0 ? cidx(i - 1, j) : cidx(i, j - 1);
      Rr = cidx(i, j);
    } else {
      L = dir == 0 ? cidx(ni - 1, j) : cidx(i, nj - 1);
      Rr = dir == 0 ? cidx(0, j) : cidx(i, 0);
    }
    const double dx = R(F_DXX), dy = R(F_DXY);
    double xl[3] = {g.xm[L] - dx * dx, g.xm[n + L] - dx * dy, g.xm[2 * n + L] - dy * dy};
    double xr[3] = {g.xm[Rr] - dx * dx, g.xm[n + Rr] - dx * dy, g.xm[2 * n + Rr] - dy * dy};
    double w[2];
    weights(xl, nn, w);
    R(F_WLX) = w[0]; R(F_WLY) = w[1]; R(F_SL) = dx * w[0] + dy * w[1];
    weights(xr, nn, w);
    R(F_WRX) = w[0]; R(F_WRY) = w[1]; R(F_SR) = dx * w[0] + dy * w[1];
    return;
  }
  // boundary face of a non-periodic side
  const size_t c = at_lo ? cidx(i, j) : (dir == 0 ? cidx(ni - 1, j) : cidx(i, nj - 1));
  size_t cn;  // interior neighbour opposite the boundary
  if (dir == 0) cn = at_lo ? cidx(1, j) : cidx(ni - 2, j);
  else cn = at_lo ? cidx(i, 1) : cidx(i, nj - 2);
  double m[2];
  mirror_disp(g, c, cn, m);
  const double xf[3] = {g.xm[c], g.xm[n + c], g.xm[2 * n + c]};
  const double xb[3] = {xf[0] - m[0] * m[0], xf[1] - m[0] * m[1], xf[2] - m[1] * m[1]};
  double w[2];
  weights(xb, nn, w);
  // wall extrapolation direction: cell centre minus the centre of the face as
  // seen from the domain (boundaryFluxLoop.h:150-261 node order)
  double p0[2], p1[2];
  if (dir == 0) {
    if (at_lo) { node_at(g.nodes, nj, 0, j, p0); node_at(g.nodes, nj, 0, j + 1, p1); }
    else { node_at(g.nodes, nj, ni, j + 1, p0); node_at(g.nodes, nj, ni, j, p1); }
  } else {
    if (at_lo) { node_at(g.nodes, nj, i + 1, 0, p0); node_at(g.nodes, nj, i, 0, p1); }
    else { node_at(g.nodes, nj, i, nj, p0); node_at(g.nodes, nj, i + 1, nj, p1); }
  }
  double nin[2], Ain, fcin[2];
  surface_dev(p0, p1, nin, &Ain, fcin);
  const double dvec[2] = {g.cx[c] - fcin[0], g.cy[c] - fcin[1]};
  double ww[2];
  weights(xf, dvec, ww);
  if (at_lo) {  // interior cell is the right cell
    R(F_WRX) = w[0]; R(F_WRY) = w[1]; R(F_SR) = 0;
    R(F_WLX) = ww[0]; R(F_WLY) = ww[1]; R(F_SL) = 0;
  } else {      // interior cell is the left cell
    R(F_WLX) = w[0]; R(F_WLY) = w[1]; R(F_SL) = 0;
    R(F_WRX) = ww[0]; R(F_WRY) = ww[1]; R(F_SR) = 0;
  }
}

}  // namespace hc
