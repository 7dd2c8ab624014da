// hc_oracle_1d.hpp -- CPU oracle of the one-dimensional Euler path.
//
// TEST INFRASTRUCTURE ONLY (see hc_oracle.hpp).  The reference's 1D glue
// (interiorResidual, spatial/residualCalc.h:74-127; boundary_xmetrics,
// spatial/lsqMetrics.h:66-101; the 1D ghost-cell, periodic and boundary-flux loops,
// spatial/boundary/ghostCellLoop.h:28-89, periodicLoop.h:28-75,
// boundaryFluxLoop.h:30-90; boundaryUpdate, spatial/boundary/boundaryUpdate.h:76-133)
// is restated with the decisions of the 2D oracle (D2 LSQ stencil with periodic wrap
// or mirrored points, D4 ghost faces).  The pointwise physics is the 2D oracle's with
// the second velocity 0 and face normals (+-1, 0): the reference's own nDim = 1 fluxes
// and boundary updates equal it bit for bit (tests/golden: flux_1d_*, bc_1d_*).
// State: primitive {u, rho, p} per cell.
#pragma once

#include "hc_oracle.hpp"

#include <vector>

namespace hco {

template <class R> struct Solver1D {
  int nc = 0;
  std::vector<R> x;  // nc + 1 nodes
  Species<R> sp{};
  int flux = FLUX_ROE, lim = LIM_VANLEER, rk = RK_SSP34, dtmode = DT_GLOBAL;
  R cfl = 0.5;
  int bc[2] = {BC_PERIODIC, BC_PERIODIC};
  R ref[2][3] = {{0, 0, 0}, {0, 0, 0}};  // far-field / fixed reference values per side
  R ghost[2][3] = {{0, 0, 0}, {0, 0, 0}};
  std::vector<R> cx, vol, xm, q0, q1, q2, lam0;
  std::vector<std::array<R, 4>> res[4];  // flux sums (rho u, rho, rho E) and lambda sum
  std::vector<std::array<R, 3>> qm;
  R t = 0, last_dt = 0;

  static void emb(const R* q3, R* q4) { q4[0] = q3[0]; q4[1] = 0; q4[2] = q3[1]; q4[3] = q3[2]; }
  // the face of a node: area 1, normal n (geometry/surface.ipp:4-11; flip for -1)
  static Face<R> face(R xf, R n) {
    Face<R> f;
    f.area = 1; f.c[0] = xf; f.c[1] = 0; f.n[0] = n; f.n[1] = 0; f.t[0] = 0; f.t[1] = n;
    return f;
  }
  FluxRes<R> flux_of(const Face<R>& f, const R* ql, const R* qr) const {
    R l[4], r[4];
    emb(ql, l); emb(qr, r);
    return face_flux(flux, sp, f, prim2state(sp, l), prim2state(sp, r));
  }
  R period() const { return x[nc] - x[0]; }
  R mirror(int side) const {
    const int c0 = side == 0 ? 0 : nc - 1, c1 = side == 0 ? 1 : nc - 2;
    const R disp = cx[c0] - cx[c1];
    const R bp = cx[c0] + disp;
    return bp - cx[c0];
  }

  void setup() {
    cx.resize(nc); vol.resize(nc);
    for (int i = 0; i < nc; ++i) { cx[i] = 0.5 * (x[i] + x[i + 1]); vol[i] = x[i + 1] - x[i]; }
    // xmetrics: neighbour pairs, the periodic pair (D2), mirrored points at other ends
    xm.assign(nc, R(0));
    for (int i = 0; i < nc - 1; ++i) { const R d = cx[i + 1] - cx[i]; xm[i] += d * d; xm[i + 1] += d * d; }
    if (bc[0] == BC_PERIODIC) { const R d = cx[0] - (cx[nc - 1] - period()); xm[nc - 1] += d * d; xm[0] += d * d; }
    for (int side = 0; side < 2; ++side)
      if (bc[side] != BC_PERIODIC) { const R m = mirror(side); xm[side == 0 ? 0 : nc - 1] += m * m; }
    const size_t n = size_t(nc);
    q0.assign(3 * n, 0); q1.assign(3 * n, 0); q2.assign(3 * n, 0); lam0.assign(n, 0);
    for (auto& r : res) r.assign(n, {0, 0, 0, 0});
    qm.assign(n, {0, 0, 0});
  }

  void boundary_update(const std::vector<R>& q) {
    for (int side = 0; side < 2; ++side) {
      if (bc[side] == BC_PERIODIC) continue;
      const int c = side == 0 ? 0 : nc - 1;
      if (bc[side] == BC_RIEMANN || bc[side] == BC_ENTROPY) {
        R qi[4], qf[4], qb[4];
        emb(&q[3 * c], qi); emb(ref[side], qf);
        const Face<R> f = face(x[side == 0 ? 0 : nc], side == 0 ? R(1) : R(-1));  // into the domain
        if (bc[side] == BC_RIEMANN) bc_riemann(sp, f, qi, qf, qb);
        else bc_entropy(sp, f, qi, qf, qb);
        ghost[side][0] = qb[0]; ghost[side][1] = qb[2]; ghost[side][2] = qb[3];
      } else {
        for (int v = 0; v < 3; ++v) ghost[side][v] = ref[side][v];
      }
    }
  }

  void qmetrics(const std::vector<R>& q) {
    for (auto& m : qm) m = {0, 0, 0};
    auto pair = [&](int a, int b, R d) {
      for (int v = 0; v < 3; ++v) { const R dq = (q[3 * b + v] - q[3 * a + v]) * d; qm[a][v] += dq; qm[b][v] += dq; }
    };
    for (int i = 0; i < nc - 1; ++i) pair(i, i + 1, cx[i + 1] - cx[i]);
    if (bc[0] == BC_PERIODIC) pair(nc - 1, 0, cx[0] - (cx[nc - 1] - period()));
  }

  // make_muscl_flux (spatial/muscl.h:13-59) across the face at node xf between cells with
  // centres cl < xf < cr, normal +1
  FluxRes<R> muscl(R xf, R cl, R cr, const R* ql, const R* qr, R xl, R xr, const std::array<R, 3>& ml,
                   const std::array<R, 3>& mr) const {
    const Face<R> f = face(xf, R(1));
    if (lim == LIM_NOLIMIT1) return flux_of(f, ql, qr);
    const R dxc = cr - cl;
    const R dl = sqrt((xf - cl) * (xf - cl)), dr = sqrt((cr - xf) * (cr - xf));
    const R idlr = 1. / (dl + dr);
    const R xbl = xl - dxc * dxc, xbr = xr - dxc * dxc;
    R qL[3], qR[3];
    for (int v = 0; v < 3; ++v) {
      const R dq = qr[v] - ql[v];
      const R gc = dq * idlr;
      const R gl = (1. / xbl) * (ml[v] - dq * dxc);
      const R gr = (1. / xbr) * (mr[v] - dq * dxc);
      qL[v] = ql[v] + dl * limit<R>(lim, gc, gl);
      qR[v] = qr[v] - dr * limit<R>(lim, gc, gr);
    }
    return flux_of(f, qL, qR);
  }

  // ghost face (D4): the ghost side unreconstructed, the interior side MUSCL with the
  // mirrored point removed from its xmetric
  FluxRes<R> muscl_ghost(int side) const {
    const int c = side == 0 ? 0 : nc - 1;
    const R xf = x[side == 0 ? 0 : nc];
    const Face<R> f = face(xf, R(1));
    const R* qi = &q_eval[3 * c];
    const R* qg = ghost[side];
    const bool ghost_left = side == 0;
    const R* ql = ghost_left ? qg : qi;
    const R* qr = ghost_left ? qi : qg;
    if (lim == LIM_NOLIMIT1) return flux_of(f, ql, qr);
    const R dd = sqrt((xf - cx[c]) * (xf - cx[c]));
    const R idlr = 1. / (dd + dd);
    const R m = mirror(side);
    const R xb = xm[c] - m * m;
    R qL[3], qR[3];
    for (int v = 0; v < 3; ++v) {
      const R dq = qr[v] - ql[v];
      const R g = (1. / xb) * qm[c][v];
      const R s = limit<R>(lim, dq * idlr, g);
      if (ghost_left) { qL[v] = qg[v]; qR[v] = qi[v] - dd * s; }
      else { qL[v] = qi[v] + dd * s; qR[v] = qg[v]; }
    }
    return flux_of(f, qL, qR);
  }
  std::vector<R> q_eval;  // the state of the residual being evaluated

  static void sub(std::array<R, 4>& a, const FluxRes<R>& f) { a[0] -= f.f[0]; a[1] -= f.f[2]; a[2] -= f.f[3]; a[3] += f.lam; }
  static void add(std::array<R, 4>& a, const FluxRes<R>& f) { a[0] += f.f[0]; a[1] += f.f[2]; a[2] += f.f[3]; a[3] += f.lam; }

  void residual(const std::vector<R>& q, std::vector<std::array<R, 4>>& r) {
    q_eval = q;
    boundary_update(q);
    qmetrics(q);
    for (auto& v : r) v = {0, 0, 0, 0};
    for (int i = 1; i < nc; ++i) {  // interior faces (spatial/residualCalc.h:110-124)
      const FluxRes<R> f = muscl(x[i], cx[i - 1], cx[i], &q[3 * (i - 1)], &q[3 * i], xm[i - 1], xm[i], qm[i - 1], qm[i]);
      sub(r[i - 1], f); add(r[i], f);
    }
    for (int side = 0; side < 2; ++side) {
      const int t = bc[side];
      if (t == BC_PERIODIC) {
        if (side == 1) continue;  // the lower face of the pair only (periodicLoop.h:50-72)
        const FluxRes<R> f = muscl(x[0], cx[nc - 1] - period(), cx[0], &q[3 * (nc - 1)], &q[0], xm[nc - 1], xm[0],
                                   qm[nc - 1], qm[0]);
        sub(r[nc - 1], f); add(r[0], f);
      } else if (t == BC_WALL) {
        // pressure flux of the interior state moved to the face (inviscidWall.ipp:33-72),
        // normal into the domain, res += F
        const int c = side == 0 ? 0 : nc - 1;
        const R xf = x[side == 0 ? 0 : nc];
        const R dir = cx[c] - xf;
        R qi[4], dq4[4];
        emb(&q[3 * c], qi);
        const R w = 1. / xm[c];
        const R g[3] = {w * qm[c][0], w * qm[c][1], w * qm[c][2]};
        const R d3[3] = {g[0] * dir, g[1] * dir, g[2] * dir};
        emb(d3, dq4);
        add(r[c], wall_flux(sp, face(xf, side == 0 ? R(1) : R(-1)), qi, dq4));
      } else {
        const FluxRes<R> f = muscl_ghost(side);
        if (side == 0) add(r[0], f); else sub(r[nc - 1], f);
      }
    }
  }

  R spectral_radius(const std::vector<std::array<R, 4>>& r) const {
    R m = std::numeric_limits<R>::min();
    for (int c = 0; c < nc; ++c) m = std::max(m, r[c][3] / vol[c]);
    return m;
  }

  void step(int nsteps) {
    const RKTable<R> tab = rk_table<R>(rk);
    const size_t n = size_t(nc);
    for (int st = 0; st < nsteps; ++st) {
      R dt = 0;
      q1 = q0;
      for (int s = 0; s < tab.nstages; ++s) {
        residual(q1, res[s]);
        if (s == 0) {
          if (dtmode == DT_GLOBAL) dt = cfl / spectral_radius(res[0]);
          else for (size_t c = 0; c < n; ++c) lam0[c] = res[0][c][3];
        }
        for (size_t c = 0; c < n; ++c) {
          R tot[3] = {0, 0, 0};
          for (int k = 0; k <= s; ++k)
            for (int v = 0; v < 3; ++v) tot[v] += tab.alpha[s][k] * res[k][c][v];
          R fac;
          if (dtmode == DT_GLOBAL) { const R dts = tab.beta[s] * dt; fac = dts / vol[c]; }
          else { const R cs = tab.beta[s] * cfl; fac = cs / lam0[c]; }
          R p4[4], c4[4];
          emb(&q0[3 * c], p4);
          prim2cons(sp, p4, c4);
          c4[0] = c4[0] + tot[0] * fac; c4[2] = c4[2] + tot[1] * fac; c4[3] = c4[3] + tot[2] * fac;
          cons2prim(sp, c4, p4);
          q2[3 * c] = p4[0]; q2[3 * c + 1] = p4[2]; q2[3 * c + 2] = p4[3];
        }
        std::swap(q1, q2);
      }
      q0 = q1;
      if (dtmode == DT_GLOBAL) { t += dt; last_dt = dt; }
      else {
        R m = std::numeric_limits<R>::max();
        for (size_t c = 0; c < n; ++c) m = std::min(m, cfl * vol[c] / lam0[c]);
        last_dt = m;
      }
    }
  }
};

}  // namespace hco
