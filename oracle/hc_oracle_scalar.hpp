// hc_oracle_scalar.hpp -- CPU oracle of the scalar advection law.
//
// TEST INFRASTRUCTURE ONLY (see hc_oracle.hpp).  The reference's law
// (conservationLaws/scalarAdvection/scalarAdvection.h:45-98) carries the
// conserved set {u, v, q} in 2D: an advected scalar q and its advecting velocity,
// constant in time.  Exact flux (conservationLaws/scalarAdvection/fluxes/exactFlux.ipp:8-21): (0, 0, u_n q),
// spectral radius |u_n|.  Rusanov and central fluxes are the reference's
// law-generic ones (conservationLaws/base/fluxes/rusanovFlux.ipp:2-50,
// centralFlux.ipp:2-14); the Riemann ghost update picks the boundary value on
// inflow and the interior value on outflow (scalarAdvection/boundary/riemann.ipp).
// The LSQ / MUSCL / residual / RK glue is the Euler oracle's (hc_oracle_solver.hpp)
// with three variables in the conserved basis and no basis transforms.
#pragma once

#include "hc_oracle_solver.hpp"

namespace hco {

template <class R> struct SFlux { R f[3]; R lam; };

enum ScalarFlux { SFLUX_RUSANOV = 0, SFLUX_CENTRAL = 1 };
enum ScalarBC { SBC_PERIODIC = 0, SBC_FIXED = 1, SBC_RIEMANN = 2 };

// projectedVelocity of the conserved set {u, v, q}
template <class R> R scalar_un(const R* n, const R* q) {
  R un = 0;
  for (int i = 0; i < 2; ++i) un += n[i] * q[i];
  return un;
}

// exactFlux (conservationLaws/scalarAdvection/fluxes/exactFlux.ipp:8-21)
template <class R> SFlux<R> scalar_exact(const R* n, const R* q) {
  const R un = scalar_un(n, q);
  SFlux<R> o;
  o.f[0] = 0.; o.f[1] = 0.;
  o.f[2] = un * q[2];
  o.lam = abs(un);
  return o;
}

// CentralFlux (conservationLaws/base/fluxes/centralFlux.ipp:2-14)
template <class R> SFlux<R> scalar_central(const Face<R>& f, const R* ql, const R* qr) {
  const SFlux<R> fl = scalar_exact(f.n, ql), fr = scalar_exact(f.n, qr);
  SFlux<R> o;
  for (int i = 0; i < 3; ++i) o.f[i] = (R)(0.5 * (fl.f[i] + fr.f[i])) * f.area;
  o.lam = std::max(fl.lam, fr.lam) * f.area;
  return o;
}

// RusanovFlux = central + RusanovDissipation (conservationLaws/base/fluxes/rusanovFlux.ipp:2-50)
template <class R> SFlux<R> scalar_rusanov(const Face<R>& f, const R* ql, const R* qr) {
  SFlux<R> o = scalar_central(f, ql, qr);
  const R lambda = std::max(abs(scalar_un(f.n, ql)), abs(scalar_un(f.n, qr)));
  const R la = lambda * f.area;
  const R c = -0.5 * la;
  for (int i = 0; i < 3; ++i) o.f[i] += c * (qr[i] - ql[i]);
  return o;
}

template <class R> SFlux<R> scalar_flux(int kind, const Face<R>& f, const R* ql, const R* qr) {
  return kind == SFLUX_CENTRAL ? scalar_central(f, ql, qr) : scalar_rusanov(f, ql, qr);
}

// Riemann ghost value (conservationLaws/scalarAdvection/boundary/riemann.ipp): the
// face-averaged set is rotated to the face frame and its velocity projected on the
// face normal (pointing into the domain), as written; inflow keeps the boundary
// value, outflow the interior one.
template <class R> void scalar_bc_riemann(const Face<R>& f, const R* qi, const R* qb, R* g) {
  R avg[3], rot[3];
  for (int v = 0; v < 3; ++v) avg[v] = qi[v] + 0.5 * (qb[v] - qi[v]);
  const R* m[2] = {f.n, f.t};
  for (int i = 0; i < 2; ++i) {
    R a = 0;
    for (int j = 0; j < 2; ++j) a += m[i][j] * avg[j];
    rot[i] = a;
  }
  rot[2] = avg[2];
  const bool inflow = scalar_un(f.n, rot) > 0;
  for (int v = 0; v < 3; ++v) g[v] = inflow ? qb[v] : qi[v];
}

template <class R> struct ScalarSolver {
  Solver<R> geo;  // mesh, cells, LSQ metric, periodic shifts, mirror points
  int flux = SFLUX_RUSANOV, lim = LIM_NOLIMIT3, rk = RK_SSP34, dtmode = DT_GLOBAL;
  R cfl = 0.5;
  int bc[4] = {SBC_PERIODIC, SBC_PERIODIC, SBC_PERIODIC, SBC_PERIODIC};
  std::vector<R> ghost[4];  // [side][face][layer][var]: layer 0 ghost, layer 1 reference
  std::vector<R> q0, q1, q2;  // conserved AoS [cell][3]
  std::vector<R> lam0;
  std::vector<SFlux<R>> res[4];
  std::vector<R> qm;          // [cell][6]: q[2*var+dim]
  R t = 0, last_dt = 0;

  int ni() const { return geo.ni; }
  int nj() const { return geo.nj; }

  void setup() {
    for (int s = 0; s < 4; ++s) geo.bc[s] = (bc[s] == SBC_PERIODIC) ? BC_PERIODIC : BC_FIXED;
    geo.setup();
    const size_t n = size_t(ni()) * nj();
    q0.assign(n * 3, 0); q1.assign(n * 3, 0); q2.assign(n * 3, 0);
    lam0.assign(n, 0);
    for (auto& r : res) r.assign(n, SFlux<R>{});
    qm.assign(n * 6, 0);
    for (int s = 0; s < 4; ++s)
      if (ghost[s].size() != size_t(geo.nface(s)) * 6) ghost[s].assign(size_t(geo.nface(s)) * 6, 0);
  }

  void boundary_update(const std::vector<R>& q) {
    for (int side = 0; side < 4; ++side) {
      if (bc[side] == SBC_PERIODIC) continue;
      for (int k = 0; k < geo.nface(side); ++k) {
        R* g = &ghost[side][size_t(k) * 6];
        const R* ref = g + 3;
        const R* qi = &q[size_t(geo.side_cell(side, k)) * 3];
        if (bc[side] == SBC_RIEMANN) scalar_bc_riemann(geo.bface_in(side, k), qi, ref, g);
        else for (int v = 0; v < 3; ++v) g[v] = ref[v];
      }
    }
  }

  void qmetrics(const std::vector<R>& q) {
    std::fill(qm.begin(), qm.end(), R(0));
    auto pair = [&](size_t a, size_t b, R dx, R dy) {
      for (int v = 0; v < 3; ++v) {
        const R dq = q[b * 3 + v] - q[a * 3 + v];
        const R mx = dq * dx, my = dq * dy;
        qm[a * 6 + 2 * v] += mx; qm[a * 6 + 2 * v + 1] += my;
        qm[b * 6 + 2 * v] += mx; qm[b * 6 + 2 * v + 1] += my;
      }
    };
    const int NI = ni(), NJ = nj();
    const auto& cells = geo.cells;
    for (int j = 0; j < NJ; ++j)
      for (int i = 0; i < NI - 1; ++i) {
        const auto& a = cells[geo.cid(i, j)]; const auto& b = cells[geo.cid(i + 1, j)];
        pair(geo.cid(i, j), geo.cid(i + 1, j), b.c[0] - a.c[0], b.c[1] - a.c[1]);
      }
    for (int i = 0; i < NI; ++i)
      for (int j = 0; j < NJ - 1; ++j) {
        const auto& a = cells[geo.cid(i, j)]; const auto& b = cells[geo.cid(i, j + 1)];
        pair(geo.cid(i, j), geo.cid(i, j + 1), b.c[0] - a.c[0], b.c[1] - a.c[1]);
      }
    if (bc[0] == SBC_PERIODIC)
      for (int j = 0; j < NJ; ++j) {
        R s[2]; geo.shift_i(j, s);
        const auto& a = cells[geo.cid(NI - 1, j)]; const auto& b = cells[geo.cid(0, j)];
        pair(geo.cid(NI - 1, j), geo.cid(0, j), b.c[0] - (a.c[0] - s[0]), b.c[1] - (a.c[1] - s[1]));
      }
    if (bc[2] == SBC_PERIODIC)
      for (int i = 0; i < NI; ++i) {
        R s[2]; geo.shift_j(i, s);
        const auto& a = cells[geo.cid(i, NJ - 1)]; const auto& b = cells[geo.cid(i, 0)];
        pair(geo.cid(i, NJ - 1), geo.cid(i, 0), b.c[0] - (a.c[0] - s[0]), b.c[1] - (a.c[1] - s[1]));
      }
  }

  // LSQ solve of the biased metric projected on dir (lsq/factor_solve.ipp:53-69)
  void bsolve(const XM<R>& xb, const R* mb, const R* dir, R* g) const {
    const XM<R> xf = factor(xb);
    for (int v = 0; v < 3; ++v) {
      QM<R> one{};
      one.q[0] = mb[2 * v]; one.q[1] = mb[2 * v + 1];
      R gv[4];
      solve(xf, one, dir, gv);
      g[v] = gv[0];
    }
  }

  SFlux<R> muscl(const Face<R>& f, const R* cl, const R* cr, const R* ql, const R* qr, const XM<R>& xl,
                 const XM<R>& xr, const R* ml, const R* mr) const {
    if (lim == LIM_NOLIMIT1) return scalar_flux(flux, f, ql, qr);
    const R dxc[2] = {cr[0] - cl[0], cr[1] - cl[1]};
    R dqc[3];
    for (int v = 0; v < 3; ++v) dqc[v] = qr[v] - ql[v];
    R d;
    d = 0; d += (f.c[0] - cl[0]) * (f.c[0] - cl[0]); d += (f.c[1] - cl[1]) * (f.c[1] - cl[1]);
    const R dl = sqrt(d);
    d = 0; d += (cr[0] - f.c[0]) * (cr[0] - f.c[0]); d += (cr[1] - f.c[1]) * (cr[1] - f.c[1]);
    const R dr = sqrt(d);
    const R idlr = 1. / (dl + dr);
    const XM<R> xc = xmetric<R>(dxc[0], dxc[1]);
    XM<R> xbl, xbr;
    for (int k = 0; k < 3; ++k) { xbl.x[k] = xl.x[k] - xc.x[k]; xbr.x[k] = xr.x[k] - xc.x[k]; }
    R mbl[6], mbr[6];
    for (int v = 0; v < 3; ++v) {
      mbl[2 * v] = ml[2 * v] - dqc[v] * dxc[0]; mbl[2 * v + 1] = ml[2 * v + 1] - dqc[v] * dxc[1];
      mbr[2 * v] = mr[2 * v] - dqc[v] * dxc[0]; mbr[2 * v + 1] = mr[2 * v + 1] - dqc[v] * dxc[1];
    }
    R gl[3], gr[3];
    bsolve(xbl, mbl, f.n, gl);
    bsolve(xbr, mbr, f.n, gr);
    R qL[3], qR[3];
    for (int v = 0; v < 3; ++v) {
      const R gc = dqc[v] * idlr;
      qL[v] = ql[v] + dl * limit<R>(lim, gc, gl[v]);
      qR[v] = qr[v] - dr * limit<R>(lim, gc, gr[v]);
    }
    return scalar_flux(flux, f, qL, qR);
  }

  SFlux<R> muscl_ghost(int side, int k, const Face<R>& f, const R* qi, const R* qg) const {
    const size_t c = geo.side_cell(side, k);
    const bool ghost_left = (side == 0 || side == 2);
    const R* ql = ghost_left ? qg : qi;
    const R* qr = ghost_left ? qi : qg;
    if (lim == LIM_NOLIMIT1) return scalar_flux(flux, f, ql, qr);
    const R* cc = geo.cells[c].c;
    R d = 0; d += (f.c[0] - cc[0]) * (f.c[0] - cc[0]); d += (f.c[1] - cc[1]) * (f.c[1] - cc[1]);
    const R dd = sqrt(d);
    const R idlr = 1. / (dd + dd);
    R m[2]; geo.mirror(side, k, m);
    const XM<R> xc = xmetric<R>(m[0], m[1]);
    XM<R> xb;
    for (int q = 0; q < 3; ++q) xb.x[q] = geo.xm[c].x[q] - xc.x[q];
    R g[3];
    bsolve(xb, &qm[c * 6], f.n, g);
    R qL[3], qR[3];
    for (int v = 0; v < 3; ++v) {
      const R dq = qr[v] - ql[v];
      const R s = limit<R>(lim, dq * idlr, g[v]);
      if (ghost_left) { qL[v] = qg[v]; qR[v] = qi[v] - dd * s; }
      else { qL[v] = qi[v] + dd * s; qR[v] = qg[v]; }
    }
    return scalar_flux(flux, f, qL, qR);
  }

  static void acc_sub(SFlux<R>& a, const SFlux<R>& f) { for (int v = 0; v < 3; ++v) a.f[v] -= f.f[v]; a.lam += f.lam; }
  static void acc_add(SFlux<R>& a, const SFlux<R>& f) { for (int v = 0; v < 3; ++v) a.f[v] += f.f[v]; a.lam += f.lam; }

  void residual(const std::vector<R>& q, std::vector<SFlux<R>>& r) {
    boundary_update(q);
    qmetrics(q);
    for (auto& x : r) x = SFlux<R>{};
    const int NI = ni(), NJ = nj();
    const auto& cells = geo.cells;
    auto face_pair = [&](const Face<R>& f, size_t a, size_t b, const R* cl) {
      const SFlux<R> fx = muscl(f, cl, cells[b].c, &q[a * 3], &q[b * 3], geo.xm[a], geo.xm[b], &qm[a * 6],
                                &qm[b * 6]);
      acc_sub(r[a], fx); acc_add(r[b], fx);
    };
    for (int j = 0; j < NJ; ++j)
      for (int i = 0; i < NI - 1; ++i) {
        const size_t a = geo.cid(i, j), b = geo.cid(i + 1, j);
        face_pair(surface(geo.node(i + 1, j), geo.node(i + 1, j + 1)), a, b, cells[a].c);
      }
    for (int i = 0; i < NI; ++i)
      for (int j = 0; j < NJ - 1; ++j) {
        const size_t a = geo.cid(i, j), b = geo.cid(i, j + 1);
        face_pair(surface(geo.node(i + 1, j + 1), geo.node(i, j + 1)), a, b, cells[a].c);
      }
    for (int side = 0; side < 4; ++side) {
      if (bc[side] == SBC_PERIODIC) {
        if (side == 0)
          for (int j = 0; j < NJ; ++j) {
            R s[2]; geo.shift_i(j, s);
            const size_t a = geo.cid(NI - 1, j), b = geo.cid(0, j);
            const R cl[2] = {cells[a].c[0] - s[0], cells[a].c[1] - s[1]};
            face_pair(surface(geo.node(0, j), geo.node(0, j + 1)), a, b, cl);
          }
        else if (side == 2)
          for (int i = 0; i < NI; ++i) {
            R s[2]; geo.shift_j(i, s);
            const size_t a = geo.cid(i, NJ - 1), b = geo.cid(i, 0);
            const R cl[2] = {cells[a].c[0] - s[0], cells[a].c[1] - s[1]};
            face_pair(surface(geo.node(i + 1, 0), geo.node(i, 0)), a, b, cl);
          }
      } else {
        for (int k = 0; k < geo.nface(side); ++k) {
          const size_t c = geo.side_cell(side, k);
          const SFlux<R> f = muscl_ghost(side, k, geo.bface_flux(side, k), &q[c * 3], &ghost[side][size_t(k) * 6]);
          if (side == 0 || side == 2) acc_add(r[c], f); else acc_sub(r[c], f);
        }
      }
    }
  }

  R spectral_radius(const std::vector<SFlux<R>>& r) const {
    R m = std::numeric_limits<R>::min();
    for (size_t c = 0; c < r.size(); ++c) m = std::max(m, r[c].lam / geo.cells[c].vol);
    return m;
  }

  void step(int nsteps) {
    const RKTable<R> tab = rk_table<R>(rk);
    const size_t n = size_t(ni()) * nj();
    for (int st = 0; st < nsteps; ++st) {
      R dt = 0;
      q1 = q0;
      for (int s = 0; s < tab.nstages; ++s) {
        residual(q1, res[s]);
        if (s == 0) {
          if (dtmode == DT_GLOBAL) dt = freeze(cfl / spectral_radius(res[0]));
          else for (size_t c = 0; c < n; ++c) lam0[c] = freeze(res[0][c].lam);
        }
        for (size_t c = 0; c < n; ++c) {
          R tot[3] = {0, 0, 0};
          for (int k = 0; k <= s; ++k)
            for (int v = 0; v < 3; ++v) tot[v] += tab.alpha[s][k] * res[k][c].f[v];
          R fac;
          if (dtmode == DT_GLOBAL) { const R dts = tab.beta[s] * dt; fac = dts / geo.cells[c].vol; }
          else { const R cs = tab.beta[s] * cfl; fac = cs / lam0[c]; }
          for (int v = 0; v < 3; ++v) q2[c * 3 + v] = q0[c * 3 + v] + tot[v] * fac;
        }
        std::swap(q1, q2);
      }
      q0 = q1;
      if (dtmode == DT_GLOBAL) { t += dt; last_dt = dt; }
    }
  }
};

}  // namespace hco
