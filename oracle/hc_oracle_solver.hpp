// hc_oracle_solver.hpp -- CPU oracle: the residual / RK glue of the reference.
//
// TEST INFRASTRUCTURE ONLY (see hc_oracle.hpp).  The reference's spatial glue
// (lsq/*, spatial/*, timestepping/rungeKutta.h) does not compile at its HEAD;
// this file restates its intent with the decisions below, which the CUDA path
// implements identically:
//   D2  LSQ stencil = the 4 face neighbours, periodic wrap neighbours included
//       (their centres translated by the periodic shift); non-periodic sides
//       add the mirrored-point xmetric with zero q contribution
//       (spatial/lsqMetrics.h:104-163, qmetrics spatial/lsqMetrics.h:181-213).
//   D3  QMetric index q[2*var+dim]; biased gradient projected on face.metric[0].
//   D4  ghost faces: ghost side unreconstructed, interior side MUSCL with the
//       mirror term removed; wall pressure from the interior state extrapolated
//       to the face with the cell's full LSQ gradient.
//   D5  alpha/beta RK accumulation form; global dt from stage 0
//       (timestepping/rungeKutta.h:96-197); local dt from the stage-0 spectral
//       radius sum, eulerForwardUpdateLocal semantics (spatial/eulerForwardUpdate.h:117-168).
#pragma once

#include "hc_oracle.hpp"

#include <omp.h>

namespace hco {

// the value of a number of the oracle's arithmetic types (double, or the dual / counting
// types, which hold it in .v)
template <class T> double value_of(const T& x) {
  if constexpr (std::is_arithmetic_v<T>) return double(x);
  else return double(x.v);
}

template <class R> struct Solver {
  int ni = 0, nj = 0;
  std::vector<R> nodes;  // (ni+1)*(nj+1)*2
  Species<R> sp{};
  int flux = FLUX_ROE, lim = LIM_VANLEER, rk = RK_SSP34, dtmode = DT_GLOBAL;
  int vscale = SCALING_CONVECTIVE, pscale = SCALING_CONVECTIVE;  // AUSM+up low-Mach scaling
  int basis = BASIS_PRIMITIVE;  // solution basis of q and of the ghost layers
  // branch signatures of the next residual evaluation, when set: (ni+1)*nj i-faces and
  // ni*(nj+1) j-faces (codes of limit_piece / flux_bits in hc_oracle.hpp)
  uint64_t* sig_i = nullptr;
  uint64_t* sig_j = nullptr;
  // with the signatures, optionally the limiter arguments (a, b) of the 8 limiter calls
  // of each face (left side's four variables, then the right side's): 16 per face
  double* arg_i = nullptr;
  double* arg_j = nullptr;
  std::vector<unsigned> bc_path[4];  // far-field path per ghost face of the last boundary update
  // dual time (set by dual_time): residual -> g0 R(q) - V b0dt Q(q) + src (AoS [cell][4])
  bool dual = false;
  R dual_g0 = 1, dual_b0dt = 0;
  std::vector<R> dual_src;
  R cfl = 0.5;
  int bc[4] = {BC_PERIODIC, BC_PERIODIC, BC_PERIODIC, BC_PERIODIC};
  // ghost arrays per side: [side][face][layer][var]; layer 0 = ghost value,
  // layer 1 = reference (far-field) value (solutionField/solutionField.h:20-31)
  std::vector<R> ghost[4];
  std::vector<Cell<R>> cells;
  std::vector<XM<R>> xm;       // full xmetric per cell
  std::vector<R> q0, q1, q2;   // solution-basis AoS [cell][4]
  std::vector<R> lam0;         // stage-0 spectral radius sums (local dt)
  std::vector<FluxRes<R>> res[4], rtot;
  std::vector<QM<R>> qm;
  R t = 0, last_dt = 0;

  const R* node(int i, int j) const { return &nodes[(size_t(i) * (nj + 1) + j) * 2]; }
  size_t cid(int i, int j) const { return size_t(i) * nj + j; }
  int nface(int side) const { return side < 2 ? nj : ni; }
  State<R> st(const R* q) const { return basis2state(sp, q, basis); }
  // signature slot of boundary face k of side `side` (i-faces i = 0 / ni, j-faces j = 0 / nj)
  // limiter-argument slot of the face whose signature slot is sg
  double* face_args(const uint64_t* sg) const {
    if (!arg_i) return nullptr;
    const size_t nfi = size_t(ni + 1) * nj;
    if (sg >= sig_i && sg < sig_i + nfi) return arg_i + size_t(sg - sig_i) * 16;
    return arg_j + size_t(sg - sig_j) * 16;
  }
  uint64_t* face_sig(int side, int k) const {
    if (side == 0) return &sig_i[size_t(k)];
    if (side == 1) return &sig_i[size_t(ni) * nj + k];
    if (side == 2) return &sig_j[size_t(k) * (nj + 1)];
    return &sig_j[size_t(k) * (nj + 1) + nj];
  }

  // periodic shift across the i (or j) boundary at face index k: image of the
  // last cell = its centre minus the shift (average over the face's two nodes)
  void shift_i(int j, R* s) const {
    for (int d = 0; d < 2; ++d)
      s[d] = 0.5 * ((node(ni, j)[d] - node(0, j)[d]) + (node(ni, j + 1)[d] - node(0, j + 1)[d]));
  }
  void shift_j(int i, R* s) const {
    for (int d = 0; d < 2; ++d)
      s[d] = 0.5 * ((node(i, nj)[d] - node(i, 0)[d]) + (node(i + 1, nj)[d] - node(i + 1, 0)[d]));
  }
  // mirrored-point displacement of a boundary cell (spatial/lsqMetrics.h:119-123)
  void mirror(int side, int k, R* m) const {
    int i0, j0, i1, j1;
    if (side == 0) { i0 = 0; j0 = k; i1 = 1; j1 = k; }
    else if (side == 1) { i0 = ni - 1; j0 = k; i1 = ni - 2; j1 = k; }
    else if (side == 2) { i0 = k; j0 = 0; i1 = k; j1 = 1; }
    else { i0 = k; j0 = nj - 1; i1 = k; j1 = nj - 2; }
    const Cell<R>& c0 = cells[cid(i0, j0)];
    const Cell<R>& c1 = cells[cid(i1, j1)];
    for (int d = 0; d < 2; ++d) {
      const R disp = c0.c[d] - c1.c[d];
      const R bp = c0.c[d] + disp;
      m[d] = bp - c0.c[d];
    }
  }
  int side_cell(int side, int k) const {
    if (side == 0) return (int)cid(0, k);
    if (side == 1) return (int)cid(ni - 1, k);
    if (side == 2) return (int)cid(k, 0);
    return (int)cid(k, nj - 1);
  }
  // boundary face as used by the flux loops (ghostCellLoop.h:133-224): sides 0/2
  // have normals pointing into the domain, sides 1/3 out of it
  Face<R> bface_flux(int side, int k) const {
    if (side == 0) return surface(node(0, k), node(0, k + 1));
    if (side == 1) return surface(node(ni, k), node(ni, k + 1));
    if (side == 2) return surface(node(k + 1, 0), node(k, 0));
    return surface(node(k + 1, nj), node(k, nj));
  }
  // boundary face with the normal into the domain (boundaryUpdate.h:171-262,
  // boundaryFluxLoop.h:150-261)
  Face<R> bface_in(int side, int k) const {
    if (side == 0) return surface(node(0, k), node(0, k + 1));
    if (side == 1) return surface(node(ni, k + 1), node(ni, k));
    if (side == 2) return surface(node(k + 1, 0), node(k, 0));
    return surface(node(k, nj), node(k + 1, nj));
  }

  void setup() {
    cells.resize(size_t(ni) * nj);
    for (int i = 0; i < ni; ++i)
      for (int j = 0; j < nj; ++j)
        cells[cid(i, j)] = volume(node(i, j), node(i + 1, j), node(i, j + 1), node(i + 1, j + 1));
    xm.assign(size_t(ni) * nj, XM<R>{{0, 0, 0}});
    auto addx = [&](size_t a, const XM<R>& v) { for (int k = 0; k < 3; ++k) xm[a].x[k] += v.x[k]; };
    // neighbour_accumulation order (parallalg/neighbour_algorithm.h:243-317)
    for (int j = 0; j < nj; ++j)
      for (int i = 0; i < ni - 1; ++i) {
        const Cell<R>& a = cells[cid(i, j)];
        const Cell<R>& b = cells[cid(i + 1, j)];
        const XM<R> v = xmetric<R>(b.c[0] - a.c[0], b.c[1] - a.c[1]);
        addx(cid(i, j), v); addx(cid(i + 1, j), v);
      }
    for (int i = 0; i < ni; ++i)
      for (int j = 0; j < nj - 1; ++j) {
        const Cell<R>& a = cells[cid(i, j)];
        const Cell<R>& b = cells[cid(i, j + 1)];
        const XM<R> v = xmetric<R>(b.c[0] - a.c[0], b.c[1] - a.c[1]);
        addx(cid(i, j), v); addx(cid(i, j + 1), v);
      }
    if (bc[0] == BC_PERIODIC)
      for (int j = 0; j < nj; ++j) {
        R s[2]; shift_i(j, s);
        const Cell<R>& a = cells[cid(ni - 1, j)];
        const Cell<R>& b = cells[cid(0, j)];
        const XM<R> v = xmetric<R>(b.c[0] - (a.c[0] - s[0]), b.c[1] - (a.c[1] - s[1]));
        addx(cid(ni - 1, j), v); addx(cid(0, j), v);
      }
    if (bc[2] == BC_PERIODIC)
      for (int i = 0; i < ni; ++i) {
        R s[2]; shift_j(i, s);
        const Cell<R>& a = cells[cid(i, nj - 1)];
        const Cell<R>& b = cells[cid(i, 0)];
        const XM<R> v = xmetric<R>(b.c[0] - (a.c[0] - s[0]), b.c[1] - (a.c[1] - s[1]));
        addx(cid(i, nj - 1), v); addx(cid(i, 0), v);
      }
    // boundary_xmetrics order (spatial/lsqMetrics.h:126-162): left/right per j, then bottom/top per i
    for (int j = 0; j < nj; ++j)
      for (int side = 0; side < 2; ++side)
        if (bc[side] != BC_PERIODIC) { R m[2]; mirror(side, j, m); addx(side_cell(side, j), xmetric<R>(m[0], m[1])); }
    for (int i = 0; i < ni; ++i)
      for (int side = 2; side < 4; ++side)
        if (bc[side] != BC_PERIODIC) { R m[2]; mirror(side, i, m); addx(side_cell(side, i), xmetric<R>(m[0], m[1])); }
    const size_t n = size_t(ni) * nj;
    q0.assign(n * 4, 0); q1.assign(n * 4, 0); q2.assign(n * 4, 0);
    lam0.assign(n, 0);
    for (auto& r : res) r.assign(n, FluxRes<R>{});
    rtot.assign(n, FluxRes<R>{});
    qm.assign(n, QM<R>{});
    for (int s = 0; s < 4; ++s)
      if (ghost[s].size() != size_t(nface(s)) * 8) ghost[s].assign(size_t(nface(s)) * 8, 0);
  }

  // ---- boundaryUpdate (spatial/boundary/boundaryUpdate.h:137-266)
  void boundary_update(const std::vector<R>& q) {
    for (int side = 0; side < 4; ++side) {
      if (bc[side] == BC_PERIODIC) continue;
      bc_path[side].resize(size_t(nface(side)));
      for (int k = 0; k < nface(side); ++k) {
        R* g = &ghost[side][size_t(k) * 8];
        const R* ref = g + 4;
        const R* qi = &q[size_t(side_cell(side, k)) * 4];
        unsigned* path = &bc_path[side][k];
        *path = 0;
        if (bc[side] == BC_RIEMANN) bc_riemann(sp, bface_in(side, k), qi, ref, g, basis, path);
        else if (bc[side] == BC_ENTROPY) bc_entropy(sp, bface_in(side, k), qi, ref, g, basis, path);
        else for (int v = 0; v < 4; ++v) g[v] = ref[v];  // Fixed (boundaryCondition.h:63-80); wall ghost unused
      }
    }
  }

  // ---- qmetrics with periodic wrap (spatial/lsqMetrics.h:181-213, D2)
  void qmetrics(const std::vector<R>& q) {
    for (auto& m : qm) m = QM<R>{};
    auto addq = [&](size_t a, const QM<R>& v) { for (int k = 0; k < 8; ++k) qm[a].q[k] += v.q[k]; };
    auto pair = [&](size_t a, size_t b, R dx, R dy) {
      R dq[4];
      for (int v = 0; v < 4; ++v) dq[v] = q[b * 4 + v] - q[a * 4 + v];
      const QM<R> m = qmetric<R>(dx, dy, dq);
      addq(a, m); addq(b, m);
    };
    for (int j = 0; j < nj; ++j)
      for (int i = 0; i < ni - 1; ++i) {
        const Cell<R>& a = cells[cid(i, j)]; const Cell<R>& b = cells[cid(i + 1, j)];
        pair(cid(i, j), cid(i + 1, j), b.c[0] - a.c[0], b.c[1] - a.c[1]);
      }
    for (int i = 0; i < ni; ++i)
      for (int j = 0; j < nj - 1; ++j) {
        const Cell<R>& a = cells[cid(i, j)]; const Cell<R>& b = cells[cid(i, j + 1)];
        pair(cid(i, j), cid(i, j + 1), b.c[0] - a.c[0], b.c[1] - a.c[1]);
      }
    if (bc[0] == BC_PERIODIC)
      for (int j = 0; j < nj; ++j) {
        R s[2]; shift_i(j, s);
        const Cell<R>& a = cells[cid(ni - 1, j)]; const Cell<R>& b = cells[cid(0, j)];
        pair(cid(ni - 1, j), cid(0, j), b.c[0] - (a.c[0] - s[0]), b.c[1] - (a.c[1] - s[1]));
      }
    if (bc[2] == BC_PERIODIC)
      for (int i = 0; i < ni; ++i) {
        R s[2]; shift_j(i, s);
        const Cell<R>& a = cells[cid(i, nj - 1)]; const Cell<R>& b = cells[cid(i, 0)];
        pair(cid(i, nj - 1), cid(i, 0), b.c[0] - (a.c[0] - s[0]), b.c[1] - (a.c[1] - s[1]));
      }
  }

  // ---- make_muscl_flux (spatial/muscl.h:13-59) with bias_solves (lsq/factor_solve.ipp:71-100)
  FluxRes<R> muscl(const Face<R>& f, const R* cl, const R* cr, const R* ql, const R* qr,
                   const XM<R>& xl, const XM<R>& xr, const QM<R>& ml, const QM<R>& mr, uint64_t* sg = nullptr) const {
    if (lim == LIM_NOLIMIT1) {  // first-order overload (spatial/muscl.h:62-87)
      if (sg) *sg = (uint64_t(flux_bits(flux, sp, f, st(ql), st(qr))) << SIG_FLUX_SHIFT) | (1ull << SIG_VALID_SHIFT);
      return face_flux(flux, sp, f, st(ql), st(qr), vscale, pscale);
    }
    const R dxc[2] = {cr[0] - cl[0], cr[1] - cl[1]};
    R dqc[4];
    for (int v = 0; v < 4; ++v) dqc[v] = qr[v] - ql[v];
    R d;
    d = 0; d += (f.c[0] - cl[0]) * (f.c[0] - cl[0]); d += (f.c[1] - cl[1]) * (f.c[1] - cl[1]);
    const R dl = sqrt(d);
    d = 0; d += (cr[0] - f.c[0]) * (cr[0] - f.c[0]); d += (cr[1] - f.c[1]) * (cr[1] - f.c[1]);
    const R dr = sqrt(d);
    const R idlr = 1. / (dl + dr);
    R gc[4];
    for (int v = 0; v < 4; ++v) gc[v] = dqc[v] * idlr;
    const XM<R> xc = xmetric<R>(dxc[0], dxc[1]);
    const QM<R> mc = qmetric<R>(dxc[0], dxc[1], dqc);
    XM<R> xbl, xbr; QM<R> mbl, mbr;
    for (int k = 0; k < 3; ++k) { xbl.x[k] = xl.x[k] - xc.x[k]; xbr.x[k] = xr.x[k] - xc.x[k]; }
    for (int k = 0; k < 8; ++k) { mbl.q[k] = ml.q[k] - mc.q[k]; mbr.q[k] = mr.q[k] - mc.q[k]; }
    R gl[4], gr[4];
    solve(factor(xbl), mbl, f.n, gl);
    solve(factor(xbr), mbr, f.n, gr);
    R qL[4], qR[4];
    for (int v = 0; v < 4; ++v) {
      const R sl = limit<R>(lim, gc[v], gl[v]);
      const R sr = limit<R>(lim, gc[v], gr[v]);
      qL[v] = ql[v] + dl * sl;
      qR[v] = qr[v] - dr * sr;
    }
    if (sg) {
      uint64_t b = 1ull << SIG_VALID_SHIFT;
      for (int v = 0; v < 4; ++v)
        b |= (uint64_t(limit_piece(lim, gc[v], gl[v])) << (4 * v)) |
             (uint64_t(limit_piece(lim, gc[v], gr[v])) << (16 + 4 * v));
      *sg = b | (uint64_t(flux_bits(flux, sp, f, st(qL), st(qR))) << SIG_FLUX_SHIFT);
      if (double* ag = face_args(sg))
        for (int v = 0; v < 4; ++v) {
          ag[2 * v] = value_of(gc[v]); ag[2 * v + 1] = value_of(gl[v]);
          ag[8 + 2 * v] = value_of(gc[v]); ag[8 + 2 * v + 1] = value_of(gr[v]);
        }
    }
    return face_flux(flux, sp, f, st(qL), st(qR), vscale, pscale);
  }

  // ghost face (D4): ghost side is not reconstructed, interior side is MUSCL
  // with the mirror term removed from its xmetric.  ghost_left says whether the
  // ghost is the face's left state (sides 0/2) or right state (sides 1/3).
  FluxRes<R> muscl_ghost(int side, int k, const Face<R>& f, const R* qi, const R* qg, uint64_t* sg = nullptr) const {
    const size_t c = side_cell(side, k);
    const bool ghost_left = (side == 0 || side == 2);
    const R* ql = ghost_left ? qg : qi;
    const R* qr = ghost_left ? qi : qg;
    const uint64_t bcb = (uint64_t(bc_path[side].empty() ? 0u : bc_path[side][k]) << SIG_BC_SHIFT) |
                         (1ull << SIG_VALID_SHIFT);
    if (lim == LIM_NOLIMIT1) {
      if (sg) *sg = bcb | (uint64_t(flux_bits(flux, sp, f, st(ql), st(qr))) << SIG_FLUX_SHIFT);
      return face_flux(flux, sp, f, st(ql), st(qr), vscale, pscale);
    }
    const R* cc = cells[c].c;
    R d = 0; d += (f.c[0] - cc[0]) * (f.c[0] - cc[0]); d += (f.c[1] - cc[1]) * (f.c[1] - cc[1]);
    const R dd = sqrt(d);
    R dqc[4];
    for (int v = 0; v < 4; ++v) dqc[v] = qr[v] - ql[v];
    const R idlr = 1. / (dd + dd);
    R m[2]; mirror(side, k, m);
    const XM<R> xc = xmetric<R>(m[0], m[1]);
    XM<R> xb;
    for (int q = 0; q < 3; ++q) xb.x[q] = xm[c].x[q] - xc.x[q];
    R g[4];
    solve(factor(xb), qm[c], f.n, g);
    R qL[4], qR[4];
    uint64_t pieces = 0;
    for (int v = 0; v < 4; ++v) {
      const R s = limit<R>(lim, dqc[v] * idlr, g[v]);
      if (ghost_left) { qL[v] = qg[v]; qR[v] = qi[v] - dd * s; }
      else { qL[v] = qi[v] + dd * s; qR[v] = qg[v]; }
      pieces |= uint64_t(limit_piece(lim, dqc[v] * idlr, g[v])) << ((ghost_left ? 16 : 0) + 4 * v);
      if (sg)
        if (double* ag = face_args(sg)) {
          ag[(ghost_left ? 8 : 0) + 2 * v] = value_of(dqc[v] * idlr);
          ag[(ghost_left ? 8 : 0) + 2 * v + 1] = value_of(g[v]);
        }
    }
    if (sg) *sg = bcb | pieces | (uint64_t(flux_bits(flux, sp, f, st(qL), st(qR))) << SIG_FLUX_SHIFT);
    return face_flux(flux, sp, f, st(qL), st(qR), vscale, pscale);
  }

  static void acc_sub(FluxRes<R>& a, const FluxRes<R>& f) { for (int v = 0; v < 4; ++v) a.f[v] -= f.f[v]; a.lam += f.lam; }
  static void acc_add(FluxRes<R>& a, const FluxRes<R>& f) { for (int v = 0; v < 4; ++v) a.f[v] += f.f[v]; a.lam += f.lam; }

  // ---- residualCalc (spatial/residualCalc.h:27-307)
  void residual(const std::vector<R>& q, std::vector<FluxRes<R>>& r) {
    boundary_update(q);
    qmetrics(q);
    for (auto& x : r) x = FluxRes<R>{};
    // i-normal faces (spatial/residualCalc.h:199-225); each j row is independent
#pragma omp parallel for schedule(static)
    for (int j = 0; j < nj; ++j)
      for (int i = 0; i < ni - 1; ++i) {
        const size_t a = cid(i, j), b = cid(i + 1, j);
        const FluxRes<R> f = muscl(surface(node(i + 1, j), node(i + 1, j + 1)), cells[a].c, cells[b].c,
                                   &q[a * 4], &q[b * 4], xm[a], xm[b], qm[a], qm[b],
                                   sig_i ? &sig_i[size_t(i + 1) * nj + j] : nullptr);
        acc_sub(r[a], f); acc_add(r[b], f);
      }
    // j-normal faces (spatial/residualCalc.h:227-253)
#pragma omp parallel for schedule(static)
    for (int i = 0; i < ni; ++i)
      for (int j = 0; j < nj - 1; ++j) {
        const size_t a = cid(i, j), b = cid(i, j + 1);
        const FluxRes<R> f = muscl(surface(node(i + 1, j + 1), node(i, j + 1)), cells[a].c, cells[b].c,
                                   &q[a * 4], &q[b * 4], xm[a], xm[b], qm[a], qm[b],
                                   sig_j ? &sig_j[size_t(i) * (nj + 1) + j + 1] : nullptr);
        acc_sub(r[a], f); acc_add(r[b], f);
      }
    // boundary residuals in boundary-id order (spatial/residualCalc.h:279-307)
    for (int side = 0; side < 4; ++side) {
      const int t = bc[side];
      if (t == BC_PERIODIC) {
        // only the lower face of each periodic pair (periodicLoop.h:115-179)
        if (side == 0)
          for (int j = 0; j < nj; ++j) {
            R s[2]; shift_i(j, s);
            const size_t a = cid(ni - 1, j), b = cid(0, j);
            const R cl[2] = {cells[a].c[0] - s[0], cells[a].c[1] - s[1]};
            const FluxRes<R> f = muscl(surface(node(0, j), node(0, j + 1)), cl, cells[b].c,
                                       &q[a * 4], &q[b * 4], xm[a], xm[b], qm[a], qm[b],
                                       sig_i ? &sig_i[size_t(j)] : nullptr);
            acc_sub(r[a], f); acc_add(r[b], f);
          }
        else if (side == 2)
          for (int i = 0; i < ni; ++i) {
            R s[2]; shift_j(i, s);
            const size_t a = cid(i, nj - 1), b = cid(i, 0);
            const R cl[2] = {cells[a].c[0] - s[0], cells[a].c[1] - s[1]};
            const FluxRes<R> f = muscl(surface(node(i + 1, 0), node(i, 0)), cl, cells[b].c,
                                       &q[a * 4], &q[b * 4], xm[a], xm[b], qm[a], qm[b],
                                       sig_j ? &sig_j[size_t(i) * (nj + 1)] : nullptr);
            acc_sub(r[a], f); acc_add(r[b], f);
          }
      } else if (t == BC_WALL) {
        // boundary flux loop (boundaryFluxLoop.h:122-265): normal into the domain, res += F
        for (int k = 0; k < nface(side); ++k) {
          const size_t c = side_cell(side, k);
          const Face<R> f = bface_in(side, k);
          const R dir[2] = {cells[c].c[0] - f.c[0], cells[c].c[1] - f.c[1]};
          R dq[4];
          solve(factor(xm[c]), qm[c], dir, dq);
          acc_add(r[c], wall_flux(sp, f, &q[c * 4], dq, basis));
          if (sig_i || sig_j) *face_sig(side, k) = 1ull << SIG_VALID_SHIFT;
        }
      } else {
        // ghost-cell loop (ghostCellLoop.h:109-228)
        for (int k = 0; k < nface(side); ++k) {
          const size_t c = side_cell(side, k);
          const FluxRes<R> f = muscl_ghost(side, k, bface_flux(side, k), &q[c * 4], &ghost[side][size_t(k) * 8],
                                           (sig_i || sig_j) ? face_sig(side, k) : nullptr);
          if (side == 0 || side == 2) acc_add(r[c], f); else acc_sub(r[c], f);
        }
      }
    }
  }

  // ---- dual time (ode.h:12-82, timestepping/dualTime.ipp:4-105,
  // OLD.fieldOperations/dualTimeResidual.ipp:2-41): the flux residual of the iterate becomes
  // g0 R(q) - V (b0/dt) Q(q) + src, src = g1 R(q_n) - V (b1 Q_n + b2 Q_{n-1}) / dt
  void cons_of(const R* q, R* qc) const {
    if (basis == BASIS_CONSERVED) for (int v = 0; v < 4; ++v) qc[v] = q[v];
    else prim2cons(sp, q, qc);
  }
  void add_dual_terms(const std::vector<R>& q, std::vector<FluxRes<R>>& r) const {
    const size_t n = size_t(ni) * nj;
    for (size_t c = 0; c < n; ++c) {
      R qc[4];
      cons_of(&q[c * 4], qc);
      const R vb = cells[c].vol * dual_b0dt;
      for (int v = 0; v < 4; ++v) r[c].f[v] = dual_g0 * r[c].f[v] + (dual_src[c * 4 + v] - vb * qc[v]);
    }
  }
  // outer physical steps of the multistep scheme (BDF1 / BDF2 / trapezium) with `inner`
  // pseudo-time RK steps each; dt <= 0: cfl_outer / spectral radius of the initial state
  R dual_time(int outer, R dtp, R cfl_outer, int scheme, int inner) {
    R beta[3] = {1., -1., 0.}, gam[2] = {1., 0.};
    if (scheme == 1) { beta[0] = 1.5; beta[1] = -2.; beta[2] = 0.5; }
    else if (scheme == 2) { gam[0] = 0.5; gam[1] = 0.5; }
    const size_t n = size_t(ni) * nj;
    if (!(dtp > 0)) { residual(q0, res[0]); dtp = cfl_outer / spectral_radius(res[0]); }
    std::vector<R> Qn(n * 4), Qm(n * 4), Rn(n * 4, R(0));
    for (size_t c = 0; c < n; ++c) cons_of(&q0[c * 4], &Qn[c * 4]);
    Qm = Qn;
    const R tsave = t;
    for (int k = 0; k < outer; ++k) {
      if (gam[1] != 0) {
        residual(q0, res[0]);
        for (size_t c = 0; c < n; ++c) for (int v = 0; v < 4; ++v) Rn[c * 4 + v] = res[0][c].f[v];
      }
      dual_src.assign(n * 4, R(0));
      const R b1dt = beta[1] / dtp, b2dt = beta[2] / dtp;
      for (size_t c = 0; c < n; ++c)
        for (int v = 0; v < 4; ++v) {
          const R lev = b1dt * Qn[c * 4 + v] + b2dt * Qm[c * 4 + v];
          dual_src[c * 4 + v] = gam[1] * Rn[c * 4 + v] - cells[c].vol * lev;
        }
      dual = true; dual_g0 = gam[0]; dual_b0dt = beta[0] / dtp;
      for (int m = 0; m < inner; ++m) step(1);
      dual = false;
      std::swap(Qn, Qm);
      for (size_t c = 0; c < n; ++c) cons_of(&q0[c * 4], &Qn[c * 4]);
    }
    t = tsave + outer * dtp;
    last_dt = dtp;
    return dtp;
  }

  // ---- spectralRadius (spatial/spectralRadius.h:19-48)
  R spectral_radius(const std::vector<FluxRes<R>>& r) const {
    R m = std::numeric_limits<R>::min();
    for (size_t c = 0; c < r.size(); ++c) m = std::max(m, r[c].lam / cells[c].vol);
    return m;
  }

  // ---- integrate (timestepping/rungeKutta.h:37-197); returns the last dt
  void step(int nsteps) {
    const RKTable<R> tab = rk_table<R>(rk);
    const size_t n = size_t(ni) * nj;
    for (int st = 0; st < nsteps; ++st) {
      R dt = 0;
      q1 = q0;
      for (int s = 0; s < tab.nstages; ++s) {
        residual(q1, res[s]);
        if (dual) add_dual_terms(q1, res[s]);
        if (s == 0) {
          if (dtmode == DT_GLOBAL) {
            dt = freeze(cfl / spectral_radius(res[0]));
            if (dual) dt = freeze(dt / (1. + dual_b0dt * dt));  // dtau / (1 + b0 dtau / dt)
          } else {
            for (size_t c = 0; c < n; ++c) lam0[c] = freeze(res[0][c].lam);
          }
        }
#pragma omp parallel for schedule(static)
        for (long c = 0; c < (long)n; ++c) {
          // rungeKuttaAccumulation (timestepping/rungeKutta.h:172-197)
          R tot[4] = {0, 0, 0, 0};
          for (int k = 0; k <= s; ++k)
            for (int v = 0; v < 4; ++v) tot[v] += tab.alpha[s][k] * res[k][c].f[v];
          // eulerForwardUpdateGlobal / Local (spatial/eulerForwardUpdate.h:38-168)
          R fac;
          if (dtmode == DT_GLOBAL) { const R dts = tab.beta[s] * dt; fac = dts / cells[c].vol; }
          else {
            const R cs = tab.beta[s] * cfl;
            fac = dual ? cs / (lam0[c] + cfl * cells[c].vol * dual_b0dt) : cs / lam0[c];
          }
          // solution basis -> conserved (+ increment) -> solution basis; a conserved
          // field is its own conserved set (set2Set of the same type copies)
          R qc[4];
          if (basis == BASIS_CONSERVED) for (int v = 0; v < 4; ++v) qc[v] = q0[c * 4 + v];
          else prim2cons(sp, &q0[c * 4], qc);
          for (int v = 0; v < 4; ++v) qc[v] = qc[v] + tot[v] * fac;
          if (basis == BASIS_CONSERVED) for (int v = 0; v < 4; ++v) q2[c * 4 + v] = qc[v];
          else cons2prim(sp, qc, &q2[c * 4]);
        }
        std::swap(q1, q2);
      }
      q0 = q1;
      if (dtmode == DT_GLOBAL) { t += dt; last_dt = dt; }
      else {
        R m = std::numeric_limits<R>::max();
        for (size_t c = 0; c < n; ++c) m = std::min(m, cfl * cells[c].vol / lam0[c]);
        last_dt = m;
      }
    }
  }
};

}  // namespace hco
