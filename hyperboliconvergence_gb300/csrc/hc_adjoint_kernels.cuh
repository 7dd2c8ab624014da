// hc_adjoint_kernels.cuh -- discrete adjoint of one residual evaluation and of
// the RK stage update, with the timestep frozen.
//
// Forward structure being reversed (stage kernel, hc_kernels.cuh):
//   QM_c = sum over c's pair faces h of (q_R(h) - q_L(h)) (x) dx_h
//   per face: gc = dq*idlr, g_side = QM_side . w_side - dq*s_side,
//             q_side' = q_side +/- d_side * limit(gc, g_side), F = flux(q_L', q_R')
//   Res_c = sum of +F (c right of the face) and -F (c left of the face)
// Reverse, three passes over the mesh:
//   1. faces: F_bar = Rbar_R - Rbar_L; flux, limiter and reconstruction
//      reversed; per face the direct adjoints of the two cells (dL, dR) and the
//      adjoints of their biased gradients (gL, gR) are written out (16 planes);
//      boundary faces add the ghost side's adjoint to the reference-state
//      adjoint of their side.
//   2. cells: QMbar_c = sum over c's faces of g_{c,f} (x) w_{c,f}.
//   3. cells: qbar_c = sum of direct terms + sum over pair faces h of c of
//      sgn_c(h) (QMbar_c + QMbar_nbr(h)) . dx_h.
#pragma once

#include "hc_adjoint.cuh"
#include "hc_kernels.cuh"
#include "hc_scalar.cuh"
#include "hc_tangent.cuh"

#include <cfloat>

namespace hc {

enum { ADJ_FIELDS = 16 };  // dL[4], dR[4], gL[4], gR[4]

template <class R> struct AdjArgs {
  int ni, nj;
  int bc[4];
  Gas<R> gas;
  int limiter;
  const R* q;        // stage state (primitive, 4 planes)
  const R* qm;       // its qmetric, 8 planes (var-major: 2*v+dim)
  const R* rbar;     // residual adjoint, 4 planes
  const R* fi;       // face records
  const R* fj;
  const R* gref[4];  // ghost reference planes per side
  R* refbar[4];      // adjoint of the ghost reference planes per side (accumulated)
  R* ai;             // face adjoint outputs, ADJ_FIELDS planes of (ni+1)*nj
  R* aj;             // ADJ_FIELDS planes of ni*(nj+1)
  R* qmbar;          // 8 planes
  R* qbar;           // output 4 planes
  const R* qbar_add; // optional: added to qbar (4 planes) or null
  R obj_scale, obj_dirx, obj_diry;  // drag objective: J = obj_scale * wall force along (dirx, diry)
};

// qmetric of cell c (phase 2 of the stage kernel, without tiling); NV variables
// (4 Euler, 3 scalar advection), 2 NV planes
template <class R, int NV = 4>
__device__ __forceinline__ void adj_qm_cell(const AdjArgs<R>& a, const R* __restrict__ q, R* qm, int c) {
  const int ni = a.ni, nj = a.nj;
  if (c >= ni * nj) return;
  const int gi = c / nj, gj = c % nj;
  const size_t n = size_t(ni) * nj;
  const bool per_i = a.bc[0] == BC_PERIODIC, per_j = a.bc[2] == BC_PERIODIC;
  const int nfi = (ni + 1) * nj, nfj = ni * (nj + 1);
  R m[2 * NV];
#pragma unroll
  for (int k = 0; k < 2 * NV; ++k) m[k] = R(0);
#pragma unroll
  for (int f = 0; f < 4; ++f) {
    const bool idir = f < 2;
    const int hi = f & 1;
    int fidx, nb;
    bool pair;
    if (idir) {
      const int fi = gi + hi;
      pair = (fi > 0 && fi < ni) || per_i;
      fidx = fi * nj + gj;
      nb = wrapi(gi + (hi ? 1 : -1), ni) * nj + gj;
    } else {
      const int fj = gj + hi;
      pair = (fj > 0 && fj < nj) || per_j;
      fidx = gi * (nj + 1) + fj;
      nb = gi * nj + wrapi(gj + (hi ? 1 : -1), nj);
    }
    if (!pair) continue;
    const R* rec = idir ? a.fi : a.fj;
    const int nf = idir ? nfi : nfj;
    const R dx = rec[size_t(F_DXX) * nf + fidx], dy = rec[size_t(F_DXY) * nf + fidx];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const R dq = hi ? (q[v * n + nb] - q[v * n + c]) : (q[v * n + c] - q[v * n + nb]);
      m[2 * v] += dq * dx;
      m[2 * v + 1] += dq * dy;
    }
  }
#pragma unroll
  for (int k = 0; k < 2 * NV; ++k) qm[k * n + c] = m[k];
}
template <class R, int NV = 4> __global__ void adj_qm_kernel(const AdjArgs<R> a, R* qm) {
  adj_qm_cell<R, NV>(a, a.q, qm, int(blockIdx.x * blockDim.x + threadIdx.x));
}

template <class R, int FK>
__device__ __forceinline__ void flux_adj(const Gas<R>& g, R nx, R ny, R A, const R* ql, const R* qr, const R* Fb,
                                         R* qlb, R* qrb) {
  if constexpr (FK == FLUX_ROE) roe_flux_adj(g, nx, ny, A, ql, qr, Fb, qlb, qrb);
  else if constexpr (FK == FLUX_RUSANOV) rusanov_flux_adj(g, nx, ny, A, ql, qr, Fb, qlb, qrb);
  else tangent_flux_adj<R, FK>(g, nx, ny, A, ql, qr, Fb, qlb, qrb);  // SLAU, AUSM+up, RoeUnprecWS
}

// pass 1: one thread per face of direction dir (0 = i-faces, 1 = j-faces)
// C: the type the face's reconstruction, flux and their reverse are computed in
// (R, or double-float for FP64 storage); loads and stores stay in R.
template <class R, int FK, class C = R>
__device__ __forceinline__ void adj_face_one(const AdjArgs<R>& a, int dir, int f) {
  const int ni = a.ni, nj = a.nj;
  const size_t n = size_t(ni) * nj;
  const bool idir = dir == 0;
  const int nf = idir ? (ni + 1) * nj : ni * (nj + 1);
  if (f >= nf) return;
  int i, j;
  if (idir) { i = f / nj; j = f % nj; } else { i = f / (nj + 1); j = f % (nj + 1); }
  const R* rec = idir ? a.fi : a.fj;
  R* out = idir ? a.ai : a.aj;
  auto rd = [&](int fld) -> C { return rec[size_t(fld) * nf + f]; };
  const C nx = rd(F_NX), ny = rd(F_NY), A = rd(F_A);
  const int lo = idir ? i : j, nalong = idir ? ni : nj;
  const int side = idir ? (lo == 0 ? 0 : 1) : (lo == 0 ? 2 : 3);
  const bool bnd = (lo == 0 || lo == nalong) && a.bc[side] != BC_PERIODIC;
  C res[ADJ_FIELDS];
#pragma unroll
  for (int k = 0; k < ADJ_FIELDS; ++k) res[k] = C(0);
  C* dL = res; C* dR = res + 4; C* gL = res + 8; C* gR = res + 12;
  const Gas<C> g = gas_as<C>(a.gas);
  const int lim = a.limiter;
  if (!bnd) {
    {
      // left/right cells (periodic wrap on the boundary lines)
      int cl, cr;
      if (idir) { cl = wrapi(i - 1, ni) * nj + j; cr = wrapi(i, ni) * nj + j; }
      else { cl = i * nj + wrapi(j - 1, nj); cr = i * nj + wrapi(j, nj); }
      C Fb[4], ql[4], qr[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        Fb[v] = a.rbar[v * n + cr] - a.rbar[v * n + cl];
        ql[v] = a.q[v * n + cl];
        qr[v] = a.q[v * n + cr];
      }
      if (lim == LIM_NOLIMIT1) {
        flux_adj<C, FK>(g, nx, ny, A, ql, qr, Fb, dL, dR);
      } else {
        const C dl = rd(F_DL), dr = rd(F_DR), idlr = rd(F_IDLR);
        const C wlx = rd(F_WLX), wly = rd(F_WLY), sl = rd(F_SL);
        const C wrx = rd(F_WRX), wry = rd(F_WRY), sr = rd(F_SR);
        C qL[4], qR[4], gc[4], gl[4], gr[4];
        // FP64 van Albada: values and derivatives of both sides from batched inversions
        constexpr bool f64 = std::is_same<C, double>::value;
        const bool vg = f64 && lim == LIM_VANALBADA;
        C dal[4], dbl[4], dar[4], dbr[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          const C dq = qr[v] - ql[v];
          gc[v] = dq * idlr;
          gl[v] = (a.qm[(2 * v) * n + cl] * wlx + a.qm[(2 * v + 1) * n + cl] * wly) - dq * sl;
          gr[v] = (a.qm[(2 * v) * n + cr] * wrx + a.qm[(2 * v + 1) * n + cr] * wry) - dq * sr;
        }
        if constexpr (f64) {
          if (vg) {
            C zl[4], zr[4];
            vanalbada_vg4(gc, gl, zl, dal, dbl);
            vanalbada_vg4(gc, gr, zr, dar, dbr);
#pragma unroll
            for (int v = 0; v < 4; ++v) {
              qL[v] = ql[v] + dl * zl[v];
              qR[v] = qr[v] - dr * zr[v];
            }
          }
        }
        if (!vg) {
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            qL[v] = ql[v] + dl * limit<C>(lim, gc[v], gl[v]);
            qR[v] = qr[v] - dr * limit<C>(lim, gc[v], gr[v]);
          }
        }
        C qLb[4] = {C(0), C(0), C(0), C(0)}, qRb[4] = {C(0), C(0), C(0), C(0)};
        flux_adj<C, FK>(g, nx, ny, A, qL, qR, Fb, qLb, qRb);
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          C da, db;
          if (vg) { da = dal[v]; db = dbl[v]; }
          else limit_grad<C>(lim, gc[v], gl[v], &da, &db);
          const C zlb = dl * qLb[v];
          C gcb = zlb * da;
          const C glb = zlb * db;
          if (vg) { da = dar[v]; db = dbr[v]; }
          else limit_grad<C>(lim, gc[v], gr[v], &da, &db);
          const C zrb = -dr * qRb[v];
          gcb += zrb * da;
          const C grb = zrb * db;
          const C dqb = gcb * idlr - glb * sl - grb * sr;
          dL[v] = qLb[v] - dqb;
          dR[v] = qRb[v] + dqb;
          gL[v] = glb;
          gR[v] = grb;
        }
      }
    }
  } else {
    const bool int_right = lo == 0;
    const int ci = idir ? (int_right ? 0 : ni - 1) * nj + j : i * nj + (int_right ? 0 : nj - 1);
    const int kf = idir ? j : i;
    const int nfs = idir ? nj : ni;
    const int bct = a.bc[side];
    C qi[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) qi[v] = a.q[v * n + ci];
    // the interior side's adjoints, moved to its slots of res at the end (a pointer chosen
    // at run time into res would put the whole array in local memory)
    C dI[4] = {C(0), C(0), C(0), C(0)}, gI[4] = {C(0), C(0), C(0), C(0)};
    if (bct == BC_WALL) {
      C Fb[4];
#pragma unroll
      for (int v = 0; v < 2; ++v) Fb[v] = int_right ? a.rbar[v * n + ci] : -a.rbar[v * n + ci];
      const C wx = int_right ? rd(F_WLX) : rd(F_WRX), wy = int_right ? rd(F_WLY) : rd(F_WRY);
      (void)wx; (void)wy;
      const C pb = A * (nx * Fb[0] + ny * Fb[1]);
      dI[3] += pb;
      gI[3] = -pb;  // pass 2 pairs it with the wall extrapolation weights
    } else {
      C Fb[4], qg[4];
      R qref[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        Fb[v] = int_right ? a.rbar[v * n + ci] : -a.rbar[v * n + ci];
        qref[v] = a.gref[side][size_t(v) * nfs + kf];
        qg[v] = qref[v];  // fixed ghost = reference state
      }
      const R sgn = int_right ? R(1) : R(-1);  // normal into the domain
      if constexpr (std::is_same<C, R>::value) {
        // Riemann / entropy far field: the ghost the forward stage computed from the
        // interior state and the reference state (in the storage type, as there)
        if (bct == BC_RIEMANN) farfield_update<R, BC_RIEMANN>(a.gas, sgn * nx, sgn * ny, qi, qref, qg);
        else if (bct == BC_ENTROPY) farfield_update<R, BC_ENTROPY>(a.gas, sgn * nx, sgn * ny, qi, qref, qg);
      }
      C qLb[4] = {C(0), C(0), C(0), C(0)}, qRb[4] = {C(0), C(0), C(0), C(0)};
      C gb_ref[4] = {C(0), C(0), C(0), C(0)};
      if (lim == LIM_NOLIMIT1) {
        if (int_right) { flux_adj<C, FK>(g, nx, ny, A, qg, qi, Fb, qLb, qRb); }
        else { flux_adj<C, FK>(g, nx, ny, A, qi, qg, Fb, qLb, qRb); }
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          dI[v] += int_right ? qRb[v] : qLb[v];
          gb_ref[v] = int_right ? qLb[v] : qRb[v];
        }
      } else {
        const C d = rd(F_DL), idlr = rd(F_IDLR);
        const C wx = int_right ? rd(F_WRX) : rd(F_WLX), wy = int_right ? rd(F_WRY) : rd(F_WLY);
        C qL[4], qR[4], gc[4], gbv[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          const C dq = int_right ? (qi[v] - qg[v]) : (qg[v] - qi[v]);
          gc[v] = dq * idlr;
          gbv[v] = a.qm[(2 * v) * n + ci] * wx + a.qm[(2 * v + 1) * n + ci] * wy;
          const C s = limit<C>(lim, gc[v], gbv[v]);
          if (int_right) { qL[v] = qg[v]; qR[v] = qi[v] - d * s; }
          else { qL[v] = qi[v] + d * s; qR[v] = qg[v]; }
        }
        flux_adj<C, FK>(g, nx, ny, A, qL, qR, Fb, qLb, qRb);
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          C da, db;
          limit_grad<C>(lim, gc[v], gbv[v], &da, &db);
          const C zb = int_right ? -d * qRb[v] : d * qLb[v];
          const C gcb = zb * da;
          gI[v] = zb * db;
          const C dqb = gcb * idlr;
          if (int_right) { dI[v] += qRb[v] + dqb; gb_ref[v] = qLb[v] - dqb; }
          else { dI[v] += qLb[v] - dqb; gb_ref[v] = qRb[v] + dqb; }
        }
      }
      if (bct == BC_FIXED) {
#pragma unroll
        for (int v = 0; v < 4; ++v) a.refbar[side][size_t(v) * nfs + kf] += cvt<R>(gb_ref[v]);
      } else if constexpr (std::is_same<C, R>::value) {
        // the ghost's adjoint through the far-field update, to the interior cell and the
        // reference state (forward-mode tangents, hc_tangent.cuh)
        R rb[4] = {R(0), R(0), R(0), R(0)};
        if (bct == BC_RIEMANN) farfield_adj<R, BC_RIEMANN>(a.gas, sgn * nx, sgn * ny, qi, qref, gb_ref, dI, rb);
        else farfield_adj<R, BC_ENTROPY>(a.gas, sgn * nx, sgn * ny, qi, qref, gb_ref, dI, rb);
#pragma unroll
        for (int v = 0; v < 4; ++v) a.refbar[side][size_t(v) * nfs + kf] += rb[v];
      }
    }
    if (int_right) {
#pragma unroll
      for (int v = 0; v < 4; ++v) { dR[v] = dI[v]; gR[v] = gI[v]; }
    } else {
#pragma unroll
      for (int v = 0; v < 4; ++v) { dL[v] = dI[v]; gL[v] = gI[v]; }
    }
  }
#pragma unroll
  for (int k = 0; k < ADJ_FIELDS; ++k) out[size_t(k) * nf + f] = cvt<R>(res[k]);
}
// both face directions in one launch: i-faces in blocks [0, nbi), j-faces in the rest
template <class R, int FK, class C = R> __global__ void adj_face_kernel(const AdjArgs<R> a, int nbi) {
  const int b = int(blockIdx.x);
  const int dir = b < nbi ? 0 : 1;
  adj_face_one<R, FK, C>(a, dir, (dir ? b - nbi : b) * int(blockDim.x) + int(threadIdx.x));
}

// ---- scalar advection law (conserved set {u, v, q}; scalar_face_flux, hc_scalar.cuh)
enum { SADJ_FIELDS = 12 };  // dL[3], dR[3], gL[3], gR[3]

// Reverse of scalar_face_flux for the three flux components (the spectral radius
// feeds only the frozen timestep): Fb -> qlb, qrb (accumulated).  Ties of the
// Rusanov max and the kink of |u_n| take the branches of the forward-mode reference
// (the left side on a tie, derivative 0 at u_n = 0).
template <class R, int FK>
__host__ __device__ __forceinline__ void scalar_flux_adj(R nx, R ny, R A, const R* ql, const R* qr, const R* Fb,
                                                         R* qlb, R* qrb) {
  const R unl = nx * ql[0] + ny * ql[1];
  const R unr = nx * qr[0] + ny * qr[1];
  const R t = R(0.5) * A * Fb[2];
  R unlb = t * ql[2], unrb = t * qr[2];
  qlb[2] += t * unl;
  qrb[2] += t * unr;
  if constexpr (FK == FLUX_RUSANOV) {
    const R al = fabs(unl), ar = fabs(unr);
    const R c = R(-0.5) * (fmax(al, ar) * A);
    R cb = R(0);
#pragma unroll
    for (int v = 0; v < 3; ++v) {
      cb += Fb[v] * (qr[v] - ql[v]);
      qrb[v] += c * Fb[v];
      qlb[v] -= c * Fb[v];
    }
    const R mb = R(-0.5) * A * cb;
    if (al >= ar) unlb += sgn(unl) * mb;
    else unrb += sgn(unr) * mb;
  }
  qlb[0] += nx * unlb; qlb[1] += ny * unlb;
  qrb[0] += nx * unrb; qrb[1] += ny * unrb;
}

// pass 1 of the scalar law: one thread per face of direction dir.  Interior and
// periodic faces: flux, limiter and reconstruction reversed; Fixed and Riemann
// boundary faces: the interior side reversed and the ghost side's adjoint added to the
// reference adjoint (or, where the Riemann ghost copied the interior, to the cell's).  Writes SADJ_FIELDS planes (the Euler layout with three variables).
template <class R, int FK> __device__ __forceinline__ void adj_face_scalar_one(const AdjArgs<R>& a, int dir, int f) {
  const int ni = a.ni, nj = a.nj;
  const size_t n = size_t(ni) * nj;
  const bool idir = dir == 0;
  const int nf = idir ? (ni + 1) * nj : ni * (nj + 1);
  if (f >= nf) return;
  int i, j;
  if (idir) { i = f / nj; j = f % nj; } else { i = f / (nj + 1); j = f % (nj + 1); }
  const R* rec = idir ? a.fi : a.fj;
  R* out = idir ? a.ai : a.aj;
  auto rd = [&](int fld) -> R { return rec[size_t(fld) * nf + f]; };
  const R nx = rd(F_NX), ny = rd(F_NY), A = rd(F_A);
  const int lo = idir ? i : j, nalong = idir ? ni : nj;
  const int side = idir ? (lo == 0 ? 0 : 1) : (lo == 0 ? 2 : 3);
  const bool bnd = (lo == 0 || lo == nalong) && a.bc[side] != BC_PERIODIC;
  R res[SADJ_FIELDS];
#pragma unroll
  for (int k = 0; k < SADJ_FIELDS; ++k) res[k] = R(0);
  R* dL = res; R* dR = res + 3; R* gL = res + 6; R* gR = res + 9;
  const int lim = a.limiter;
  if (!bnd) {
    int cl, cr;
    if (idir) { cl = wrapi(i - 1, ni) * nj + j; cr = wrapi(i, ni) * nj + j; }
    else { cl = i * nj + wrapi(j - 1, nj); cr = i * nj + wrapi(j, nj); }
    R Fb[3], ql[3], qr[3];
#pragma unroll
    for (int v = 0; v < 3; ++v) {
      Fb[v] = a.rbar[v * n + cr] - a.rbar[v * n + cl];
      ql[v] = a.q[v * n + cl];
      qr[v] = a.q[v * n + cr];
    }
    if (lim == LIM_NOLIMIT1) {
      scalar_flux_adj<R, FK>(nx, ny, A, ql, qr, Fb, dL, dR);
    } else {
      const R dl = rd(F_DL), dr = rd(F_DR), idlr = rd(F_IDLR);
      const R wlx = rd(F_WLX), wly = rd(F_WLY), sl = rd(F_SL);
      const R wrx = rd(F_WRX), wry = rd(F_WRY), sr = rd(F_SR);
      R qL[3], qR[3], gc[3], gl[3], gr[3];
#pragma unroll
      for (int v = 0; v < 3; ++v) {
        const R dq = qr[v] - ql[v];
        gc[v] = dq * idlr;
        gl[v] = (a.qm[(2 * v) * n + cl] * wlx + a.qm[(2 * v + 1) * n + cl] * wly) - dq * sl;
        gr[v] = (a.qm[(2 * v) * n + cr] * wrx + a.qm[(2 * v + 1) * n + cr] * wry) - dq * sr;
        qL[v] = ql[v] + dl * limit<R>(lim, gc[v], gl[v]);
        qR[v] = qr[v] - dr * limit<R>(lim, gc[v], gr[v]);
      }
      R qLb[3] = {R(0), R(0), R(0)}, qRb[3] = {R(0), R(0), R(0)};
      scalar_flux_adj<R, FK>(nx, ny, A, qL, qR, Fb, qLb, qRb);
#pragma unroll
      for (int v = 0; v < 3; ++v) {
        R da, db;
        limit_grad<R>(lim, gc[v], gl[v], &da, &db);
        const R zlb = dl * qLb[v];
        R gcb = zlb * da;
        const R glb = zlb * db;
        limit_grad<R>(lim, gc[v], gr[v], &da, &db);
        const R zrb = -dr * qRb[v];
        gcb += zrb * da;
        const R grb = zrb * db;
        const R dqb = gcb * idlr - glb * sl - grb * sr;
        dL[v] = qLb[v] - dqb;
        dR[v] = qRb[v] + dqb;
        gL[v] = glb;
        gR[v] = grb;
      }
    }
  } else {
    const bool int_right = lo == 0;
    const int ci = idir ? (int_right ? 0 : ni - 1) * nj + j : i * nj + (int_right ? 0 : nj - 1);
    const int kf = idir ? j : i;
    const int nfs = idir ? nj : ni;
    R dI[3] = {R(0), R(0), R(0)}, gI[3] = {R(0), R(0), R(0)};  // moved to res at the end
    R Fb[3], qi[3], qg[3], qref[3];
#pragma unroll
    for (int v = 0; v < 3; ++v) {
      Fb[v] = int_right ? a.rbar[v * n + ci] : -a.rbar[v * n + ci];
      qi[v] = a.q[v * n + ci];
      qref[v] = a.gref[side][size_t(v) * nfs + kf];
      qg[v] = qref[v];
    }
    // Riemann ghost: the reference value on inflow, the interior value on outflow (the
    // switch itself has no derivative); the ghost's adjoint goes to whichever it copied
    bool ghost_is_ref = true;
    if (a.bc[side] == BC_RIEMANN) {
      const R sgn = int_right ? R(1) : R(-1);  // normal into the domain
      ghost_is_ref = scalar_riemann_ghost(sgn * nx, sgn * ny, qi, qref, qg);
    }
    R qLb[3] = {R(0), R(0), R(0)}, qRb[3] = {R(0), R(0), R(0)};
    R gb_ref[3] = {R(0), R(0), R(0)};
    if (lim == LIM_NOLIMIT1) {
      if (int_right) scalar_flux_adj<R, FK>(nx, ny, A, qg, qi, Fb, qLb, qRb);
      else scalar_flux_adj<R, FK>(nx, ny, A, qi, qg, Fb, qLb, qRb);
#pragma unroll
      for (int v = 0; v < 3; ++v) {
        dI[v] += int_right ? qRb[v] : qLb[v];
        gb_ref[v] = int_right ? qLb[v] : qRb[v];
      }
    } else {
      const R d = rd(F_DL), idlr = rd(F_IDLR);
      const R wx = int_right ? rd(F_WRX) : rd(F_WLX), wy = int_right ? rd(F_WRY) : rd(F_WLY);
      R qL[3], qR[3], gc[3], gbv[3];
#pragma unroll
      for (int v = 0; v < 3; ++v) {
        const R dq = int_right ? (qi[v] - qg[v]) : (qg[v] - qi[v]);
        gc[v] = dq * idlr;
        gbv[v] = a.qm[(2 * v) * n + ci] * wx + a.qm[(2 * v + 1) * n + ci] * wy;
        const R sv = limit<R>(lim, gc[v], gbv[v]);
        if (int_right) { qL[v] = qg[v]; qR[v] = qi[v] - d * sv; }
        else { qL[v] = qi[v] + d * sv; qR[v] = qg[v]; }
      }
      scalar_flux_adj<R, FK>(nx, ny, A, qL, qR, Fb, qLb, qRb);
#pragma unroll
      for (int v = 0; v < 3; ++v) {
        R da, db;
        limit_grad<R>(lim, gc[v], gbv[v], &da, &db);
        const R zb = int_right ? -d * qRb[v] : d * qLb[v];
        gI[v] = zb * db;
        const R dqb = zb * da * idlr;
        if (int_right) { dI[v] += qRb[v] + dqb; gb_ref[v] = qLb[v] - dqb; }
        else { dI[v] += qLb[v] - dqb; gb_ref[v] = qRb[v] + dqb; }
      }
    }
#pragma unroll
    for (int v = 0; v < 3; ++v) {
      if (ghost_is_ref) a.refbar[side][size_t(v) * nfs + kf] += gb_ref[v];
      else dI[v] += gb_ref[v];
    }
    if (int_right) {
#pragma unroll
      for (int v = 0; v < 3; ++v) { dR[v] = dI[v]; gR[v] = gI[v]; }
    } else {
#pragma unroll
      for (int v = 0; v < 3; ++v) { dL[v] = dI[v]; gL[v] = gI[v]; }
    }
  }
#pragma unroll
  for (int k = 0; k < SADJ_FIELDS; ++k) out[size_t(k) * nf + f] = res[k];
}
template <class R, int FK> __global__ void adj_face_scalar_kernel(const AdjArgs<R> a, int dir) {
  adj_face_scalar_one<R, FK>(a, dir, int(blockIdx.x * blockDim.x + threadIdx.x));
}

// Reverse of a stage update that is linear on the conserved set, q_out = q0 + (sum_k
// alpha_k R_k) fac (the scalar law), fac = beta dt / V frozen: q0bar += qbar_out,
// rbar_k += alpha_k fac qbar_out.
template <class R, int NV>
__device__ __forceinline__ void adj_update_lin_cell(int ncell, const R* __restrict__ vol,
                                                    const R* __restrict__ qbar_out, R* __restrict__ q0bar, R* rbar0,
                                                    R* rbar1, R* rbar2, R* rbar3, R alpha0, R alpha1, R alpha2,
                                                    R alpha3, int stage, R dts, int c) {
  if (c >= ncell) return;
  const size_t n = size_t(ncell);
  const R fac = dts / vol[c];
  R* rb[4] = {rbar0, rbar1, rbar2, rbar3};
  const R al[4] = {alpha0, alpha1, alpha2, alpha3};
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    const R qb = qbar_out[v * n + c];
    q0bar[v * n + c] += qb;
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (k <= stage) rb[k][v * n + c] += al[k] * qb * fac;
  }
}
template <class R, int NV>
__global__ void adj_update_lin_kernel(int ncell, const R* __restrict__ vol, const R* __restrict__ qbar_out,
                                      R* __restrict__ q0bar, R* rbar0, R* rbar1, R* rbar2, R* rbar3, R alpha0,
                                      R alpha1, R alpha2, R alpha3, int stage, R dts) {
  adj_update_lin_cell<R, NV>(ncell, vol, qbar_out, q0bar, rbar0, rbar1, rbar2, rbar3, alpha0, alpha1, alpha2, alpha3,
                             stage, dts, int(blockIdx.x * blockDim.x + threadIdx.x));
}

// pass 2: qmetric adjoint of cell c (NV variables; face fields dL, dR, gL, gR of NV each)
template <class R, int NV = 4> __device__ __forceinline__ void adj_qmbar_cell(const AdjArgs<R>& a, int c) {
  const int ni = a.ni, nj = a.nj;
  if (c >= ni * nj) return;
  const int gi = c / nj, gj = c % nj;
  const size_t n = size_t(ni) * nj;
  const int nfi = (ni + 1) * nj, nfj = ni * (nj + 1);
  R m[2 * NV];
#pragma unroll
  for (int k = 0; k < 2 * NV; ++k) m[k] = R(0);
#pragma unroll
  for (int f = 0; f < 4; ++f) {
    const bool idir = f < 2;
    const int hi = f & 1;  // hi: c is the left cell of this face
    const int lo = idir ? gi + hi : gj + hi;
    const int nalong = idir ? ni : nj;
    const int side = idir ? (lo == 0 ? 0 : 1) : (lo == 0 ? 2 : 3);
    const bool bnd = (lo == 0 || lo == nalong) && a.bc[side] != BC_PERIODIC;
    const int fidx = idir ? lo * nj + gj : gi * (nj + 1) + lo;
    const int nf = idir ? nfi : nfj;
    const R* rec = idir ? a.fi : a.fj;
    const R* adj = idir ? a.ai : a.aj;
    const bool wall = bnd && a.bc[side] == BC_WALL;
    // c is left (hi) -> gL with wL, right -> gR with wR; wall faces keep the
    // extrapolation weights in the other side's slots
    const bool use_left_slot = wall ? !hi : hi;
    const R wx = rec[size_t(use_left_slot ? F_WLX : F_WRX) * nf + fidx];
    const R wy = rec[size_t(use_left_slot ? F_WLY : F_WRY) * nf + fidx];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const R gv = adj[size_t(hi ? 2 * NV + v : 3 * NV + v) * nf + fidx];
      m[2 * v] += gv * wx;
      m[2 * v + 1] += gv * wy;
    }
  }
#pragma unroll
  for (int k = 0; k < 2 * NV; ++k) a.qmbar[k * n + c] = m[k];
}
template <class R, int NV = 4> __global__ void adj_qmbar_kernel(const AdjArgs<R> a) {
  adj_qmbar_cell<R, NV>(a, int(blockIdx.x * blockDim.x + threadIdx.x));
}

// pass 3: gather the state adjoint of cell c (NV variables) into qb
template <class R, int NV>
__device__ __forceinline__ void adj_gather_vals(const AdjArgs<R>& a, int c, R* qb) {
  const int ni = a.ni, nj = a.nj;
  const int gi = c / nj, gj = c % nj;
  const size_t n = size_t(ni) * nj;
  const int nfi = (ni + 1) * nj, nfj = ni * (nj + 1);
  const bool per_i = a.bc[0] == BC_PERIODIC, per_j = a.bc[2] == BC_PERIODIC;
#pragma unroll
  for (int v = 0; v < NV; ++v) qb[v] = a.qbar_add ? a.qbar_add[v * n + c] : R(0);
#pragma unroll
  for (int f = 0; f < 4; ++f) {
    const bool idir = f < 2;
    const int hi = f & 1;
    const int lo = idir ? gi + hi : gj + hi;
    const int fidx = idir ? lo * nj + gj : gi * (nj + 1) + lo;
    const int nf = idir ? nfi : nfj;
    const R* adj = idir ? a.ai : a.aj;
#pragma unroll
    for (int v = 0; v < NV; ++v) qb[v] += adj[size_t(hi ? v : NV + v) * nf + fidx];
    const bool pair = idir ? ((lo > 0 && lo < ni) || per_i) : ((lo > 0 && lo < nj) || per_j);
    if (!pair) continue;
    const R* rec = idir ? a.fi : a.fj;
    const R dx = rec[size_t(F_DXX) * nf + fidx], dy = rec[size_t(F_DXY) * nf + fidx];
    const int nb = idir ? wrapi(gi + (hi ? 1 : -1), ni) * nj + gj : gi * nj + wrapi(gj + (hi ? 1 : -1), nj);
    const R sg = hi ? R(-1) : R(1);  // c left of the face -> -1
#pragma unroll
    for (int v = 0; v < NV; ++v)
      qb[v] += sg * ((a.qmbar[(2 * v) * n + c] + a.qmbar[(2 * v) * n + nb]) * dx +
                     (a.qmbar[(2 * v + 1) * n + c] + a.qmbar[(2 * v + 1) * n + nb]) * dy);
  }
}
template <class R, int NV = 4> __device__ __forceinline__ void adj_gather_cell(const AdjArgs<R>& a, int c) {
  if (c >= a.ni * a.nj) return;
  const size_t n = size_t(a.ni) * a.nj;
  R qb[NV];
  adj_gather_vals<R, NV>(a, c, qb);
#pragma unroll
  for (int v = 0; v < NV; ++v) a.qbar[v * n + c] = qb[v];
}
template <class R, int NV = 4> __global__ void adj_gather_kernel(const AdjArgs<R> a) {
  adj_gather_cell<R, NV>(a, int(blockIdx.x * blockDim.x + threadIdx.x));
}

// Reverse of one stage update q_out = prim(cons(q0) + (sum_k alpha_k R_k) * fac),
// fac = beta*dt/V frozen, at cell c: qb (the adjoint of q_out) -> q0bar and rbar_k (k <=
// stage), accumulated, or (first: the step's last stage, the first update reversed)
// written, which spares zeroing them
template <class R>
__device__ __forceinline__ void adj_update_apply(const Gas<R>& g, const R* __restrict__ q_out,
                                                 const R* __restrict__ q0, const R* __restrict__ vol, const R* qb,
                                                 R* __restrict__ q0bar, R* const* rbar, const R* alpha, int stage,
                                                 R dts, size_t n, int c, bool first) {
  R q[4], qz[4], cb[4], z[4] = {R(0), R(0), R(0), R(0)};
#pragma unroll
  for (int v = 0; v < 4; ++v) { q[v] = q_out[v * n + c]; qz[v] = q0[v * n + c]; }
  cons2prim_adj(g, q, qb, cb);
  prim2cons_adj(g, qz, cb, z);
  const R fac = dts / vol[c];
  if (first) {
#pragma unroll
    for (int v = 0; v < 4; ++v) q0bar[v * n + c] = z[v];
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (k <= stage)
#pragma unroll
        for (int v = 0; v < 4; ++v) rbar[k][v * n + c] = alpha[k] * cb[v] * fac;
  } else {
#pragma unroll
    for (int v = 0; v < 4; ++v) q0bar[v * n + c] += z[v];
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (k <= stage)
#pragma unroll
        for (int v = 0; v < 4; ++v) rbar[k][v * n + c] += alpha[k] * cb[v] * fac;
  }
}

// ---- the drag objective's adjoint
// J = obj_scale * sum over wall faces of -sgn_in A p_wall (n . dir), p_wall = p_c - QM_c(p) . w
// (the wall pressure extrapolated with the cell's LSQ gradient, inviscidWall.ipp:33-72).
// Per wall face: pb = A (n . Fb), Fb = -sgn_in obj_scale dir; p_c takes pb directly and
// the cell's pressure qmetric adjoint -pb w, which the gather spreads over the cell and
// its pair neighbours.  wall_pb: pb and w of wall face k of `side`.
template <class R>
__device__ __forceinline__ void wall_pb(const AdjArgs<R>& a, int side, int k, R& pb, R& wx, R& wy) {
  const bool idir = side < 2, int_right = side == 0 || side == 2;
  const int ni = a.ni, nj = a.nj;
  const int nf = idir ? (ni + 1) * nj : ni * (nj + 1);
  const int fidx = idir ? (side == 0 ? 0 : ni) * nj + k : k * (nj + 1) + (side == 2 ? 0 : nj);
  const R* rec = idir ? a.fi : a.fj;
  const R nx = rec[size_t(F_NX) * nf + fidx], ny = rec[size_t(F_NY) * nf + fidx], A = rec[size_t(F_A) * nf + fidx];
  const R sgn_in = int_right ? R(1) : R(-1);
  const R fb0 = -sgn_in * a.obj_scale * a.obj_dirx, fb1 = -sgn_in * a.obj_scale * a.obj_diry;
  pb = A * (nx * fb0 + ny * fb1);
  wx = rec[size_t(int_right ? F_WLX : F_WRX) * nf + fidx];
  wy = rec[size_t(int_right ? F_WLY : F_WRY) * nf + fidx];
}
// the pressure qmetric adjoint (m6, m7) of cell (ci, cj) from its wall faces; false: none
template <class R> __device__ __forceinline__ bool drag_qmbar(const AdjArgs<R>& a, int ci, int cj, R& m6, R& m7) {
  bool any = false;
  m6 = m7 = R(0);
#pragma unroll
  for (int f = 0; f < 4; ++f) {
    const int side = f;  // face order of the qmetric: i-lo, i-hi, j-lo, j-hi = sides 0..3
    const bool on = side == 0 ? ci == 0 : side == 1 ? ci == a.ni - 1 : side == 2 ? cj == 0 : cj == a.nj - 1;
    if (!on || a.bc[side] != BC_WALL) continue;
    R pb, wx, wy;
    wall_pb(a, side, side < 2 ? cj : ci, pb, wx, wy);
    m6 += -pb * wx;
    m7 += -pb * wy;
    any = true;
  }
  return any;
}
// the drag adjoint of cell c's pressure: its wall faces' pb and the pair-face spread of
// the pressure qmetric adjoints of c and its neighbours (zero away from the walls)
template <class R> __device__ __forceinline__ R drag_cell(const AdjArgs<R>& a, int c) {
  const int ni = a.ni, nj = a.nj;
  const int gi = c / nj, gj = c % nj;
  const bool per_i = a.bc[0] == BC_PERIODIC, per_j = a.bc[2] == BC_PERIODIC;
  R out = R(0);
  R m6c, m7c;
  const bool mc = drag_qmbar(a, gi, gj, m6c, m7c);
#pragma unroll
  for (int f = 0; f < 4; ++f) {
    const bool idir = f < 2;
    const int hi = f & 1;
    const int lo = idir ? gi + hi : gj + hi;
    const int nalong = idir ? ni : nj;
    const int side = idir ? (lo == 0 ? 0 : 1) : (lo == 0 ? 2 : 3);
    if ((lo == 0 || lo == nalong) && a.bc[side] == BC_WALL) {
      R pb, wx, wy;
      wall_pb(a, side, idir ? gj : gi, pb, wx, wy);
      out += pb;
    }
    const bool pair = idir ? ((lo > 0 && lo < ni) || per_i) : ((lo > 0 && lo < nj) || per_j);
    if (!pair) continue;
    const int ni_ = idir ? wrapi(gi + (hi ? 1 : -1), ni) : gi, nj_ = idir ? gj : wrapi(gj + (hi ? 1 : -1), nj);
    R m6n, m7n;
    const bool mn = drag_qmbar(a, ni_, nj_, m6n, m7n);
    if (!mc && !mn) continue;
    const int nf = idir ? (ni + 1) * nj : ni * (nj + 1);
    const int fidx = idir ? lo * nj + gj : gi * (nj + 1) + lo;
    const R* rec = idir ? a.fi : a.fj;
    const R dx = rec[size_t(F_DXX) * nf + fidx], dy = rec[size_t(F_DXY) * nf + fidx];
    const R sg = hi ? R(-1) : R(1);
    out += sg * ((m6c + m6n) * dx + (m7c + m7n) * dy);
  }
  return out;
}

// ---- the fused cell pass of the Euler reverse (single mesh): per cell,
//   qb = gather of the face adjoints (pass 3, qbar_add included) | qbar_in | 0
//   qb.p += the drag objective's adjoint (drag)
//   update: the RK update of the stage before reversed with qbar_out = qb; else qb -> qbar_out
//   qm_q: the qmetric of that stage's state for the next face pass
// so that a stage's reverse is three launches: faces, qmetric adjoint, this pass.
template <class R> struct AdjCellArgs {
  int gather, drag, update;
  int first;  // the step's first update reversed: writes q0bar and the rbar_k instead of adding
  const R* qbar_in;
  R* qbar_out;
  Gas<R> g;
  const R* q_out;
  const R* q0;
  const R* vol;
  R* q0bar;
  R* rbar[4];
  R alpha[4];
  int stage;
  R dts;
  const R* qm_q;
};
template <class R> __device__ __forceinline__ void adj_cell_body(const AdjArgs<R>& a, const AdjCellArgs<R>& u, int c) {
  const int ncell = a.ni * a.nj;
  if (c >= ncell) return;
  const size_t n = size_t(ncell);
  R qb[4];
  if (u.gather) {
    adj_gather_vals<R, 4>(a, c, qb);
  } else {
#pragma unroll
    for (int v = 0; v < 4; ++v) qb[v] = u.qbar_in ? u.qbar_in[v * n + c] : R(0);
  }
  if (u.drag) qb[3] += drag_cell(a, c);
  if (u.update) {
    adj_update_apply(u.g, u.q_out, u.q0, u.vol, qb, u.q0bar, u.rbar, u.alpha, u.stage, u.dts, n, c, u.first != 0);
  } else {
#pragma unroll
    for (int v = 0; v < 4; ++v) u.qbar_out[v * n + c] = qb[v];
  }
  if (u.qm_q) adj_qm_cell<R, 4>(a, u.qm_q, const_cast<R*>(a.qm), c);
}
// the cell pass is bound by memory latency: residency over registers (FP32 8 blocks of 256,
// FP64 6; measured on the 64-instance FP32 batch, 2.93 s against 3.29 s at the default)
template <int R_BYTES> struct CellResidency {
  static constexpr int value = R_BYTES == 4 ? 8 : 6;
};
template <class R>
__global__ void __launch_bounds__(256, CellResidency<sizeof(R)>::value)
    adj_cell_kernel(const AdjArgs<R> a, const AdjCellArgs<R> u) {
  adj_cell_body(a, u, int(blockIdx.x * blockDim.x + threadIdx.x));
}

// Drag of the wall faces of the state q (force on the body along (dirx, diry)
// times scale): per face -sgn_in * A * p_wall * (n . dir) * scale, written to
// out[k] for wall face k of the flattened wall-face list of the side.
template <class R>
__global__ void wall_force_kernel(const AdjArgs<R> a, const R* qm, int side, R* out) {
  const int ni = a.ni, nj = a.nj;
  const size_t n = size_t(ni) * nj;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int nfs = side < 2 ? nj : ni;
  if (k >= nfs) return;
  const bool idir = side < 2;
  const bool int_right = side == 0 || side == 2;
  const int i = idir ? (int_right ? 0 : ni) : k;
  const int j = idir ? k : (int_right ? 0 : nj);
  const int nf = idir ? (ni + 1) * nj : ni * (nj + 1);
  const int fidx = idir ? i * nj + j : i * (nj + 1) + j;
  const R* rec = idir ? a.fi : a.fj;
  const R nx = rec[size_t(F_NX) * nf + fidx], ny = rec[size_t(F_NY) * nf + fidx], A = rec[size_t(F_A) * nf + fidx];
  const R wx = rec[size_t(int_right ? F_WLX : F_WRX) * nf + fidx];
  const R wy = rec[size_t(int_right ? F_WLY : F_WRY) * nf + fidx];
  const int ci = idir ? (int_right ? 0 : ni - 1) * nj + j : i * nj + (int_right ? 0 : nj - 1);
  const R pw = a.q[3 * n + ci] - (qm[6 * n + ci] * wx + qm[7 * n + ci] * wy);
  const R sgn_in = int_right ? R(1) : R(-1);
  out[k] = -sgn_in * A * pw * (nx * a.obj_dirx + ny * a.obj_diry) * a.obj_scale;
}

// ---------------------------------------------------------------- batched launches
// The reverse passes of every instance of a batch (hc_batch_adjoint.cu), one grid
// per pass.  The grid is cut into segments -- one per instance for the cell
// passes, one per instance and face direction for the face pass -- with seg[s]
// the first block of segment s (nseg + 1 ascending entries).  A block finds its
// segment by binary search, thread 0 writes the instance's AdjArgs (its slices of
// the pools) to shared memory, and the block runs the single-mesh body on them:
// every instance gets exactly the arithmetic of a single-mesh adjoint.
template <class R> struct AdjBatchArgs {
  const BatchInst* inst;
  const int* seg;
  int nseg;
  Gas<R> gas;
  int limiter;
  const R* q;         // stage state pool (4 planes per instance at 4*cell)
  R* qm;              // qmetric pool (8 planes per instance at 8*cell)
  const R* rbar;      // residual adjoint pool (4*cell)
  const R* fi;        // face records (FREC planes per instance at FREC*fi / FREC*fj)
  const R* fj;
  const R* gref;      // ghost reference pool (per side at inst.gref[side])
  R* refbar;          // its adjoint, same layout
  R* ai;              // face adjoint pools (ADJ_FIELDS planes per instance at ADJ_FIELDS*fi / *fj)
  R* aj;
  R* qmbar;           // 8*cell
  R* qbar;            // 4*cell
  const R* qbar_add;  // 4*cell or null
};

__device__ __forceinline__ int find_segment(const int* seg, int nseg, int block) {
  int lo = 0, hi = nseg - 1;  // the largest s with seg[s] <= block
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (seg[mid] <= block) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

template <class R> __device__ __forceinline__ void batch_adj_args(const AdjBatchArgs<R>& b, int k, AdjArgs<R>& a) {
  const BatchInst& in = b.inst[k];
  a.ni = in.ni; a.nj = in.nj;
  for (int s = 0; s < 4; ++s) a.bc[s] = in.bc[s];
  a.gas = b.gas;
  a.limiter = b.limiter;
  const long long c4 = 4 * in.cell, c8 = 8 * in.cell;
  a.q = b.q + c4;
  a.qm = b.qm + c8;
  a.rbar = b.rbar ? b.rbar + c4 : nullptr;
  a.fi = b.fi + (long long)FREC * in.fi;
  a.fj = b.fj + (long long)FREC * in.fj;
  for (int s = 0; s < 4; ++s) { a.gref[s] = b.gref + in.gref[s]; a.refbar[s] = b.refbar + in.gref[s]; }
  a.ai = b.ai + (long long)ADJ_FIELDS * in.fi;
  a.aj = b.aj + (long long)ADJ_FIELDS * in.fj;
  a.qmbar = b.qmbar + c8;
  a.qbar = b.qbar ? b.qbar + c4 : nullptr;
  a.qbar_add = b.qbar_add ? b.qbar_add + c4 : nullptr;
  a.obj_scale = a.obj_dirx = a.obj_diry = R(0);
}

// the block's instance arguments in shared memory and its block index within the segment
template <class R> struct AdjBlock {
  AdjArgs<R> a;
  int local;  // block index within the segment
  int seg;
};
template <class R> __device__ __forceinline__ void adj_block_setup(const AdjBatchArgs<R>& b, int per_inst,
                                                                   AdjBlock<R>& sb) {
  if (threadIdx.x == 0) {
    const int s = find_segment(b.seg, b.nseg, int(blockIdx.x));
    batch_adj_args(b, s / per_inst, sb.a);
    sb.local = int(blockIdx.x) - b.seg[s];
    sb.seg = s;
  }
  __syncthreads();
}

// (a scalar-law batch keeps the pools' 4-plane state, 8-plane qmetric and
// ADJ_FIELDS-plane face slabs and uses the first NV, 2 NV and SADJ_FIELDS planes)
template <class R, int NV = 4> __global__ void adj_qm_batch_kernel(const AdjBatchArgs<R> b) {
  __shared__ AdjBlock<R> sb;
  adj_block_setup(b, 1, sb);
  adj_qm_cell<R, NV>(sb.a, sb.a.q, const_cast<R*>(sb.a.qm), sb.local * int(blockDim.x) + int(threadIdx.x));
}
template <class R, int FK, class C = R> __global__ void adj_face_batch_kernel(const AdjBatchArgs<R> b) {
  __shared__ AdjBlock<R> sb;
  adj_block_setup(b, 2, sb);
  adj_face_one<R, FK, C>(sb.a, sb.seg & 1, sb.local * int(blockDim.x) + int(threadIdx.x));
}
template <class R, int FK> __global__ void adj_face_scalar_batch_kernel(const AdjBatchArgs<R> b) {
  __shared__ AdjBlock<R> sb;
  adj_block_setup(b, 2, sb);
  adj_face_scalar_one<R, FK>(sb.a, sb.seg & 1, sb.local * int(blockDim.x) + int(threadIdx.x));
}
template <class R, int NV = 4> __global__ void adj_qmbar_batch_kernel(const AdjBatchArgs<R> b) {
  __shared__ AdjBlock<R> sb;
  adj_block_setup(b, 1, sb);
  adj_qmbar_cell<R, NV>(sb.a, sb.local * int(blockDim.x) + int(threadIdx.x));
}
template <class R, int NV = 4> __global__ void adj_gather_batch_kernel(const AdjBatchArgs<R> b) {
  __shared__ AdjBlock<R> sb;
  adj_block_setup(b, 1, sb);
  adj_gather_cell<R, NV>(sb.a, sb.local * int(blockDim.x) + int(threadIdx.x));
}

// Reverse of one stage update of a scalar-law batch for every instance (the Euler batch
// reverses its updates in the fused cell pass); the frozen timestep of each instance is
// cfl / max rate of the step, as the forward run took it.
template <class R> struct AdjUpdateBatch {
  const BatchInst* inst;
  const int* seg;  // the cell-pass segments
  int nseg;
  Gas<R> g;
  const R* q_out;
  const R* q0;
  const R* vol;
  const R* qbar_out;
  R* q0bar;
  R* rbar[4];
  R alpha[4];
  int stage;
  double beta, cfl;
  const double* rates;  // max rates of the step, one per instance
};
// the fused cell pass (adj_cell_body) for every instance of a batch: the pool pointers of
// u shifted to the block's instance, its own frozen timestep
template <class R> struct AdjCellBatch {
  AdjCellArgs<R> u;  // pool pointers; dts unused
  double beta, cfl;
  const double* rates;  // max rates of the step, one per instance
};
template <class R>
__global__ void __launch_bounds__(256, CellResidency<sizeof(R)>::value)
    adj_cell_batch_kernel(const AdjBatchArgs<R> b, const AdjCellBatch<R> ub) {
  __shared__ AdjBlock<R> sb;
  adj_block_setup(b, 1, sb);
  const BatchInst& in = b.inst[sb.seg];
  const long long c4 = 4 * in.cell;
  AdjCellArgs<R> u = ub.u;
  u.qbar_in = u.qbar_in ? u.qbar_in + c4 : nullptr;
  u.qbar_out = u.qbar_out ? u.qbar_out + c4 : nullptr;
  u.q_out = u.q_out ? u.q_out + c4 : nullptr;
  u.q0 = u.q0 ? u.q0 + c4 : nullptr;
  u.vol = u.vol ? u.vol + in.cell : nullptr;
  u.q0bar = u.q0bar ? u.q0bar + c4 : nullptr;
  for (int k = 0; k < 4; ++k) u.rbar[k] = u.rbar[k] ? u.rbar[k] + c4 : nullptr;
  u.qm_q = u.qm_q ? u.qm_q + c4 : nullptr;
  u.dts = R(ub.beta * (ub.cfl / fmax(DBL_MIN, ub.rates[sb.seg])));
  adj_cell_body(sb.a, u, sb.local * int(blockDim.x) + int(threadIdx.x));
}

// Face passes of the Euler fluxes reversed by tangents (flux SLAU, SLAU as written,
// AUSM+up, RoeUnprecWS or the face-frame Roe), compiled in their own unit
// (hc_adjoint_tangent.cu); both directions in one launch, i-faces in blocks [0, nbi)
template <class R>
cudaError_t launch_adj_face_tangent(int flux, const AdjArgs<R>& a, int nbi, unsigned blocks, int threads,
                                    cudaStream_t s);
template <class R>
cudaError_t launch_adj_face_tangent_batch(int flux, const AdjBatchArgs<R>& b, unsigned blocks, int threads,
                                          cudaStream_t s);
inline bool flux_by_tangent(int flux) {
  return flux == FLUX_SLAU || flux == FLUX_SLAU_REF || flux == FLUX_AUSMPUP || flux == FLUX_ROE_WS ||
         flux == FLUX_ROE_FACE;
}

// the same for a scalar-law batch (the update is linear on the conserved set)
template <class R> __global__ void adj_update_lin_batch_kernel(const AdjUpdateBatch<R> u) {
  const int s = find_segment(u.seg, u.nseg, int(blockIdx.x));
  const BatchInst& in = u.inst[s];
  const long long c4 = 4 * in.cell;
  const double dt = u.cfl / fmax(DBL_MIN, u.rates[s]);
  const int c = (int(blockIdx.x) - u.seg[s]) * int(blockDim.x) + int(threadIdx.x);
  adj_update_lin_cell<R, 3>(in.ni * in.nj, u.vol + in.cell, u.qbar_out + c4, u.q0bar + c4, u.rbar[0] + c4,
                            u.rbar[1] + c4, u.rbar[2] + c4, u.rbar[3] + c4, u.alpha[0], u.alpha[1], u.alpha[2],
                            u.alpha[3], u.stage, R(u.beta * dt), c);
}

}  // namespace hc
