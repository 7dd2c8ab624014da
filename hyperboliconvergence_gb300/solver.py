"""Host-side mirror of the reference's integrate() interface over the C ABI.

The reference drives one run as (timestepping/rungeKutta.h:37-51)

    integrate(policy, UnsteadyTimeControls{nTimesteps, cfl}, rungeKutta,
              make_muscl_flux(Limiter{}, Flux{}), boundaryConditions, species,
              mesh, solutionField)

``Solver`` takes the same ingredients -- flux and limiter names, RK table,
CFL, species, mesh nodes, boundary-condition types with their reference
states, and the primitive solution field -- and runs them on the GPU through
libhcgb300.so.  Errors raise ``HCError`` (the C ABI returns status codes).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi
from ._capi import BC, DTMODE, FLUX, LIMITER, PRECISION, RK, Config, HCError, StepStats, check


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Mesh:
    """Structured 2D mesh: (ni+1) x (nj+1) nodes, node (i,j) at nodes[i, j] = (x, y)."""

    def __init__(self, nodes: np.ndarray):
        nodes = np.ascontiguousarray(nodes, dtype=np.float64)
        if nodes.ndim != 3 or nodes.shape[2] != 2:
            raise ValueError("nodes must have shape (ni+1, nj+1, 2)")
        self.nodes = nodes
        self.ni, self.nj = nodes.shape[0] - 1, nodes.shape[1] - 1

    @classmethod
    def cylinder(cls, nr: int, nth: int, rc: float, rb: float, stretch: float = 1.0) -> "Mesh":
        """O-grid around a cylinder (make_cylinder_mesh, mesh/generate/twoD.h:139-179)."""
        out = np.empty((nr + 1, nth + 1, 2))
        check(_capi.load().hc_mesh_cylinder_nodes(nr, nth, rc, rb, stretch, _dptr(out)))
        return cls(out)

    @classmethod
    def linspace(cls, nx: int, ny: int, lox: float, hix: float, loy: float, hiy: float) -> "Mesh":
        """Uniform Cartesian mesh (make_linspace_mesh, mesh/generate/twoD.h:15-40)."""
        out = np.empty((nx + 1, ny + 1, 2))
        check(_capi.load().hc_mesh_linspace_nodes(nx, ny, lox, hix, loy, hiy, _dptr(out)))
        return cls(out)

    def centres(self) -> np.ndarray:
        """Vertex centroids of the cells, shape (2, ni, nj)."""
        p = self.nodes
        c = 0.25 * p[:-1, :-1] + 0.25 * p[1:, :-1] + 0.25 * p[:-1, 1:] + 0.25 * p[1:, 1:]
        return np.moveaxis(c, 2, 0).copy()

    def nface(self, side: int) -> int:
        return self.nj if side < 2 else self.ni


class Mesh1D:
    """One-dimensional mesh (Mesh<1,Real>, mesh/generate/oneD.h:11-36): nc cells between
    increasing nodes x[0..nc].  A Solver on it runs the 1D Euler path with states of
    shape (3, nc), {u, rho, p}."""

    one_d = True

    def __init__(self, x: np.ndarray):
        x = np.ascontiguousarray(x, dtype=np.float64)
        if x.ndim != 1 or x.size < 4 or np.any(np.diff(x) <= 0):
            raise ValueError("nodes must be an increasing 1D array of at least 4 points")
        self.nodes = x
        self.ni, self.nj = x.size - 1, 1

    @classmethod
    def linspace(cls, nc: int, lo: float, hi: float) -> "Mesh1D":
        """Uniform 1D mesh (make_linspace_mesh, mesh/generate/oneD.h:11-36)."""
        return cls(lo + (hi - lo) / nc * np.arange(nc + 1))

    def centres(self) -> np.ndarray:
        return 0.5 * (self.nodes[:-1] + self.nodes[1:])

    def nface(self, side: int) -> int:
        return 1 if side < 2 else 0


class Solver:
    """One mesh, its boundary conditions and state, advanced by explicit RK on the GPU."""

    def __init__(self, mesh: Mesh, bc, ref=None, flux="roe", limiter="vanleer", rk="ssp34",
                 precision="fp64", dt="global", cfl=0.5, species=(1.4, 287.058, 1e-4), stream=None, law="euler",
                 low_mach=None, basis="primitive", tile=None, corrections=None):
        self.lib = _capi.load()
        self.mesh = mesh
        self.precision = precision
        self.flux, self.limiter, self.rk, self.dt, self.cfl = flux, limiter, rk, dt, float(cfl)
        self.species = tuple(float(x) for x in species)
        cfg = Config(FLUX[flux] if isinstance(flux, str) else int(flux),
                     LIMITER[limiter] if isinstance(limiter, str) else int(limiter),
                     RK[rk] if isinstance(rk, str) else int(rk),
                     PRECISION[precision], DTMODE[dt], float(cfl), _capi.LAW[law], _capi.BASIS[basis])
        self.basis = basis
        self.law = law
        self.one_d = getattr(mesh, "one_d", False)
        # variables: {u, v, q} (scalar), {u, v, rho, p} (Euler) or {u, rho, p} (1D Euler)
        self.nv = 3 if law == "scalar" or self.one_d else 4
        self._shape = (self.nv, mesh.ni) if self.one_d else (self.nv, mesh.ni, mesh.nj)
        h = C.c_void_p()
        check(self.lib.hc_context_create(C.byref(cfg), C.byref(h)))
        self.h = h
        if stream is not None:
            self.set_stream(stream)
        if self.one_d:
            check(self.lib.hc_mesh_upload_1d(self.h, mesh.ni, _dptr(mesh.nodes)))
        else:
            check(self.lib.hc_mesh_upload(self.h, mesh.ni, mesh.nj, _dptr(mesh.nodes)))
        check(self.lib.hc_set_species(self.h, *[float(s) for s in species]))
        if tile is not None:
            self.set_tile(tile)
        self.corrections = _capi.fix_mask(corrections)
        if self.corrections:
            check(self.lib.hc_set_corrections(self.h, self.corrections))
        self.tile = tile
        self.steps_done = 0
        self.last = None
        self.low_mach = None
        if low_mach is not None:
            self.set_low_mach(*low_mach)
        self.bc = list(bc)
        self.set_bcs(bc, ref)

    def set_tile(self, tile: str) -> None:
        """Cells per CTA tile of the 2D FP64/FP32 stage kernels: "8x32", "4x32" or "16x16"
        (the results do not depend on it)."""
        check(self.lib.hc_set_tile(self.h, _capi.TILE[tile]))
        self.tile = tile

    def set_corrections(self, corrections) -> None:
        """Corrections of the reference's defects (hc_set_corrections): None, "all", or names
        among "mach_split_p1" and "farfield_transverse"."""
        self.corrections = _capi.fix_mask(corrections)
        check(self.lib.hc_set_corrections(self.h, self.corrections))

    def set_staged_loads(self, on: bool = True) -> None:
        """The FP32 stage's tile loads staged by TMA tensor copies (the default) or plain
        per-thread loads (hc_set_staged_loads); bit-identical results."""
        check(self.lib.hc_set_staged_loads(self.h, 1 if on else 0))

    def inject_stalled_copy(self, on: bool = True) -> None:
        """Test hook of the failure detection (hc_inject_stalled_copy): the TMA-staged FP32
        stage kernel's copy barrier waits for bytes that never come, its bounded wait runs out
        and the step raises HC_ERR_TIMEOUT with the context still usable."""
        check(self.lib.hc_inject_stalled_copy(self.h, 1 if on else 0))

    def set_adjoint_tapes(self, ntapes: int = -1) -> None:
        """Stage tapes of the adjoint's checkpointing (hc_set_adjoint_tapes): -1 one per
        snapshot and one more (no step's stages recomputed), 0 none (every reversed step
        replays its stages from its start state), k at most k."""
        check(self.lib.hc_set_adjoint_tapes(self.h, int(ntapes)))

    def set_low_mach(self, velocity="convective", pressure="convective", lref=1.0,
                     dt=np.finfo(np.float64).max) -> None:
        """AUSM+up's low-Mach scalings, AusmPlusUP<velocity, pressure> with "convective",
        "acoustic" or "adaptive", and the species lref and dt of the adaptive ratio
        lref/(as dt) (conservationLaws/euler/fluxes/ausmPlusUP.ipp:61-87)."""
        vs = _capi.SCALING[velocity] if isinstance(velocity, str) else int(velocity)
        ps = _capi.SCALING[pressure] if isinstance(pressure, str) else int(pressure)
        check(self.lib.hc_set_low_mach(self.h, vs, ps, float(lref), float(dt)))
        self.low_mach = (velocity, pressure, float(lref), float(dt))

    def set_bcs(self, bc, ref=None) -> None:
        """Boundary types per side and their reference (ghost) states, 4 planes per side."""
        mesh = self.mesh
        bc = list(bc) + ["periodic"] * (4 - len(bc))  # a 1D mesh has sides 0 and 1 only
        ref = None if ref is None else list(ref) + [None] * (4 - len(ref))
        bct = (C.c_int * 4)(*[BC[b] if isinstance(b, str) else int(b) for b in bc])
        self._refs = []
        ptrs = (C.POINTER(C.c_double) * 4)()
        for s in range(4):
            r = None if ref is None else ref[s]
            if r is None:
                ptrs[s] = C.POINTER(C.c_double)()
            else:
                arr = np.ascontiguousarray(np.broadcast_to(
                    np.asarray(r, dtype=np.float64).reshape(self.nv, -1), (self.nv, mesh.nface(s))))
                self._refs.append(arr)
                ptrs[s] = _dptr(arr)
        check(self.lib.hc_set_bcs(self.h, bct, ptrs))
        self.bc = list(bc)
        self.ref = [None if ref is None or ref[s] is None or mesh.nface(s) == 0 else
                    np.broadcast_to(np.asarray(ref[s], dtype=np.float64).reshape(self.nv, -1),
                                    (self.nv, mesh.nface(s))).copy()
                    for s in range(4)]

    # -- discrete adjoint -----------------------------------------------------
    def _objective(self, kind, scale=1.0, direction=(1.0, 0.0), target=None, weight=(1.0, 1.0, 1.0, 1.0)):
        from ._capi import OBJECTIVE, Objective
        o = Objective()
        o.kind = OBJECTIVE[kind]
        o.scale = float(scale)
        o.dir[0], o.dir[1] = float(direction[0]), float(direction[1])
        self._target = None
        if target is not None:
            self._target = np.ascontiguousarray(target, dtype=np.float64)
            o.target = _dptr(self._target)
        for k in range(4):
            o.weight[k] = float(weight[k])
        return o

    def objective(self, nsteps, kind="drag", rates=None, **kw):
        """J over nsteps from the current state; returns (J, per-step max rates)."""
        o = self._objective(kind, **kw)
        J = C.c_double()
        rout = np.empty(int(nsteps))
        rin = None if rates is None else np.ascontiguousarray(rates, dtype=np.float64)
        check(self.lib.hc_objective_forward(self.h, int(nsteps), C.byref(o),
                                            _dptr(rin) if rin is not None else None, _dptr(rout), C.byref(J)))
        return J.value, rout

    def gradient(self, nsteps, snapshots=20, kind="drag", rates=None, **kw):
        """J and its gradient with respect to the current state and the fixed-ghost
        reference states; returns (J, q0_bar, [ref_bar per side], rates, stats).  Euler:
        drag or L2 objective, 4 planes; scalar advection: L2 objective on {u, v, q}, 3 planes
        (weight[3] unused)."""
        from ._capi import AdjointStats
        o = self._objective(kind, **kw)
        m = self.mesh
        nv = self.nv
        q0b = np.empty((nv, m.ni, m.nj))
        rb = np.empty(sum(nv * m.nface(s) for s in range(4)))
        rout = np.empty(int(nsteps))
        st = AdjointStats()
        rin = None if rates is None else np.ascontiguousarray(rates, dtype=np.float64)
        check(self.lib.hc_adjoint_gradient(self.h, int(nsteps), int(snapshots), C.byref(o),
                                           _dptr(rin) if rin is not None else None, _dptr(q0b), _dptr(rb),
                                           _dptr(rout), C.byref(st)))
        refb, off = [], 0
        for s in range(4):
            nf = m.nface(s)
            refb.append(rb[off:off + nv * nf].reshape(nv, nf).copy())
            off += nv * nf
        return st.J, q0b, refb, rout, st

    def record(self, nsteps, snapshots=20, kind="drag", rates=None, **kw):
        """The forward half of `gradient` (hc_adjoint_record): (J, rates) of nsteps steps from
        the current state; the checkpoints stay in the context for `reverse`."""
        o = self._objective(kind, **kw)
        self._tape_objective = o
        J = C.c_double()
        rout = np.empty(int(nsteps))
        rin = None if rates is None else np.ascontiguousarray(rates, dtype=np.float64)
        check(self.lib.hc_adjoint_record(self.h, int(nsteps), int(snapshots), C.byref(o),
                                         _dptr(rin) if rin is not None else None, _dptr(rout), C.byref(J)))
        return J.value, rout

    def reverse(self, q0_bar=None, ref_bar=None):
        """The reverse half (hc_adjoint_reverse) into float64 CUDA tensors: q0_bar of the state's
        shape, ref_bar of sum over sides of nv * nface values (either may be None)."""
        from ._capi import AdjointStats
        st = AdjointStats()

        def ptr(t):
            return None if t is None else C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double))
        check(self.lib.hc_adjoint_reverse(self.h, ptr(q0_bar), ptr(ref_bar), 1, C.byref(st)))
        self._tape_objective = None
        return st

    def upload_device(self, prim) -> None:
        """The state from a CUDA tensor of the context's precision (hc_state_upload_device)."""
        check(self.lib.hc_state_upload_device(self.h, C.c_void_p(prim.contiguous().data_ptr())))

    def close(self):
        if getattr(self, "h", None):
            self.lib.hc_context_destroy(self.h)
            self.h = None

    __del__ = close

    def set_stream(self, stream) -> None:
        """Run on this cudaStream_t handle (0 = the legacy default stream)."""
        check(self.lib.hc_set_stream(self.h, C.c_void_p(int(stream) if stream else None)))

    def get_stream(self) -> int:
        out = C.c_void_p()
        check(self.lib.hc_get_stream(self.h, C.byref(out)))
        return out.value or 0

    # -- solution field ------------------------------------------------------
    def set_state(self, prim: np.ndarray) -> None:
        """Upload the state in the solver's basis: primitive {u, v, rho, p} (Euler, the
        default), conserved {rho u, rho v, rho, rho E} (Euler, basis="conserved"), or {u, v, q}
        (scalar advection), shape (nv, ni, nj)."""
        a = np.ascontiguousarray(prim, dtype=np.float64)
        if a.shape != self._shape:
            raise ValueError(f"state must have shape {self._shape}")
        check(self.lib.hc_state_upload(self.h, _dptr(a)))

    def get_state(self, out: np.ndarray | None = None) -> np.ndarray:
        """Download the state (into ``out`` when given: C-contiguous float64)."""
        shape = self._shape
        if out is None:
            out = np.empty(shape)
        elif out.shape != shape or out.dtype != np.float64 or \
                not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a C-contiguous float64 array of the state's shape")
        check(self.lib.hc_state_download(self.h, _dptr(out)))
        return out

    def set_state_device(self, ptr: int) -> None:
        check(self.lib.hc_state_upload_device(self.h, C.c_void_p(ptr)))

    def get_state_device(self, ptr: int) -> None:
        check(self.lib.hc_state_download_device(self.h, C.c_void_p(ptr)))

    # -- path ----------------------------------------------------------------
    def residual(self) -> np.ndarray:
        """Flux sums (nv conserved planes) and spectral-radius sum of the current state."""
        out = np.empty((self.nv + 1,) + self._shape[1:])
        check(self.lib.hc_residual(self.h, _dptr(out)))
        return out

    def dual_time(self, outer_steps: int, dt: float = 0.0, cfl_outer: float = 0.5, scheme: str = "bdf2",
                  inner_max: int = 50, inner_drop: float = 0.0, check_every: int = 5):
        """Dual-time stepping (include/hc.h, hc_dual_time_run): outer_steps physical steps of
        the multistep scheme ("bdf1", "bdf2", "trapezium"), each solved by at most inner_max
        pseudo-time RK steps (the solver's rk, cfl and dt mode) until the density dual-time
        residual fell by inner_drop; dt <= 0 takes cfl_outer / max(lambda/V) of the current
        state.  Returns the stats (dt, t, inner_steps, last_inner, res0_last, res_last)."""
        from ._capi import MULTISTEP, DualTimeControls, DualTimeStats
        ctl = DualTimeControls(int(outer_steps), float(dt), float(cfl_outer), MULTISTEP[scheme], int(inner_max),
                               float(inner_drop), int(check_every))
        st = DualTimeStats()
        check(self.lib.hc_dual_time_run(self.h, C.byref(ctl), C.byref(st)))
        return st

    def face_signatures(self, with_args: bool = False):
        """Branch signatures of one residual evaluation of the current state (include/hc.h,
        hc_face_signatures): uint64 arrays of shape (ni+1, nj) for the i-faces and (ni, nj+1)
        for the j-faces; with_args also returns the limiter arguments, arrays (ni+1, nj, 8, 2)
        and (ni, nj+1, 8, 2) of (a, b) per limiter call."""
        m = self.mesh
        si = np.zeros((m.ni + 1, m.nj), dtype=np.uint64)
        sj = np.zeros((m.ni, m.nj + 1), dtype=np.uint64)
        ai = np.zeros((m.ni + 1, m.nj, 8, 2)) if with_args else None
        aj = np.zeros((m.ni, m.nj + 1, 8, 2)) if with_args else None
        u64 = C.POINTER(C.c_uint64)
        check(self.lib.hc_face_signatures(self.h, si.ctypes.data_as(u64), sj.ctypes.data_as(u64),
                                          None if ai is None else ai.ctypes.data,
                                          None if aj is None else aj.ctypes.data))
        return ((si, sj), (ai, aj)) if with_args else (si, sj)

    def step(self, n: int = 1) -> StepStats:
        st = StepStats()
        check(self.lib.hc_step(self.h, int(n), C.byref(st)))
        self.steps_done += int(n)
        self.last = st
        return st

    def step_host(self, state_in: np.ndarray, state_out: np.ndarray, n: int = 1) -> StepStats:
        """n steps of a host state (hc_step_host): state_in uploaded, stepped, the result
        written to state_out (C-contiguous float64 arrays of the state's shape; page-locked
        memory lets the copies run asynchronously), one synchronisation."""
        for a in (state_in, state_out):
            if a.shape != self._shape or a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
                raise ValueError(f"states must be C-contiguous float64 arrays of shape {self._shape}")
        st = StepStats()
        check(self.lib.hc_step_host(self.h, int(n), _dptr(state_in), _dptr(state_out), C.byref(st)))
        self.steps_done += int(n)
        self.last = st
        return st

    def wall_force(self, direction=(1.0, 0.0)) -> float:
        """Pressure force on the wall sides along `direction` (hc_wall_force)."""
        d = np.ascontiguousarray(direction, dtype=np.float64)
        out = np.zeros(1)
        check(self.lib.hc_wall_force(self.h, _dptr(d), _dptr(out)))
        return float(out[0])

    def set_time(self, t: float, steps_done: int | None = None) -> None:
        """The accumulated time (and, optionally, the count of steps taken) a resumed run
        continues from (hc_set_time)."""
        check(self.lib.hc_set_time(self.h, float(t)))
        if steps_done is not None:
            self.steps_done = int(steps_done)

    def steady(self, max_steps: int, residual_drop: float = 1e-10, check_every: int = 100, smoothing=None):
        """Run to a steady state (SteadyTimeControls, controls.h:31-48): steps until the
        stage-0 density-residual L2 norm drops by residual_drop or max_steps; returns
        (SteadyStats, residual-norm history read every check_every steps).  smoothing
        (1D meshes): the implicit residual smoothing's alpha (>= 1) applied to every stage's
        residual (use_residual_smoothing with smoothing_factor = alpha)."""
        from ._capi import SteadyControls, SteadyStats
        ctl = SteadyControls(int(max_steps), float(residual_drop), int(check_every), 0 if smoothing is None else 1,
                             0.0 if smoothing is None else float(smoothing))
        hist = np.empty(int(max_steps) // int(check_every) + 2)
        st = SteadyStats()
        check(self.lib.hc_steady_run(self.h, C.byref(ctl), _dptr(hist), hist.size, C.byref(st)))
        self.steps_done += int(st.steps)
        return st, hist[:st.history_len].copy()

    def smooth_1d(self, r, alpha: float, kind: str = "implicit", ends: str = "a",
                  in_place: bool = False) -> np.ndarray:
        """Residual smoothing of the legacy 1D path (hc_smooth_1d) of each row of r (shape
        (nplanes, n) or (n,)) on this context's device and stream: kind "implicit" or
        "explicit", ends "p" (periodic), "a" (one-neighbour) or "n" (unscaled).  in_place
        passes the same device buffer as input and output."""
        import torch
        a = np.ascontiguousarray(r, dtype=np.float64)
        a2 = a.reshape(-1, a.shape[-1])
        src = torch.from_numpy(a2).cuda()
        dst = src if in_place else torch.empty_like(src)
        torch.cuda.synchronize()
        check(self.lib.hc_smooth_1d(self.h, {"implicit": 0, "explicit": 1}[kind], C.c_void_p(src.data_ptr()),
                                    C.c_void_p(dst.data_ptr()), a2.shape[1], a2.shape[0], float(alpha), ord(ends)))
        torch.cuda.synchronize()
        return dst.cpu().numpy().reshape(a.shape)

    def step_async(self, n: int = 1) -> None:
        check(self.lib.hc_step_async(self.h, int(n)))
        self.steps_done += int(n)

    def sync(self) -> StepStats:
        st = StepStats()
        check(self.lib.hc_sync(self.h, C.byref(st)))
        return st


# ratios b/a (b = c a, with a > 0) at which each limiter changes piece; the sign of a is
# one more breakpoint (limit_piece in csrc/hc_physics.cuh)
LIMITER_BREAKS = {"vanalbada": (0.0,), "vanleer": (0.0,), "minmod": (0.0, 1.0), "superbee": (0.0, 0.5, 1.0, 2.0),
                  "mc": (0.0, 1.0 / 3.0, 3.0), "cada3": (-2.0, -2.0 / 7.0, 0.0, 0.4, 2.5)}


def branch_flips(sig_a, sig_b, cell_mask: bool = False, args=None, limiter=None, roundoff=1e-9) -> dict:
    """Where two evaluations of the same state took different branches: the faces whose
    signatures differ (limiter pieces, flux branches, far-field paths), and the cells with
    such a face.  sig_a, sig_b: (i-face, j-face) signature arrays from face_signatures;
    cell_mask adds the (ni, nj) boolean mask of those cells.  With args (the reference
    evaluation's limiter arguments from face_signatures(with_args=True)) and the limiter's
    name, limiter flips whose arguments lie within `roundoff` of the variable's argument
    scale from a breakpoint -- an argument zero in exact arithmetic, computed as round-off
    -- are told apart: "faces_above_roundoff" counts the faces with another flip."""
    (ia, ja), (ib, jb) = sig_a, sig_b
    fi, fj = ia != ib, ja != jb
    cells = fi[:-1, :] | fi[1:, :] | fj[:, :-1] | fj[:, 1:]
    lim_mask = np.uint64(0xFFFFFFFF)
    out = {"faces": int(fi.sum() + fj.sum()), "faces_total": int(fi.size + fj.size),
           "limiter_faces": int((((ia ^ ib) & lim_mask) != 0).sum() + (((ja ^ jb) & lim_mask) != 0).sum()),
           "cells": int(cells.sum()), "cells_total": int(cells.size)}
    if args is not None and limiter is not None:
        a = np.concatenate([args[0].reshape(-1, 8, 2), args[1].reshape(-1, 8, 2)])
        x = np.concatenate([(ia ^ ib).ravel(), (ja ^ jb).ravel()])
        diff = np.stack([((x >> np.uint64(4 * k)) & np.uint64(15)) != 0 for k in range(8)], axis=1)
        slot_scale = np.abs(a).max(axis=(0, 2))
        var_scale = np.tile(np.maximum(slot_scale[:4], slot_scale[4:]), 2)  # per variable, both sides
        lo, hi = a[..., 0], a[..., 1]
        u = np.where(lo > 0, lo, -lo)
        v = np.where(lo > 0, hi, -hi)
        dist = np.abs(lo)
        for c in LIMITER_BREAKS.get(limiter, ()):
            dist = np.minimum(dist, np.abs(v - c * u))
        noise = dist <= roundoff * var_scale[None, :]
        above = (diff & ~noise).any(axis=1) | ((x >> np.uint64(32)) != 0)
        out["faces_above_roundoff"] = int(above.sum())
    if cell_mask:
        out["cell_mask"] = cells
    return out


__all__ = ["Mesh", "Mesh1D", "Solver", "HCError", "branch_flips"]
