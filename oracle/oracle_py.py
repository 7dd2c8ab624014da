"""ctypes wrapper over the CPU oracle (oracle/_build/libhcoracle*.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py``, always as the checker or the
timed CPU baseline, never as the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_SO = os.path.join(HERE, "_ref", "libhcref.so")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")

# enum values shared with oracle/hc_oracle.hpp and include/hc.h
FLUX = {"roe": 0, "slau": 1, "slau_ref": 2, "ausmpup": 3, "rusanov": 4, "central": 5, "roe_ws": 6,
        "roe_face": 7}
SCALING = {"convective": 0, "acoustic": 1, "adaptive": 2}
BASIS = {"primitive": 0, "conserved": 1}
LIMITER = {"nolimit1": 0, "nolimit2": 1, "nolimit3": 2, "vanalbada": 3, "minmod": 4,
           "superbee": 5, "mc": 6, "vanleer": 7, "vanleer_ref": 8, "cada3": 9}
BC = {"periodic": 0, "fixed": 1, "riemann": 2, "entropy": 3, "wall": 4}
RK = {"ssp11": 0, "ssp22": 1, "ssp33": 2, "ssp34": 3}
DT = {"global": 0, "local": 1}
# corrections of the reference's defects (FIX_* in hc_oracle.hpp, hc_fix in include/hc.h)
FIX = {"mach_split_p1": 1, "farfield_transverse": 2}


def fix_mask(corrections) -> int:
    if corrections is None:
        return 0
    if isinstance(corrections, int):
        return corrections
    if isinstance(corrections, str):
        return sum(FIX.values()) if corrections == "all" else FIX[corrections]
    return sum(FIX[c] for c in set(corrections))


def build(quiet: bool = True) -> None:
    """Compile the oracle with make (parity and timing variants)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)


def _declare(lib: C.CDLL, prefix: str) -> None:
    d, i, v = C.c_double, C.c_int, C.c_void_p
    sigs = {
        "flux": (None, [i, _dp, _dp, _dp, _dp, _dp]),
        "exact_flux": (None, [_dp, _dp, _dp, _dp]),
        "limit": (d, [i, d, d]),
        "surface": (None, [_dp, _dp, _dp]),
        "volume": (None, [_dp, _dp]),
        "prim2state": (None, [_dp, _dp, _dp]),
        "prim2cons": (None, [_dp, _dp, _dp]),
        "cons2prim": (None, [_dp, _dp, _dp]),
        "bc_update": (None, [i, _dp, _dp, _dp, _dp, _dp]),
        "wall_flux": (None, [_dp, _dp, _dp, _dp, _dp]),
        "delta": (None, [i, _dp, _dp, _dp, _dp]),
        "rk_table": (None, [i, _dp]),
        "linspace_nodes": (None, [i, i, d, d, d, d, _dp]),
        "ausmpup_scaled": (None, [i, i, _dp, _dp, _dp, _dp, _dp]),
    }
    for name, (res, args) in sigs.items():
        f = getattr(lib, prefix + name)
        f.restype = res
        f.argtypes = args


class Pointwise:
    """Pointwise functions of either the oracle (prefix hco_) or the reference probe (ref_)."""

    def __init__(self, lib: C.CDLL, prefix: str):
        self.lib, self.p = lib, prefix
        _declare(lib, prefix)
        if prefix == "hco_":
            lib.hco_cylinder_nodes.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, _dp]
        else:
            lib.ref_cylinder_nodes.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, _dp]

    def fn(self, name):
        return getattr(self.lib, self.p + name)

    def flux(self, kind, species, face, ql, qr):
        out = np.empty(5)
        self.fn("flux")(kind, species, face, ql, qr, out)
        return out

    def flux_fixed(self, kind, corrections, species, face, ql, qr):
        """The flux with corrections of the reference's defects (oracle only)."""
        f = self.lib.hco_flux_fixed
        f.argtypes = [C.c_int, C.c_uint, _dp, _dp, _dp, _dp, _dp]
        out = np.empty(5)
        f(int(kind), fix_mask(corrections), species, face, ql, qr, out)
        return out

    def bc_update_fixed(self, kind, corrections, species, face, qi, qf):
        f = self.lib.hco_bc_update_fixed
        f.argtypes = [C.c_int, C.c_uint, _dp, _dp, _dp, _dp, _dp]
        out = np.empty(4)
        f(int(kind), fix_mask(corrections), species, face, qi, qf, out)
        return out

    def ausmpup_scaled(self, vscale, pscale, species5, face, ql, qr):
        """AUSM+up with low-Mach scalings (SCALING); species5 = (gamma, R, minf, lref, dt)."""
        out = np.empty(5)
        self.fn("ausmpup_scaled")(int(vscale), int(pscale), np.asarray(species5, dtype=np.float64),
                                  face, ql, qr, out)
        return out

    # conserved-basis fields (BASIS "conserved"): the oracle's hco_*_basis functions or
    # the reference probe's ref_*_cons functions
    def _basis_fn(self, name):
        i, dpp = C.c_int, _dp
        if self.p == "hco_":
            f = self.fn(name + "_basis")
            f.argtypes = {"flux": [i, i, dpp, dpp, dpp, dpp, dpp], "bc_update": [i, i, dpp, dpp, dpp, dpp, dpp],
                          "wall_flux": [i, dpp, dpp, dpp, dpp, dpp]}[name]
        else:
            f = self.fn(name + "_cons")
            f.argtypes = {"flux": [i, dpp, dpp, dpp, dpp, dpp], "bc_update": [i, dpp, dpp, dpp, dpp, dpp],
                          "wall_flux": [dpp, dpp, dpp, dpp, dpp]}[name]
        f.restype = None
        return f

    def flux_cons(self, kind, species, face, ql, qr):
        out = np.empty(5)
        f = self._basis_fn("flux")
        if self.p == "hco_":
            f(kind, 1, species, face, ql, qr, out)
        else:
            f(kind, species, face, ql, qr, out)
        return out

    def bc_update_cons(self, kind, species, face, qi, qf):
        out = np.empty(4)
        f = self._basis_fn("bc_update")
        if self.p == "hco_":
            f(kind, 1, species, face, qi, qf, out)
        else:
            f(kind, species, face, qi, qf, out)
        return out

    def wall_flux_cons(self, species, face, qi, dq):
        out = np.empty(5)
        f = self._basis_fn("wall_flux")
        if self.p == "hco_":
            f(1, species, face, qi, dq, out)
        else:
            f(species, face, qi, dq, out)
        return out

    def exact_flux(self, species, normal, q):
        out = np.empty(5)
        self.fn("exact_flux")(species, normal, q, out)
        return out

    def limit(self, kind, a, b):
        return self.fn("limit")(kind, float(a), float(b))

    def surface(self, p0, p1):
        out = np.empty(7)
        self.fn("surface")(p0, p1, out)
        return out

    def volume(self, p):
        out = np.empty(3)
        self.fn("volume")(p, out)
        return out

    def prim2state(self, species, q):
        out = np.empty(8)
        self.fn("prim2state")(species, q, out)
        return out

    def prim2cons(self, species, q):
        out = np.empty(4)
        self.fn("prim2cons")(species, q, out)
        return out

    def cons2prim(self, species, qc):
        out = np.empty(4)
        self.fn("cons2prim")(species, qc, out)
        return out

    def bc_update(self, kind, species, face, qi, qf):
        out = np.empty(4)
        self.fn("bc_update")(kind, species, face, qi, qf, out)
        return out

    def wall_flux(self, species, face, qi, dq):
        out = np.empty(5)
        self.fn("wall_flux")(species, face, qi, dq, out)
        return out

    def delta(self, kind, species, q, din):
        out = np.empty(4)
        self.fn("delta")(kind, species, q, din, out)
        return out

    def rk_table(self, kind):
        out = np.empty(22)
        self.fn("rk_table")(kind, out)
        return out

    def cylinder_nodes(self, nr, nth, rc, rb, stretch=1.0):
        out = np.empty((nr + 1) * (nth + 1) * 2)
        if self.p == "hco_":
            self.fn("cylinder_nodes")(nr, nth, rc, rb, stretch, out)
        else:
            self.fn("cylinder_nodes")(nr, nth, rc, rb, out)
        return out

    def linspace_nodes(self, nx, ny, lox, hix, loy, hiy):
        out = np.empty((nx + 1) * (ny + 1) * 2)
        self.fn("linspace_nodes")(nx, ny, lox, hix, loy, hiy, out)
        return out


_libs: dict = {}


def load(fast: bool = False) -> C.CDLL:
    """Load the oracle library (building it if missing)."""
    name = "libhcoracle_fast.so" if fast else "libhcoracle.so"
    if name in _libs:
        return _libs[name]
    path = os.path.join(BUILD, name)
    if not os.path.exists(path):
        build()
    lib = C.CDLL(path)
    v, i, d = C.c_void_p, C.c_int, C.c_double
    lib.hco_create.restype = v
    lib.hco_create.argtypes = [i, i, _dp, _ip, i, i, i, i, d, _dp]
    lib.hco_destroy.argtypes = [v]
    lib.hco_set_ghost_ref.argtypes = [v, i, _dp]
    lib.hco_get_ghost.argtypes = [v, i, _dp]
    lib.hco_set_state.argtypes = [v, _dp]
    lib.hco_get_state.argtypes = [v, _dp]
    lib.hco_residual.argtypes = [v, _dp]
    lib.hco_step.argtypes = [v, i, _dp]
    lib.hco_cells.argtypes = [v, _dp]
    lib.hco_set_threads.argtypes = [i]
    lib.hco_get_threads.restype = i
    _libs[name] = lib
    return lib


def pointwise(fast: bool = False) -> Pointwise:
    return Pointwise(load(fast), "hco_")


def reference_pointwise() -> Pointwise | None:
    """The reference's own pointwise code, when oracle/_ref was built here."""
    if not os.path.exists(REF_SO):
        return None
    return Pointwise(C.CDLL(REF_SO), "ref_")


class OracleSolver:
    """CPU restatement of the reference integrate() over one 2D structured mesh."""

    def __init__(self, ni, nj, nodes, bc, flux="roe", limiter="vanleer", rk="ssp34", dt="global",
                 cfl=0.5, species=(1.4, 287.058, 1e-4), ghost_ref=None, fast=False, low_mach=None,
                 basis="primitive", corrections=None):
        self.lib = load(fast)
        self.ni, self.nj = ni, nj
        bcv = np.array([BC[b] if isinstance(b, str) else int(b) for b in bc], dtype=np.int32)
        self.h = self.lib.hco_create(ni, nj, np.ascontiguousarray(nodes, dtype=np.float64), bcv,
                                     FLUX[flux] if isinstance(flux, str) else flux,
                                     LIMITER[limiter] if isinstance(limiter, str) else limiter,
                                     RK[rk] if isinstance(rk, str) else rk,
                                     DT[dt] if isinstance(dt, str) else dt,
                                     float(cfl), np.asarray(species, dtype=np.float64))
        self.lib.hco_set_basis.argtypes = [C.c_void_p, C.c_int]
        self.lib.hco_set_basis(self.h, BASIS[basis] if isinstance(basis, str) else int(basis))
        if corrections:
            self.lib.hco_set_corrections.argtypes = [C.c_void_p, C.c_uint]
            self.lib.hco_set_corrections(self.h, fix_mask(corrections))
        if low_mach is not None:
            # (velocity scaling, pressure scaling, lref, species dt) of AUSM+up
            vs, ps, lref, sdt = low_mach
            self.lib.hco_set_low_mach.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double]
            self.lib.hco_set_low_mach(self.h, SCALING.get(vs, vs) if isinstance(vs, str) else int(vs),
                                      SCALING.get(ps, ps) if isinstance(ps, str) else int(ps),
                                      float(lref), float(sdt))
        if ghost_ref is not None:
            for side in range(4):
                if ghost_ref[side] is not None:
                    nf = nj if side < 2 else ni
                    arr = np.ascontiguousarray(np.broadcast_to(
                        np.asarray(ghost_ref[side], dtype=np.float64).reshape(4, -1), (4, nf)))
                    self.lib.hco_set_ghost_ref(self.h, side, arr)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.hco_destroy(self.h)
            self.h = None

    def set_state(self, prim_soa):
        self.lib.hco_set_state(self.h, np.ascontiguousarray(prim_soa, dtype=np.float64))

    def get_state(self):
        out = np.empty((4, self.ni, self.nj))
        self.lib.hco_get_state(self.h, out)
        return out

    def residual(self):
        out = np.empty((5, self.ni, self.nj))
        self.lib.hco_residual(self.h, out)
        return out

    def step(self, n=1):
        out = np.empty(2)
        self.lib.hco_step(self.h, int(n), out)
        return float(out[0]), float(out[1])

    def dual_time(self, outer, dt=0.0, cfl_outer=0.5, scheme="bdf2", inner=10):
        """Dual-time stepping (the CUDA path's hc_dual_time_run with a fixed inner count);
        returns the physical timestep."""
        self.lib.hco_dual_time.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int]
        self.lib.hco_dual_time.restype = C.c_double
        k = {"bdf1": 0, "bdf2": 1, "trapezium": 2}[scheme] if isinstance(scheme, str) else int(scheme)
        return self.lib.hco_dual_time(self.h, int(outer), float(dt), float(cfl_outer), k, int(inner))

    def face_signatures(self, with_args=False):
        """Branch signatures of one residual evaluation (the CUDA path's codes); with_args
        also returns the limiter arguments, arrays (ni+1, nj, 8, 2) and (ni, nj+1, 8, 2) of
        (a, b) per limiter call (left side's four variables, then the right side's)."""
        si = np.zeros((self.ni + 1, self.nj), dtype=np.uint64)
        sj = np.zeros((self.ni, self.nj + 1), dtype=np.uint64)
        ai = np.zeros((self.ni + 1, self.nj, 8, 2)) if with_args else None
        aj = np.zeros((self.ni, self.nj + 1, 8, 2)) if with_args else None
        u64 = C.POINTER(C.c_uint64)
        self.lib.hco_face_signatures.argtypes = [C.c_void_p, u64, u64, C.c_void_p, C.c_void_p]
        self.lib.hco_face_signatures(self.h, si.ctypes.data_as(u64), sj.ctypes.data_as(u64),
                                     None if ai is None else ai.ctypes.data, None if aj is None else aj.ctypes.data)
        return ((si, sj), (ai, aj)) if with_args else (si, sj)

    def cells(self):
        out = np.empty((3, self.ni, self.nj))
        self.lib.hco_cells(self.h, out)
        return out


class OracleSolver1D:
    """CPU restatement of the reference's one-dimensional Euler path (hc_oracle_1d.hpp);
    state {u, rho, p} as 3 planes of nc values; ref: (left, right) reference states."""

    def __init__(self, nodes, bc, flux="roe", limiter="vanleer", rk="ssp34", dt="global", cfl=0.5,
                 species=(1.4, 287.058, 1e-4), ref=None, fast=False):
        self.lib = load(fast)
        lib = self.lib
        lib.hco1_create.restype = C.c_void_p
        lib.hco1_create.argtypes = [C.c_int, _dp, _ip, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, _dp, C.c_void_p]
        lib.hco1_destroy.argtypes = [C.c_void_p]
        lib.hco1_set_state.argtypes = [C.c_void_p, _dp]
        lib.hco1_get_state.argtypes = [C.c_void_p, _dp]
        lib.hco1_residual.argtypes = [C.c_void_p, _dp]
        lib.hco1_step.argtypes = [C.c_void_p, C.c_int, _dp]
        x = np.ascontiguousarray(nodes, dtype=np.float64)
        self.nc = x.size - 1
        bcv = np.array([BC[b] if isinstance(b, str) else int(b) for b in bc], dtype=np.int32)
        refa = None if ref is None else np.ascontiguousarray(
            [np.zeros(3) if r is None else np.asarray(r, dtype=np.float64) for r in ref], dtype=np.float64)
        self._ref = refa
        self.h = lib.hco1_create(self.nc, x, bcv, FLUX[flux] if isinstance(flux, str) else flux,
                                 LIMITER[limiter] if isinstance(limiter, str) else limiter,
                                 RK[rk] if isinstance(rk, str) else rk, DT[dt] if isinstance(dt, str) else dt,
                                 float(cfl), np.asarray(species, dtype=np.float64),
                                 None if refa is None else refa.ctypes.data)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.hco1_destroy(self.h)
            self.h = None

    def set_state(self, prim):
        self.lib.hco1_set_state(self.h, np.ascontiguousarray(prim, dtype=np.float64))

    def get_state(self):
        out = np.empty((3, self.nc))
        self.lib.hco1_get_state(self.h, out)
        return out

    def residual(self):
        out = np.empty((4, self.nc))
        self.lib.hco1_residual(self.h, out)
        return out

    def step(self, n=1):
        out = np.empty(2)
        self.lib.hco1_step(self.h, int(n), out)
        return float(out[0]), float(out[1])


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _sides(arrs, ni, nj, nv=4):
    """Per-side nv-plane arrays (None for unused sides) as a C array of pointers."""
    keep, ptrs = [], (C.c_void_p * 4)()
    for side in range(4):
        a = None if arrs is None else arrs[side]
        if a is None:
            ptrs[side] = None
            continue
        nf = nj if side < 2 else ni
        a = np.ascontiguousarray(np.broadcast_to(np.asarray(a, dtype=np.float64).reshape(nv, -1), (nv, nf)))
        keep.append(a)
        ptrs[side] = a.ctypes.data
    return ptrs, keep


def objective(mesh_nodes, ni, nj, bc, q0, nsteps, kind="drag", flux="roe", limiter="vanalbada", rk="ssp34",
              cfl=0.5, species=(1.4, 287.058, 0.4), ref=None, scale=1.0, direction=(1.0, 0.0), target=None,
              weight=(1.0, 1.0, 1.0, 1.0), dq0=None, dref=None, freeze_dt=True):
    """J of an RK run of the oracle with the global timestep (drag: scale/N times the
    wall force along `direction` summed over steps 1..N; l2: weighted squared distance
    of the final primitive state from `target`).  With a direction (dq0 and/or dref)
    also returns the exact derivative of J along it (forward-mode dual numbers
    through the same oracle code), with the timesteps frozen at their values (the
    discrete adjoint's convention) unless freeze_dt is False.  Returns (J, dJ or None)."""
    lib = load(False)
    if not getattr(lib, "_obj_declared", False):
        v, i, d = C.c_void_p, C.c_int, C.c_double
        lib.hco_objective.argtypes = [i, i, v, v, i, i, i, d, v, v, v, i, i, d, d, d, v, v, v]
        lib.hco_objective_jvp.argtypes = [i, i, v, v, i, i, i, d, v, v, v, v, v, i, i, d, d, d, v, v, i, v]
        lib._obj_declared = True
    nodes = np.ascontiguousarray(mesh_nodes, dtype=np.float64)
    bcv = np.array([BC[b] if isinstance(b, str) else int(b) for b in bc], dtype=np.int32)
    sp = np.asarray(species, dtype=np.float64)
    q = np.ascontiguousarray(q0, dtype=np.float64)
    refp, keep_r = _sides(ref, ni, nj)
    tgt = None if target is None else np.ascontiguousarray(target, dtype=np.float64)
    w = np.asarray(weight, dtype=np.float64)
    out = np.zeros(2)
    fl = FLUX[flux] if isinstance(flux, str) else flux
    lm = LIMITER[limiter] if isinstance(limiter, str) else limiter
    r = RK[rk] if isinstance(rk, str) else rk
    k = {"drag": 0, "l2": 1}[kind]
    if dq0 is None and dref is None:
        lib.hco_objective(ni, nj, _ptr(nodes), _ptr(bcv), fl, lm, r, float(cfl), _ptr(sp), refp, _ptr(q),
                          int(nsteps), k, float(scale), float(direction[0]), float(direction[1]), _ptr(tgt),
                          _ptr(w), _ptr(out))
        return float(out[0]), None
    dq = None if dq0 is None else np.ascontiguousarray(dq0, dtype=np.float64)
    drefp, keep_d = _sides(dref, ni, nj)
    lib.hco_objective_jvp(ni, nj, _ptr(nodes), _ptr(bcv), fl, lm, r, float(cfl), _ptr(sp), refp, drefp, _ptr(q),
                          _ptr(dq), int(nsteps), k, float(scale), float(direction[0]), float(direction[1]),
                          _ptr(tgt), _ptr(w), 1 if freeze_dt else 0, _ptr(out))
    return float(out[0]), float(out[1])


SBC = {"periodic": 0, "fixed": 1, "riemann": 2}
SFLUX = {"rusanov": 0, "central": 1}


def _declare_scalar(lib):
    if getattr(lib, "_scalar_declared", False):
        return
    v, i, d = C.c_void_p, C.c_int, C.c_double
    lib.hcos_create.restype = v
    lib.hcos_create.argtypes = [i, i, _dp, _ip, i, i, i, i, d]
    lib.hcos_destroy.argtypes = [v]
    lib.hcos_set_ghost_ref.argtypes = [v, i, _dp]
    lib.hcos_set_state.argtypes = [v, _dp]
    lib.hcos_get_state.argtypes = [v, _dp]
    lib.hcos_residual.argtypes = [v, _dp]
    lib.hcos_step.argtypes = [v, i, _dp]
    lib.hcos_flux.argtypes = [i, _dp, _dp, _dp, _dp]
    lib.hcos_bc_riemann.argtypes = [_dp, _dp, _dp, _dp]
    lib._scalar_declared = True


def scalar_flux(kind, face, ql, qr):
    lib = load(False)
    _declare_scalar(lib)
    out = np.empty(4)
    lib.hcos_flux(int(kind), np.ascontiguousarray(face, dtype=np.float64), np.ascontiguousarray(ql, dtype=np.float64),
                  np.ascontiguousarray(qr, dtype=np.float64), out)
    return out


def scalar_bc_riemann(face, qi, qb):
    lib = load(False)
    _declare_scalar(lib)
    out = np.empty(3)
    lib.hcos_bc_riemann(np.ascontiguousarray(face, dtype=np.float64), np.ascontiguousarray(qi, dtype=np.float64),
                        np.ascontiguousarray(qb, dtype=np.float64), out)
    return out


def scalar_objective(mesh_nodes, ni, nj, bc, q0, nsteps, target, flux="rusanov", limiter="vanalbada", rk="ssp34",
                     cfl=0.5, ref=None, weight=(1.0, 1.0, 1.0), dq0=None, dref=None, freeze_dt=True):
    """L2 objective of an RK run of the scalar oracle (global timestep): J = sum over cells
    and the three conserved variables {u, v, q} of weight[v] (q_N - target)^2.  With a
    direction (dq0 and/or dref) also the exact derivative of J along it (forward-mode dual
    numbers through the same oracle code), timesteps frozen unless freeze_dt is False.
    Returns (J, dJ or None)."""
    lib = load(False)
    if not getattr(lib, "_sobj_declared", False):
        v, i, d = C.c_void_p, C.c_int, C.c_double
        lib.hcos_objective.argtypes = [i, i, v, v, i, i, i, d, v, v, v, v, i, v, v, i, v]
        lib._sobj_declared = True
    nodes = np.ascontiguousarray(mesh_nodes, dtype=np.float64)
    bcv = np.array([SBC[b] if isinstance(b, str) else int(b) for b in bc], dtype=np.int32)
    q = np.ascontiguousarray(q0, dtype=np.float64)
    tgt = np.ascontiguousarray(target, dtype=np.float64)
    w = np.asarray(list(weight)[:3], dtype=np.float64)
    refp, keep_r = _sides(ref, ni, nj, 3)
    has_dir = dq0 is not None or dref is not None
    dq = None if dq0 is None else np.ascontiguousarray(dq0, dtype=np.float64)
    drefp, keep_d = _sides(dref, ni, nj, 3)
    out = np.zeros(2)
    lib.hcos_objective(ni, nj, _ptr(nodes), _ptr(bcv), SFLUX[flux] if isinstance(flux, str) else flux,
                       LIMITER[limiter] if isinstance(limiter, str) else limiter, RK[rk] if isinstance(rk, str) else rk,
                       float(cfl), refp, drefp if dref is not None else None, _ptr(q),
                       _ptr(dq) if has_dir and dq is not None else None, int(nsteps), _ptr(tgt), _ptr(w),
                       1 if freeze_dt else 0, _ptr(out))
    if not has_dir:
        return float(out[0]), None
    return float(out[0]), float(out[1])


def smooth_1d(r0, alpha, kind="implicit", ends="a"):
    """Residual smoothing of the legacy 1D path (hc_oracle_smooth.hpp) of each row of r0
    (shape (nplanes, n) or (n,)): kind "implicit" (centralImplicitSmoothing) or "explicit"
    (centralExplicitSmoothing); ends "p" periodic, "a" one-neighbour, "n" unscaled."""
    lib = load(False)
    if not getattr(lib, "_smooth_declared", False):
        lib.hco_smooth_1d.argtypes = [C.c_int, _dp, _dp, C.c_longlong, C.c_int, C.c_double, C.c_int]
        lib._smooth_declared = True
    a = np.ascontiguousarray(r0, dtype=np.float64)
    a2 = a.reshape(-1, a.shape[-1])
    out = np.empty_like(a2)
    lib.hco_smooth_1d({"implicit": 0, "explicit": 1}[kind], a2, out, a2.shape[1], a2.shape[0], float(alpha),
                      ord(ends))
    return out.reshape(a.shape)


class ScalarOracleSolver:
    """CPU restatement of integrate() for the scalar advection law (conserved {u, v, q})."""

    def __init__(self, ni, nj, nodes, bc, flux="rusanov", limiter="nolimit3", rk="ssp34", dt="global", cfl=0.5,
                 ghost_ref=None, fast=False):
        self.lib = load(fast)
        _declare_scalar(self.lib)
        self.ni, self.nj = ni, nj
        bcv = np.array([SBC[b] if isinstance(b, str) else int(b) for b in bc], dtype=np.int32)
        self.h = self.lib.hcos_create(ni, nj, np.ascontiguousarray(nodes, dtype=np.float64), bcv,
                                      SFLUX[flux] if isinstance(flux, str) else flux,
                                      LIMITER[limiter] if isinstance(limiter, str) else limiter,
                                      RK[rk] if isinstance(rk, str) else rk, DT[dt] if isinstance(dt, str) else dt,
                                      float(cfl))
        if ghost_ref is not None:
            for side in range(4):
                if ghost_ref[side] is not None:
                    nf = nj if side < 2 else ni
                    arr = np.ascontiguousarray(np.broadcast_to(
                        np.asarray(ghost_ref[side], dtype=np.float64).reshape(3, -1), (3, nf)))
                    self.lib.hcos_set_ghost_ref(self.h, side, arr)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.hcos_destroy(self.h)
            self.h = None

    def set_state(self, soa):
        self.lib.hcos_set_state(self.h, np.ascontiguousarray(soa, dtype=np.float64))

    def get_state(self):
        out = np.empty((3, self.ni, self.nj))
        self.lib.hcos_get_state(self.h, out)
        return out

    def residual(self):
        out = np.empty((4, self.ni, self.nj))
        self.lib.hcos_residual(self.h, out)
        return out

    def step(self, n=1):
        out = np.empty(2)
        self.lib.hcos_step(self.h, int(n), out)
        return float(out[0]), float(out[1])
