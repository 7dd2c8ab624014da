"""Batched path: many independent meshes of uneven sizes in one set of device
buffers, advanced by one persistent launch per RK stage (include/hc.h,
hc_batch_*).  The reference runs one mesh per process and has no counterpart.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi
from ._capi import (BATCH_MODE, BC, DTMODE, FLUX, LIMITER, ORDER, PRECISION, RK, TILE, Config, Schedule,
                    StepStats, check)
from .solver import Mesh, _dptr


class Batch:
    """Instances = list of (mesh, bc, ref, state); shared law/flux/limiter/RK/CFL/species.
    law="euler": states {u, v, rho, p} (4 planes); law="scalar": scalar advection,
    states {u, v, q} (3 planes), Rusanov or central flux."""

    def __init__(self, instances, flux="slau", limiter="vanalbada", rk="ssp34", precision="fp32", dt="global",
                 cfl=0.5, species=(1.4, 287.058, 0.5), stream=None, basis="primitive", law="euler",
                 corrections=None):
        self.lib = _capi.load()
        self.meshes = [inst[0] for inst in instances]
        self.law = law
        self.nv = 3 if law == "scalar" else 4
        nv = self.nv
        n = len(instances)
        cfg = Config(FLUX[flux], LIMITER[limiter], RK[rk], PRECISION[precision], DTMODE[dt], float(cfl),
                     _capi.LAW[law], _capi.BASIS[basis])
        ni = (C.c_int * n)(*[m.ni for m in self.meshes])
        nj = (C.c_int * n)(*[m.nj for m in self.meshes])
        nodes = (C.POINTER(C.c_double) * n)(*[_dptr(m.nodes) for m in self.meshes])
        bcs = (C.c_int * (4 * n))()
        refs = (C.POINTER(C.c_double) * (4 * n))()
        self._keep = []
        for k, (mesh, bc, ref, _q) in enumerate(instances):
            for s in range(4):
                bcs[4 * k + s] = BC[bc[s]] if isinstance(bc[s], str) else int(bc[s])
                r = None if ref is None else ref[s]
                if r is None:
                    refs[4 * k + s] = C.POINTER(C.c_double)()
                else:
                    arr = np.ascontiguousarray(np.broadcast_to(np.asarray(r, dtype=np.float64).reshape(nv, -1),
                                                               (nv, mesh.nface(s))))
                    self._keep.append(arr)
                    refs[4 * k + s] = _dptr(arr)
        h = C.c_void_p()
        check(self.lib.hc_batch_create(C.byref(cfg), n, ni, nj, nodes, bcs, refs, *[float(x) for x in species],
                                       C.byref(h)))
        self.h = h
        self.corrections = _capi.fix_mask(corrections)
        if self.corrections:
            check(self.lib.hc_batch_set_corrections(self.h, self.corrections))
        self.n = n
        if stream is not None:
            check(self.lib.hc_batch_set_stream(self.h, C.c_void_p(int(stream) if stream else None)))
        for k, inst in enumerate(instances):
            self.set_state(k, inst[3])

    def close(self):
        if getattr(self, "h", None):
            self.lib.hc_batch_destroy(self.h)
            self.h = None

    __del__ = close

    @property
    def cells(self) -> int:
        return sum(m.ni * m.nj for m in self.meshes)

    def set_state(self, k: int, prim: np.ndarray) -> None:
        a = np.ascontiguousarray(prim, dtype=np.float64)
        m = self.meshes[k]
        if a.shape != (self.nv, m.ni, m.nj):
            raise ValueError("state shape mismatch")
        check(self.lib.hc_batch_state_upload(self.h, k, _dptr(a)))

    def get_state(self, k: int) -> np.ndarray:
        m = self.meshes[k]
        out = np.empty((self.nv, m.ni, m.nj))
        check(self.lib.hc_batch_state_download(self.h, k, _dptr(out)))
        return out

    def schedule(self) -> dict:
        s = Schedule()
        check(self.lib.hc_batch_get_schedule(self.h, C.byref(s)))
        inv_t = {v: k for k, v in TILE.items()}
        inv_o = {v: k for k, v in ORDER.items()}
        return {"tile": inv_t[s.tile], "ctas_per_sm": s.ctas_per_sm, "order": inv_o[s.order],
                "ms_per_step": float(s.ms_per_step)}

    def set_schedule(self, tile="8x32", ctas_per_sm=2, order="largest_first") -> None:
        s = Schedule(TILE[tile], int(ctas_per_sm), ORDER[order], 0.0)
        check(self.lib.hc_batch_set_schedule(self.h, C.byref(s)))

    def autotune(self, steps: int = 2) -> dict:
        s = Schedule()
        check(self.lib.hc_batch_autotune(self.h, int(steps), C.byref(s)))
        return self.schedule() | {"ms_per_step": float(s.ms_per_step)}

    def step_async(self, n: int = 1, mode: str = "persistent") -> None:
        check(self.lib.hc_batch_step_async(self.h, int(n), BATCH_MODE[mode]))

    def capture(self, n: int) -> None:
        check(self.lib.hc_batch_graph_capture(self.h, int(n)))

    def replay(self) -> None:
        check(self.lib.hc_batch_graph_launch(self.h))

    def sync(self):
        st = (StepStats * self.n)()
        check(self.lib.hc_batch_sync(self.h, st))
        return list(st)

    def kernel_launches(self) -> int:
        return int(self.lib.hc_batch_kernel_launches(self.h))

    def set_adjoint_tapes(self, ntapes: int = -1) -> None:
        """Stage tapes of the batched adjoint's checkpointing (hc_batch_set_adjoint_tapes):
        -1 one per snapshot and one more, 0 none, k at most k."""
        check(self.lib.hc_batch_set_adjoint_tapes(self.h, int(ntapes)))

    def gradient(self, nsteps, targets, snapshots=20, weight=(1.0, 1.0, 1.0, 1.0), want=None):
        """Every instance's L2 objective J_k = sum w_v (q_k(N) - target_k)^2 after nsteps
        steps and its gradient with respect to the instance's current state, from one
        batched adjoint (hc_batch_adjoint_gradient).  `want`: indices whose gradients
        are copied back (default all).  Returns (J array, {k: q0_bar}, stats).  Scalar
        batches: 3 planes {u, v, q}, weight[3] unused."""
        from ._capi import AdjointStats, Objective
        n, nv = self.n, self.nv
        tg = [np.ascontiguousarray(t, dtype=np.float64) for t in targets]
        for k, t in enumerate(tg):
            m = self.meshes[k]
            if t.shape != (nv, m.ni, m.nj):
                raise ValueError(f"target {k} must have shape ({nv}, {m.ni}, {m.nj})")
        tptr = (C.POINTER(C.c_double) * n)(*[_dptr(t) for t in tg])
        want = range(n) if want is None else list(want)
        grads = {k: np.empty((nv, self.meshes[k].ni, self.meshes[k].nj)) for k in want}
        gptr = (C.POINTER(C.c_double) * n)()
        for k, g in grads.items():
            gptr[k] = _dptr(g)
        o = Objective()
        o.kind = _capi.OBJECTIVE["l2"]
        for v in range(4):
            o.weight[v] = float(weight[v])
        J = np.empty(n)
        st = AdjointStats()
        check(self.lib.hc_batch_adjoint_gradient(self.h, int(nsteps), int(snapshots), C.byref(o), tptr, _dptr(J),
                                                 gptr, C.byref(st)))
        return J, grads, st


    def upload_device(self, k: int, prim) -> None:
        """Instance k's state from a float64 CUDA tensor of shape (nv, ni, nj), asynchronous
        on the batch's stream (hc_batch_state_upload_device)."""
        m = self.meshes[k]
        if tuple(prim.shape) != (self.nv, m.ni, m.nj) or not prim.is_cuda or prim.dtype != _torch().float64:
            raise ValueError(f"instance {k}: a float64 CUDA tensor of shape ({self.nv}, {m.ni}, {m.nj}) is needed")
        check(self.lib.hc_batch_state_upload_device(self.h, k, C.c_void_p(prim.contiguous().data_ptr())))

    def _l2(self, weight, on_device):
        from ._capi import Objective
        o = Objective()
        o.kind = _capi.OBJECTIVE["l2"]
        for v in range(4):
            o.weight[v] = float(weight[v])
        o.target_on_device = 1 if on_device else 0
        return o

    def record(self, nsteps, targets, snapshots=20, weight=(1.0, 1.0, 1.0, 1.0)) -> np.ndarray:
        """The forward half of `gradient` (hc_batch_adjoint_record): every instance's J after
        nsteps steps; the checkpoints stay in the batch for `reverse`.  targets: per instance
        an array, or a float64 CUDA tensor (read on the device)."""
        n = self.n
        dev = all(hasattr(t, "is_cuda") and t.is_cuda for t in targets)
        if dev:
            self._tape_targets = [t.detach().contiguous() for t in targets]
            ptrs = [C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double)) for t in self._tape_targets]
        else:
            self._tape_targets = [np.ascontiguousarray(t, dtype=np.float64) for t in targets]
            ptrs = [_dptr(t) for t in self._tape_targets]
        for k, t in enumerate(self._tape_targets):
            m = self.meshes[k]
            if tuple(t.shape) != (self.nv, m.ni, m.nj):
                raise ValueError(f"target {k} must have shape ({self.nv}, {m.ni}, {m.nj})")
        tptr = (C.POINTER(C.c_double) * n)(*ptrs)
        o = self._l2(weight, dev)
        J = np.empty(n)
        check(self.lib.hc_batch_adjoint_record(self.h, int(nsteps), int(snapshots), C.byref(o), tptr, _dptr(J)))
        return J

    def reverse(self, out=None):
        """The reverse half (hc_batch_adjoint_reverse): out[k] a float64 CUDA tensor of instance
        k's state shape receiving dJ_k/dq0_k on the device (None entries skipped), or None for
        host arrays returned as {k: q0_bar}.  Returns (grads or None, stats)."""
        from ._capi import AdjointStats
        n = self.n
        gptr = (C.POINTER(C.c_double) * n)()
        host = None
        if out is None:
            host = {k: np.empty((self.nv, m.ni, m.nj)) for k, m in enumerate(self.meshes)}
            for k, g in host.items():
                gptr[k] = _dptr(g)
        else:
            for k, g in enumerate(out):
                if g is not None:
                    gptr[k] = C.cast(C.c_void_p(g.data_ptr()), C.POINTER(C.c_double))
        st = AdjointStats()
        check(self.lib.hc_batch_adjoint_reverse(self.h, gptr, 0 if out is None else 1, C.byref(st)))
        self._tape_targets = None
        self.last_stats = st
        return host, st


def _torch():
    import torch
    return torch


def uneven_riemann_batch(n: int, seed: int, sizes=tuple(range(64, 1025, 32))):
    """n four-quadrant Riemann instances with Ni, Nj drawn uniformly from `sizes`."""
    from . import cases
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        ni, nj = int(rng.choice(sizes)), int(rng.choice(sizes))
        mesh, bc, ref, q, _sp = cases.quadrant_riemann(ni, nj, rng)
        out.append((mesh, bc, ref, q))
    return out


__all__ = ["Batch", "uneven_riemann_batch", "Mesh"]
