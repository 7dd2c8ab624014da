"""torch.autograd.Functions over the discrete adjoint of the RK time loop.

``run_objective(solver, q0, refs, nsteps, ...)`` returns the objective J (drag
averaged over the steps, or an L2 distance of the final state to a target) of
an RK run started from the primitive state ``q0`` with the fixed-ghost
reference states ``refs`` (one tensor of 4 planes per side, or None).

``batch_l2_objective(batch, q0s, targets, nsteps, ...)`` returns, for every
instance k of a batch, J_k = sum_v w_v (q_k(N) - target_k)^2 after nsteps steps
from the primitive states ``q0s[k]``: a tensor of shape (ninst,).

Both run the forward sweep once, in forward(): it records the checkpoints of the
binomial schedule in the library (hc_adjoint_record, hc_batch_adjoint_record),
and backward() runs only the reverse sweep from them (hc_adjoint_reverse,
hc_batch_adjoint_reverse), which writes the gradients straight into CUDA
tensors.  CUDA inputs stay on the device: states go in by device pointer, the
L2 targets are read on the device.  The timesteps are frozen at the forward
run's values.  A solver or batch holds one recording at a time: a second
forward before the first one's backward drops the first recording, whose
backward then fails.
"""
from __future__ import annotations

import numpy as np
import torch

from .solver import Solver


def _wait_for_torch(t: torch.Tensor) -> None:
    """The library runs on its own stream: let torch's work producing t finish first."""
    if t.is_cuda:
        torch.cuda.current_stream(t.device).synchronize()


class _RunObjective(torch.autograd.Function):
    @staticmethod
    def forward(ctx, q0, solver: Solver, nsteps: int, snapshots: int, kind: str, kw: dict, *refs):
        refn = [None if r is None else r.detach().to("cpu", torch.float64).numpy() for r in refs]
        solver.set_bcs(solver.bc, refn)
        if q0.is_cuda:
            dtype = torch.float32 if solver.precision == "fp32" else torch.float64
            q = q0.detach().to(dtype).contiguous()
            _wait_for_torch(q)  # the conversion runs on torch's stream, the upload on the library's
            solver.upload_device(q)
        else:
            solver.set_state(q0.detach().to(torch.float64).numpy())
        J, rates = solver.record(nsteps, snapshots, kind=kind, **kw)
        ctx.solver, ctx.rates = solver, rates
        ctx.q0_meta = (q0.device, q0.dtype)
        ctx.ref_meta = [None if r is None else (r.device, r.dtype) for r in refs]
        return torch.tensor(J, dtype=torch.float64, device=q0.device)

    @staticmethod
    def backward(ctx, gJ):
        s = ctx.solver
        m = s.mesh
        nv = s.nv
        q0b = torch.empty((nv, m.ni, m.nj), dtype=torch.float64, device="cuda")
        nref = sum(nv * m.nface(side) for side in range(4))
        refb = torch.empty(max(nref, 1), dtype=torch.float64, device="cuda")
        _wait_for_torch(refb)  # torch's earlier work on these blocks, before the library writes them
        s.reverse(q0b, refb)
        g = gJ.detach().to(device="cuda", dtype=torch.float64)
        dev, dt = ctx.q0_meta
        dq0 = (q0b * g).to(device=dev, dtype=dt)
        drefs, off = [], 0
        for side, meta in enumerate(ctx.ref_meta):
            nf = m.nface(side)
            if meta is not None:
                drefs.append((refb[off:off + nv * nf].reshape(nv, nf) * g).to(device=meta[0], dtype=meta[1]))
            else:
                drefs.append(None)
            off += nv * nf
        return (dq0, None, None, None, None, None, *drefs)


def run_objective(solver: Solver, q0: torch.Tensor, refs, nsteps: int, snapshots: int = 20, kind: str = "drag",
                  **kw) -> torch.Tensor:
    """Differentiable J(q0, refs) of an nsteps RK run on `solver`'s mesh and configuration."""
    refs = list(refs) if refs is not None else [None] * 4
    return _RunObjective.apply(q0, solver, int(nsteps), int(snapshots), kind, dict(kw), *refs)


class _BatchL2(torch.autograd.Function):
    @staticmethod
    def forward(ctx, batch, nsteps: int, snapshots: int, weight, targets, *q0s):
        qs = [q.detach().to(device="cuda", dtype=torch.float64).contiguous() for q in q0s]
        tg = [t.detach().to(device="cuda", dtype=torch.float64).contiguous() if torch.is_tensor(t)
              else torch.from_numpy(np.ascontiguousarray(t, dtype=np.float64)).cuda() for t in targets]
        # the conversions run on torch's stream, the uploads and the sweep on the library's
        torch.cuda.current_stream().synchronize()
        for k, q in enumerate(qs):
            batch.upload_device(k, q)
        J = batch.record(nsteps, tg, snapshots, weight)
        ctx.batch = batch
        ctx.meta = [(tuple(q.shape), q.device, q.dtype) for q in q0s]
        return torch.from_numpy(J).to(q0s[0].device)

    @staticmethod
    def backward(ctx, gJ):
        outs = [torch.empty(shape, dtype=torch.float64, device="cuda") for shape, _, _ in ctx.meta]
        torch.cuda.current_stream().synchronize()
        ctx.batch.reverse(outs)
        g = gJ.detach().to(device="cuda", dtype=torch.float64)
        grads = [(o * g[k]).to(device=dev, dtype=dt) for k, (o, (_, dev, dt)) in enumerate(zip(outs, ctx.meta))]
        return (None, None, None, None, None, *grads)


def batch_l2_objective(batch, q0s, targets, nsteps: int, snapshots: int = 20,
                       weight=(1.0, 1.0, 1.0, 1.0)) -> torch.Tensor:
    """Differentiable per-instance L2 objectives J_k(q0_k) of an nsteps batched RK run, one
    batched adjoint for every instance's gradient (the config-5 pattern); q0s and targets
    one tensor (or array, for targets) per instance, of the instance's state shape."""
    return _BatchL2.apply(batch, int(nsteps), int(snapshots), tuple(float(w) for w in weight), list(targets), *q0s)


def freestream(mach: torch.Tensor, alpha: torch.Tensor, gamma: float = 1.4):
    """Primitive freestream (u, v, rho, p) with unit speed of sound, rho = 1."""
    one = torch.ones((), dtype=torch.float64, device=mach.device)
    return torch.stack([mach * torch.cos(alpha), mach * torch.sin(alpha), one, one / gamma])


__all__ = ["run_objective", "batch_l2_objective", "freestream"]
