"""torch.autograd.Function over the discrete adjoint of the RK time loop.

``run_objective(solver, q0, refs, nsteps, ...)`` returns the objective J (drag
averaged over the steps, or an L2 distance of the final state to a target) of
an RK run started from the primitive state ``q0`` with the fixed-ghost
reference states ``refs`` (one tensor of 4 planes per side, or None).  Its
backward pass calls the hand-written adjoint (include/hc.h,
hc_adjoint_gradient) with binomial checkpointing; the timesteps are frozen at
the forward run's values.  Inputs may be float64 CPU or CUDA tensors.
"""
from __future__ import annotations

import numpy as np
import torch

from .solver import Solver


class _RunObjective(torch.autograd.Function):
    @staticmethod
    def forward(ctx, q0, solver: Solver, nsteps: int, snapshots: int, kind: str, kw: dict, *refs):
        q0n = q0.detach().to("cpu", torch.float64).numpy()
        refn = [None if r is None else r.detach().to("cpu", torch.float64).numpy() for r in refs]
        solver.set_bcs(solver.bc, refn)
        solver.set_state(q0n)
        J, rates = solver.objective(nsteps, kind=kind, **kw)
        ctx.solver, ctx.nsteps, ctx.snapshots, ctx.kind, ctx.kw = solver, nsteps, snapshots, kind, kw
        ctx.q0n, ctx.refn, ctx.rates = q0n, refn, rates
        ctx.devices = (q0.device, [None if r is None else r.device for r in refs])
        ctx.has_ref = [r is not None for r in refs]
        return torch.tensor(J, dtype=torch.float64, device=q0.device)

    @staticmethod
    def backward(ctx, gJ):
        s = ctx.solver
        s.set_bcs(s.bc, ctx.refn)
        s.set_state(ctx.q0n)
        _J, q0b, refb, _rates, _st = s.gradient(ctx.nsteps, ctx.snapshots, kind=ctx.kind, rates=ctx.rates,
                                                **ctx.kw)
        g = float(gJ)
        dq0 = torch.from_numpy(q0b * g).to(ctx.devices[0])
        drefs = []
        for k, has in enumerate(ctx.has_ref):
            drefs.append(torch.from_numpy(refb[k] * g).to(ctx.devices[1][k]) if has else None)
        return (dq0, None, None, None, None, None, *drefs)


def run_objective(solver: Solver, q0: torch.Tensor, refs, nsteps: int, snapshots: int = 20, kind: str = "drag",
                  **kw) -> torch.Tensor:
    """Differentiable J(q0, refs) of an nsteps RK run on `solver`'s mesh and configuration."""
    refs = list(refs) if refs is not None else [None] * 4
    return _RunObjective.apply(q0, solver, int(nsteps), int(snapshots), kind, dict(kw), *refs)


def freestream(mach: torch.Tensor, alpha: torch.Tensor, gamma: float = 1.4):
    """Primitive freestream (u, v, rho, p) with unit speed of sound, rho = 1."""
    one = torch.ones((), dtype=torch.float64, device=mach.device)
    return torch.stack([mach * torch.cos(alpha), mach * torch.sin(alpha), one, one / gamma])


__all__ = ["run_objective", "freestream"]
