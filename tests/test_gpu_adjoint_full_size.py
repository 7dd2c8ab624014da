"""The adjoint at the differentiated configuration's size: the 256 x 512 cylinder O-grid
(radius 0.5 to 20, radial stretching 1.01), M 0.4, Roe + van Albada, ssp34 at CFL 0.5 with the
global timestep, time-averaged drag, binomial checkpointing -- shortened to 12 steps so that
central differences stay cheap (the 400-step run is the bench's).

* <grad J, d> along a smooth direction d against the central difference of J at frozen
  timesteps (h = 1e-6, relative 1e-6; measured 5e-9), from a smooth non-uniform start whose
  limiter arguments sit away from the kinks.
* dJ/dMach and dJ/dalpha of the drag coefficient through the autograd Function (the start and
  the fixed far field both the freestream of (M, alpha)) against central differences."""
import math

import numpy as np
import pytest

from hyperboliconvergence_gb300.solver import Mesh, Solver

pytestmark = pytest.mark.gpu

NR, NTH, MACH, ALPHA, N, H = 256, 512, 0.4, 0.1, 12, 1e-6
SP = (1.4, 287.058, MACH)


def freestream_np(m, a):
    return np.array([m * math.cos(a), m * math.sin(a), 1.0, 1.0 / 1.4])


def solver(mesh, ref):
    return Solver(mesh, ["wall", "fixed", "periodic", "periodic"], ref, flux="roe", limiter="vanalbada",
                  rk="ssp34", precision="fp64", dt="global", cfl=0.5, species=SP)


def test_state_gradient_matches_central_difference():
    mesh = Mesh.cylinder(NR, NTH, 0.5, 20.0, 1.01)
    qinf = freestream_np(MACH, ALPHA)
    c = mesh.centres()
    shape = 0.5 * np.exp(-((c[0] - 1.0) ** 2 + c[1] ** 2)) + 0.01 * c[0] + 0.007 * c[1]
    q = qinf[:, None, None] + np.array([0.02, 0.02, 0.03, 0.02])[:, None, None] * shape[None]
    s = solver(mesh, [None, np.broadcast_to(qinf[:, None], (4, NTH)).copy(), None, None])
    s.set_state(q)
    kw = dict(kind="drag", scale=1.0)
    J, g, _, rates, st = s.gradient(N, snapshots=4, **kw)
    assert st.replays == 0
    d = 1e-2 * np.stack([np.sin(2 * c[0]) * np.cos(c[1]), np.cos(c[0]) * np.sin(3 * c[1]),
                         np.exp(-0.1 * (c[0] ** 2 + c[1] ** 2)), np.cos(c[0] + c[1])])
    s.set_state(q + H * d)
    jp, _ = s.objective(N, rates=rates, **kw)
    s.set_state(q - H * d)
    jm, _ = s.objective(N, rates=rates, **kw)
    fd = (jp - jm) / (2 * H)
    ad = float(np.sum(g * d))
    assert abs(fd - ad) <= 1e-6 * abs(fd), (fd, ad)


def test_mach_and_alpha_derivatives_through_the_function():
    torch = pytest.importorskip("torch")
    from hyperboliconvergence_gb300.autograd import freestream, run_objective
    mesh = Mesh.cylinder(NR, NTH, 0.5, 20.0, 1.01)
    s = solver(mesh, [None, np.zeros((4, NTH)), None, None])

    def cd_of(m, a):
        qinf = freestream(m, a)
        q0 = qinf[:, None, None].expand(4, NR, NTH).contiguous()
        ref1 = qinf[:, None].expand(4, NTH).contiguous()
        j = run_objective(s, q0, [None, ref1, None, None], N, snapshots=4, kind="drag", scale=1.0,
                          direction=(1.0, 0.0))
        return j / (0.5 * m * m)

    m = torch.tensor(MACH, dtype=torch.float64, requires_grad=True)
    a = torch.tensor(ALPHA, dtype=torch.float64, requires_grad=True)
    cd_of(m, a).backward()
    q = freestream_np(MACH, ALPHA)
    s.set_bcs(s.bc, [None, np.broadcast_to(q[:, None], (4, NTH)).copy(), None, None])
    s.set_state(np.broadcast_to(q[:, None, None], (4, NR, NTH)).copy())
    _, rates = s.objective(N, kind="drag", scale=1.0)

    def cd_np(mv, av):
        qv = freestream_np(mv, av)
        s.set_bcs(s.bc, [None, np.broadcast_to(qv[:, None], (4, NTH)).copy(), None, None])
        s.set_state(np.broadcast_to(qv[:, None, None], (4, NR, NTH)).copy())
        j, _ = s.objective(N, kind="drag", rates=rates, scale=1.0)
        return j / (0.5 * mv * mv)

    fdm = (cd_np(MACH + H, ALPHA) - cd_np(MACH - H, ALPHA)) / (2 * H)
    fda = (cd_np(MACH, ALPHA + H) - cd_np(MACH, ALPHA - H)) / (2 * H)
    assert abs(m.grad.item() - fdm) <= 1e-6 * abs(fdm), (m.grad.item(), fdm)
    assert abs(a.grad.item() - fda) <= 1e-6 * max(abs(fda), 1e-12), (a.grad.item(), fda)
