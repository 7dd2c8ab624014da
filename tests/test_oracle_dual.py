"""Forward-mode dual numbers through the oracle (the FP64 reference gradient of
the discrete adjoint): exact directional derivatives of RK-run objectives
against central differences of the plain FP64 oracle, on CPU."""
import numpy as np
import pytest

from hyperboliconvergence_gb300 import cases
from hyperboliconvergence_gb300.solver import Mesh
from oracle import oracle_py

H = 1e-6


def cylinder(nr=8, nth=24, mach=0.4):
    mesh = Mesh.cylinder(nr, nth, 0.5, 4.0, 1.05)
    qinf = np.array([mach * np.cos(0.1), mach * np.sin(0.1), 1.0, 1.0 / 1.4])
    c = mesh.centres()
    shape = 0.5 * np.exp(-((c[0] - 1.0) ** 2 + c[1] ** 2)) + 0.1 * c[0] + 0.07 * c[1]
    q = qinf[:, None, None] + np.array([0.02, 0.02, 0.03, 0.02])[:, None, None] * shape[None]
    ref = [None, np.broadcast_to(qinf[:, None], (4, nth)).copy(), None, None]
    return mesh, ["wall", "fixed", "periodic", "periodic"], ref, q


@pytest.mark.parametrize("limiter", ["nolimit2", "vanalbada", "minmod"])
def test_dual_drag_derivative_matches_fd(limiter):
    mesh, bc, ref, q = cylinder()
    d = q - ref[1][:, :1, None]  # scales the limiter arguments: no kink crossings
    kw = dict(kind="drag", flux="roe", limiter=limiter, rk="ssp34", ref=ref, scale=3.0)
    # central differences of the plain oracle move the timestep with the state
    J, dJ = oracle_py.objective(mesh.nodes, mesh.ni, mesh.nj, bc, q, 4, dq0=d, freeze_dt=False, **kw)
    jp, _ = oracle_py.objective(mesh.nodes, mesh.ni, mesh.nj, bc, q + H * d, 4, **kw)
    jm, _ = oracle_py.objective(mesh.nodes, mesh.ni, mesh.nj, bc, q - H * d, 4, **kw)
    fd = (jp - jm) / (2 * H)
    assert abs(dJ) > 0
    assert abs(fd - dJ) <= 1e-7 * abs(dJ), (fd, dJ)
    # holding the timesteps changes the derivative (the adjoint's convention)
    _, dJf = oracle_py.objective(mesh.nodes, mesh.ni, mesh.nj, bc, q, 4, dq0=d, **kw)
    assert dJf != dJ


def test_dual_l2_derivative_matches_fd_reference_direction():
    mesh, bc, ref, q = cylinder()
    dref = [None, np.zeros_like(ref[1]), None, None]
    dref[1][0] = 0.01
    dref[1][3] = 0.002
    kw = dict(kind="l2", flux="rusanov", limiter="nolimit3", rk="ssp33", target=q * 0.98)
    J, dJ = oracle_py.objective(mesh.nodes, mesh.ni, mesh.nj, bc, q, 5, ref=ref, dref=dref, freeze_dt=False, **kw)
    refp = [None, ref[1] + H * dref[1], None, None]
    refm = [None, ref[1] - H * dref[1], None, None]
    jp, _ = oracle_py.objective(mesh.nodes, mesh.ni, mesh.nj, bc, q, 5, ref=refp, **kw)
    jm, _ = oracle_py.objective(mesh.nodes, mesh.ni, mesh.nj, bc, q, 5, ref=refm, **kw)
    fd = (jp - jm) / (2 * H)
    assert abs(fd - dJ) <= 1e-6 * abs(dJ), (fd, dJ)


def test_dual_value_equals_plain_objective():
    mesh, bc, ref, q = cylinder()
    kw = dict(kind="drag", flux="roe", limiter="vanalbada", rk="ssp34", ref=ref, scale=1.0)
    J0, _ = oracle_py.objective(mesh.nodes, mesh.ni, mesh.nj, bc, q, 3, **kw)
    J1, _ = oracle_py.objective(mesh.nodes, mesh.ni, mesh.nj, bc, q, 3, dq0=np.zeros_like(q), **kw)
    assert J0 == J1
