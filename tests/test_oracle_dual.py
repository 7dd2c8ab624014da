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


def scalar_case():
    """Scalar advection on an O-grid with fixed inner and outer rings: a smooth bump
    advected by a uniform velocity, seeded target."""
    mesh = Mesh.cylinder(8, 24, 0.5, 4.0, 1.05)
    c = mesh.centres()
    q = np.empty((3, 8, 24))
    q[0], q[1] = 0.6 + 0.05 * c[1], 0.3 - 0.04 * c[0]
    q[2] = 1.0 + 0.4 * np.exp(-((c[0] - 1.0) ** 2 + c[1] ** 2))
    ref = [np.stack([np.full(24, 0.6), np.full(24, 0.3), np.full(24, 1.1)]),
           np.stack([np.full(24, 0.6), np.full(24, 0.3), np.full(24, 0.9)]), None, None]
    target = q * (1 + 0.02 * np.random.default_rng(5).standard_normal(q.shape))
    return mesh, ["fixed", "fixed", "periodic", "periodic"], ref, q, target


@pytest.mark.parametrize("flux", ["rusanov", "central"])
@pytest.mark.parametrize("limiter", ["nolimit2", "vanalbada", "minmod"])
def test_dual_scalar_l2_derivative_matches_fd(flux, limiter):
    mesh, bc, ref, q, target = scalar_case()
    # scales each variable's deviation from its uniform part, so every limiter argument
    # scales too (no kink crossings within the differences' steps)
    d = np.stack([0.5 * (q[0] - 0.6), 0.5 * (q[1] - 0.3), q[2] - 1.0])
    kw = dict(flux=flux, limiter=limiter, ref=ref, weight=(0.5, 2.0, 1.0))
    J, dJ = oracle_py.scalar_objective(mesh.nodes, mesh.ni, mesh.nj, bc, q, 4, target, dq0=d, freeze_dt=False, **kw)
    jp, _ = oracle_py.scalar_objective(mesh.nodes, mesh.ni, mesh.nj, bc, q + H * d, 4, target, **kw)
    jm, _ = oracle_py.scalar_objective(mesh.nodes, mesh.ni, mesh.nj, bc, q - H * d, 4, target, **kw)
    fd = (jp - jm) / (2 * H)
    assert abs(dJ) > 0
    assert abs(fd - dJ) <= 1e-7 * abs(dJ), (fd, dJ)
    j0, _ = oracle_py.scalar_objective(mesh.nodes, mesh.ni, mesh.nj, bc, q, 4, target, **kw)
    assert j0 == J


def test_dual_scalar_reference_layer_derivative():
    """Derivative with respect to a fixed side's reference layer (the ghost state)."""
    mesh, bc, ref, q, target = scalar_case()
    dref = [np.ones((3, 24)) * np.array([0.0, 0.0, 1.0])[:, None], None, None, None]
    kw = dict(flux="rusanov", limiter="vanalbada", weight=(1.0, 1.0, 1.0))
    _, dJ = oracle_py.scalar_objective(mesh.nodes, mesh.ni, mesh.nj, bc, q, 3, target, ref=ref, dref=dref,
                                       freeze_dt=False, **kw)
    rp = [ref[0] + H * dref[0], ref[1], None, None]
    rm = [ref[0] - H * dref[0], ref[1], None, None]
    jp, _ = oracle_py.scalar_objective(mesh.nodes, mesh.ni, mesh.nj, bc, q, 3, target, ref=rp, **kw)
    jm, _ = oracle_py.scalar_objective(mesh.nodes, mesh.ni, mesh.nj, bc, q, 3, target, ref=rm, **kw)
    fd = (jp - jm) / (2 * H)
    assert abs(dJ) > 0
    assert abs(fd - dJ) <= 1e-6 * abs(dJ), (fd, dJ)
