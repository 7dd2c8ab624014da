"""Discrete adjoint of the scalar advection law (hc_adjoint_gradient on a scalar-law
context, the L2 objective on {u, v, q}).

The reference gradient is the oracle's forward-mode derivative with the timesteps
frozen at their values (oracle_py.scalar_objective, itself checked against central
differences in test_oracle_dual): <grad J, d> along seeded noise directions of the
initial state and of a fixed side's reference layer agree to 1e-9 in FP64, J to the
FP64 parity bar; fixed and Riemann (inflow/outflow) sides.  Binomial checkpointing reverses bit for bit like storing every
state; FP32 gradients agree with FP64 to FP32 accuracy.
"""
import numpy as np
import pytest

from hyperboliconvergence_gb300.solver import Mesh, Solver
from oracle import oracle_py

pytestmark = pytest.mark.gpu

NSTEPS = 6
W = (0.5, 2.0, 1.0)


def generic_fields(c, base=(0.8, -0.5)):
    """Smooth fields with no symmetry of the mesh: no face sees a limiter argument or a
    Rusanov tie that vanishes in exact arithmetic (there the derivative would follow
    round-off, differently in the oracle and the product)."""
    x, y = c
    u = base[0] + 0.1 * np.sin(2 * np.pi * (y + 0.13)) + 0.07 * np.cos(2 * np.pi * (x + 0.29)) + 0.03 * x * y
    v = base[1] + 0.05 * np.cos(2 * np.pi * (x + 0.41)) + 0.06 * np.sin(2 * np.pi * (y + 0.07)) - 0.02 * x
    q = 1.0 + 0.5 * np.exp(-((x - 0.43) ** 2 + (y - 0.61) ** 2) / 0.02) + 0.1 * np.sin(3.1 * x + 1.7 * y + 0.3)
    return np.stack([u, v, q])


def periodic_case():
    mesh = Mesh.linspace(24, 20, 0.0, 1.0, 0.0, 1.0)
    q = generic_fields(mesh.centres())
    target = q * (1 + 0.03 * np.random.default_rng(8).standard_normal(q.shape))
    return mesh, ["periodic"] * 4, None, q, target


def ogrid_case():
    mesh = Mesh.cylinder(8, 24, 0.5, 4.0, 1.05)
    q = generic_fields(mesh.centres() * 0.3, base=(0.6, 0.3))
    ref = [np.stack([np.full(24, 0.6), np.full(24, 0.3), 1.1 + 0.05 * np.sin(np.arange(24.0))]),
           np.stack([np.full(24, 0.62), np.full(24, 0.28), 0.9 + 0.03 * np.cos(np.arange(24.0))]), None, None]
    target = q * (1 + 0.02 * np.random.default_rng(5).standard_normal(q.shape))
    return mesh, ["fixed", "fixed", "periodic", "periodic"], ref, q, target


def riemann_case():
    """Inflow/outflow Riemann sides (j) over a rotating-plus-generic velocity."""
    mesh = Mesh.linspace(20, 28, 0.0, 1.0, 0.0, 1.0)
    c = mesh.centres()
    q = generic_fields(c, base=(0.0, 0.0))
    q[0] += -(c[1] - 0.5)
    q[1] += c[0] - 0.5
    xs = np.linspace(0.02, 0.98, 20)
    ref = [None, None, np.stack([-(xs - 0.5), np.full(20, -0.45), 1.0 + 0.1 * np.sin(5 * xs)]),
           np.stack([-(xs - 0.5), np.full(20, 0.55), 1.2 + 0.1 * np.cos(4 * xs)])]
    target = q * (1 + 0.02 * np.random.default_rng(6).standard_normal(q.shape))
    return mesh, ["periodic", "periodic", "riemann", "riemann"], ref, q, target


CASES = {"fixed_ogrid": ogrid_case(), "periodic": periodic_case(), "riemann": riemann_case()}


def gpu_gradient(case, flux, limiter, precision="fp64", snapshots=2, nsteps=NSTEPS):
    mesh, bc, ref, q, target = case
    s = Solver(mesh, bc, ref, flux=flux, limiter=limiter, precision=precision, law="scalar")
    s.set_state(q)
    before = s.get_state()
    J, qb, refb, rates, st = s.gradient(nsteps, snapshots=snapshots, kind="l2", target=target, weight=W + (0.0,))
    assert np.array_equal(s.get_state(), before)  # the context's state is left as it was
    return J, qb, refb, st


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("flux", ["rusanov", "central"])
@pytest.mark.parametrize("limiter", ["nolimit1", "nolimit3", "vanalbada", "minmod", "vanleer"])
def test_scalar_adjoint_matches_dual_reference(name, flux, limiter):
    case = CASES[name]
    mesh, bc, ref, q, target = case
    J, qb, refb, st = gpu_gradient(case, flux, limiter)
    assert st.adjoint_steps == NSTEPS
    rng = np.random.default_rng(11)
    kw = dict(flux=flux, limiter=limiter, ref=ref, weight=W)
    for _ in range(2):
        d = rng.standard_normal(q.shape)
        J0, dJ = oracle_py.scalar_objective(mesh.nodes, mesh.ni, mesh.nj, bc, q, NSTEPS, target, dq0=d, **kw)
        assert J == pytest.approx(J0, rel=1e-12)
        got = float(np.sum(qb * d))
        assert got == pytest.approx(dJ, rel=1e-9, abs=1e-12 * np.abs(qb).sum()), (got, dJ)
    if ref is not None:
        # the first non-periodic side's reference layer
        side = next(k for k in range(4) if ref[k] is not None)
        dr = rng.standard_normal(ref[side].shape)
        drefs = [None] * 4
        drefs[side] = dr
        _, dJ = oracle_py.scalar_objective(mesh.nodes, mesh.ni, mesh.nj, bc, q, NSTEPS, target, dref=drefs, **kw)
        got = float(np.sum(refb[side] * dr))
        assert got == pytest.approx(dJ, rel=1e-9, abs=1e-12 * np.abs(refb[side]).sum()), (got, dJ)
        for k in range(4):
            if ref[k] is None:
                assert np.all(refb[k] == 0)


def test_scalar_adjoint_checkpointing_equals_stored_reversal():
    case = CASES["fixed_ogrid"]
    J1, g1, r1, s1 = gpu_gradient(case, "rusanov", "vanalbada", snapshots=1, nsteps=9)
    J2, g2, r2, s2 = gpu_gradient(case, "rusanov", "vanalbada", snapshots=9, nsteps=9)
    assert J1 == J2
    assert np.array_equal(g1, g2)
    assert all(np.array_equal(a, b) for a, b in zip(r1, r2))
    assert s1.forward_steps > s2.forward_steps


def test_scalar_adjoint_fp32_close_to_fp64():
    case = CASES["periodic"]
    J64, g64, _, _ = gpu_gradient(case, "rusanov", "nolimit3")
    J32, g32, _, _ = gpu_gradient(case, "rusanov", "nolimit3", precision="fp32")
    assert J32 == pytest.approx(J64, rel=1e-4)
    assert np.abs(g32 - g64).max() <= 1e-4 * np.abs(g64).max()


def test_scalar_adjoint_unsupported():
    mesh = Mesh.linspace(20, 28, 0.0, 1.0, 0.0, 1.0)
    q = np.ones((3, 20, 28))
    s = Solver(mesh, ["periodic"] * 4, None, flux="rusanov", law="scalar")
    s.set_state(q)
    with pytest.raises(Exception, match="L2 objective"):
        s.gradient(2, kind="drag")
