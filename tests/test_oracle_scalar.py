"""Scalar advection law: the oracle's pointwise functions against the golden
vectors of the reference's own code (bit for bit), and properties of the oracle
solver (conservation, constant-state preservation, upwind transport)."""
import os

import numpy as np
import pytest

from hyperboliconvergence_gb300.solver import Mesh
from oracle import oracle_py

GOLD = os.path.join(os.path.dirname(__file__), "golden", "scalar_golden.npz")


@pytest.fixture(scope="module")
def g():
    return np.load(GOLD)


@pytest.mark.parametrize("kind", [0, 1])
def test_scalar_fluxes_bit_exact(g, kind):
    got = np.stack([oracle_py.scalar_flux(kind, f, a, b) for f, a, b in zip(g["faces"], g["ql"], g["qr"])])
    assert np.array_equal(got, g[f"flux_{kind}"])


def test_scalar_riemann_ghost_bit_exact(g):
    got = np.stack([oracle_py.scalar_bc_riemann(f, a, b) for f, a, b in zip(g["faces"], g["ql"], g["qr"])])
    assert np.array_equal(got, g["riemann"])


def gaussian_scalar(n=32, vel=(0.8, -0.5)):
    mesh = Mesh.linspace(n, n, 0.0, 1.0, 0.0, 1.0)
    c = mesh.centres()
    q = np.empty((3, n, n))
    q[0], q[1] = vel
    q[2] = 1.0 + 0.5 * np.exp(-((c[0] - 0.5) ** 2 + (c[1] - 0.5) ** 2) / (2 * 0.08 ** 2))
    return mesh, q


def test_scalar_periodic_conservation_and_velocity():
    mesh, q = gaussian_scalar()
    o = oracle_py.ScalarOracleSolver(mesh.ni, mesh.nj, mesh.nodes.ravel(), ["periodic"] * 4, limiter="vanalbada")
    o.set_state(q)
    o.step(10)
    s = o.get_state()
    assert np.allclose(s[2].sum(), q[2].sum(), rtol=1e-13)
    assert np.array_equal(s[0], q[0]) and np.array_equal(s[1], q[1])


def test_scalar_constant_state_and_transport():
    mesh, q = gaussian_scalar()
    q[2] = 2.0
    o = oracle_py.ScalarOracleSolver(mesh.ni, mesh.nj, mesh.nodes.ravel(), ["periodic"] * 4)
    o.set_state(q)
    o.step(5)
    assert np.abs(o.get_state()[2] - 2.0).max() < 1e-14
    # a bump moves downstream: its centroid follows the velocity
    mesh, q = gaussian_scalar()
    o = oracle_py.ScalarOracleSolver(mesh.ni, mesh.nj, mesh.nodes.ravel(), ["periodic"] * 4, limiter="vanalbada")
    o.set_state(q)
    dt, t = o.step(20)
    c = mesh.centres()
    w0 = q[2] - 1.0
    w1 = o.get_state()[2] - 1.0
    shift = np.array([(w1 * c[k]).sum() / w1.sum() - (w0 * c[k]).sum() / w0.sum() for k in range(2)])
    # oracle time is a quarter of the physical time (cell volume = |J| of the bilinear map)
    assert np.allclose(shift, 4 * t * np.array([0.8, -0.5]), rtol=0.05, atol=2e-3)
