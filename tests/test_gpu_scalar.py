"""Scalar advection law on the GPU (through the C ABI) against the scalar oracle:
residuals within 1e-11 of each variable's flux scale, one RK step within the
FP64 bar (1e-12 relative L-inf per conserved variable), FP32 error bounded,
and conservation on a periodic mesh."""
import numpy as np
import pytest

from hyperboliconvergence_gb300.solver import Mesh, Solver
from oracle import oracle_py

pytestmark = pytest.mark.gpu


def rel_linf(a, b):
    num = np.abs(a - b).reshape(a.shape[0], -1).max(axis=1)
    den = np.abs(b).reshape(b.shape[0], -1).max(axis=1)
    return float((num / np.maximum(den, 1e-300)).max())


def gaussian(mesh, amp=0.5, w=0.1):
    c = mesh.centres()
    return 1.0 + amp * np.exp(-((c[0] - 0.5) ** 2 + (c[1] - 0.5) ** 2) / (2 * w * w))


def cases():
    out = {}
    m = Mesh.linspace(24, 20, 0.0, 1.0, 0.0, 1.0)
    q = np.empty((3, 24, 20)); q[0], q[1] = 0.8, -0.5; q[2] = gaussian(m)
    out["uniform_periodic"] = (m, ["periodic"] * 4, None, q)
    m = Mesh.linspace(20, 28, 0.0, 1.0, 0.0, 1.0)
    c = m.centres()
    q = np.stack([-(c[1] - 0.5), c[0] - 0.5, gaussian(m, 0.8, 0.12)])
    ref = [None, None, np.stack([-(np.linspace(0, 1, 20) - 0.5), np.full(20, -0.5), np.ones(20)]),
           np.stack([-(np.linspace(0, 1, 20) - 0.5), np.full(20, 0.5), np.full(20, 1.2)])]
    out["rotating_riemann"] = (m, ["periodic", "periodic", "riemann", "riemann"], ref, q)
    m = Mesh.cylinder(12, 40, 0.5, 4.0, 1.02)
    c = m.centres()
    q = np.empty((3, 12, 40)); q[0], q[1] = 0.6, 0.3
    q[2] = 1.0 + 0.4 * np.exp(-((c[0] - 1.0) ** 2 + c[1] ** 2))
    ref = [np.stack([np.full(40, 0.6), np.full(40, 0.3), np.full(40, 1.1)]),
           np.stack([np.full(40, 0.6), np.full(40, 0.3), np.full(40, 0.9)]), None, None]
    out["fixed_ogrid"] = (m, ["fixed", "fixed", "periodic", "periodic"], ref, q)
    return out


CASES = cases()


def pair(name, flux="rusanov", limiter="vanalbada", rk="ssp34", dt="global", precision="fp64"):
    mesh, bc, ref, q = CASES[name]
    gpu = Solver(mesh, bc, ref, flux=flux, limiter=limiter, rk=rk, precision=precision, dt=dt, cfl=0.5, law="scalar")
    gpu.set_state(q)
    ora = oracle_py.ScalarOracleSolver(mesh.ni, mesh.nj, mesh.nodes.ravel(), bc, flux=flux, limiter=limiter, rk=rk,
                                       dt=dt, cfl=0.5, ghost_ref=ref)
    ora.set_state(q)
    return gpu, ora


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("flux", ["rusanov", "central"])
@pytest.mark.parametrize("limiter", ["nolimit1", "nolimit3", "vanalbada", "minmod", "vanleer"])
def test_scalar_residual_parity(name, flux, limiter):
    gpu, ora = pair(name, flux, limiter)
    rg, ro = gpu.residual(), ora.residual()
    scale = np.abs(ro[:3]).reshape(3, -1).max(axis=1)
    err = np.abs(rg[:3] - ro[:3]).reshape(3, -1).max(axis=1)
    assert np.all(err <= 1e-11 * np.maximum(scale, scale.max())), (err, scale)
    assert np.abs(rg[3] - ro[3]).max() <= 1e-12 * np.abs(ro[3]).max()


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("rk,dt", [("ssp11", "global"), ("ssp22", "local"), ("ssp33", "global"), ("ssp34", "global"),
                                   ("ssp34", "local")])
def test_scalar_one_step_parity(name, rk, dt):
    gpu, ora = pair(name, rk=rk, dt=dt)
    st = gpu.step(1)
    dto, _ = ora.step(1)
    assert rel_linf(gpu.get_state(), ora.get_state()) <= 1e-12
    if dt == "global":
        assert st.dt == pytest.approx(dto, rel=1e-12)


def test_scalar_ten_steps_and_conservation():
    gpu, ora = pair("uniform_periodic", limiter="vanleer")
    q0 = gpu.get_state()
    for _ in range(10):
        gpu.set_state(ora.get_state())
        gpu.step(1)
        ora.step(1)
        assert rel_linf(gpu.get_state(), ora.get_state()) <= 1e-12
    gpu.set_state(q0)
    gpu.step(20)
    s = gpu.get_state()
    assert abs(s[2].sum() - q0[2].sum()) <= 1e-12 * abs(q0[2].sum())
    assert np.array_equal(s[:2], q0[:2])


def test_scalar_fp32_error():
    gpu, ora = pair("rotating_riemann", precision="fp32")
    gpu.step(5)
    ora.step(5)
    assert rel_linf(gpu.get_state(), ora.get_state()) < 1e-5


def test_scalar_rejects_euler_only_options():
    from hyperboliconvergence_gb300 import HCError
    mesh, bc, ref, q = CASES["uniform_periodic"]
    with pytest.raises(HCError):
        Solver(mesh, bc, ref, flux="roe", law="scalar")
    with pytest.raises(HCError):
        Solver(mesh, ["wall", "wall", "periodic", "periodic"], [None] * 4, flux="rusanov", law="scalar")
