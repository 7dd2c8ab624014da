"""The bench workload at its full size (512 x 1024 cylinder O-grid, Roe + van Albada,
ssp34, local dt, CFL 0.5): FP64 against the CPU oracle (OpenMP) after two RK steps at the
FP64 bar, from the uniform freestream and from a state that is non-uniform everywhere;
FP64 against the double-float path (an independent arithmetic) after three steps; and
mass, momentum and energy conservation on a periodic 1024 x 1024 Gaussian-sum mesh."""
import numpy as np
import pytest

from hyperboliconvergence_gb300 import cases
from hyperboliconvergence_gb300.solver import Solver
from oracle import oracle_py

pytestmark = pytest.mark.gpu

KW = dict(flux="roe", limiter="vanalbada", rk="ssp34", dt="local", cfl=0.5)


def cons(q, g=1.4):
    u, v, r, p = q
    return np.stack([r * u, r * v, r, p / (g - 1) + 0.5 * r * (u * u + v * v)])


def rel(a, b):
    ca, cb = cons(a), cons(b)
    err = np.abs(ca - cb).reshape(4, -1).max(1)
    scale = np.abs(cb).reshape(4, -1).max(1)
    scale[0:2] = scale[0:2].max()  # both momentum components against one momentum scale
    return float((err / scale).max())


def workload(developed):
    mesh, bc, ref, q, sp = cases.cylinder(512, 1024, mach=0.3)
    if developed:
        c = mesh.centres()
        r = np.hypot(c[0], c[1])
        f = np.sin(3.0 * np.arctan2(c[1], c[0])) * np.exp(-0.3 * (r - 0.5)) + 0.2 * np.cos(0.7 * r)
        q = q * (1 + 0.01 * f[None])
    return mesh, bc, ref, q, sp


@pytest.mark.parametrize("developed", [False, True])
def test_full_size_matches_oracle(developed):
    mesh, bc, ref, q, sp = workload(developed)
    s = Solver(mesh, bc, ref, precision="fp64", species=sp, **KW)
    s.set_state(q)
    o = oracle_py.OracleSolver(mesh.ni, mesh.nj, mesh.nodes.ravel(), bc, species=sp, ghost_ref=ref, **KW)
    o.set_state(q)
    for _ in range(2):
        s.step(1)
        o.step(1)
        assert rel(s.get_state(), o.get_state()) <= 1e-12


def test_full_size_fp64_and_double_float_agree():
    mesh, bc, ref, q, sp = workload(True)
    out = []
    for prec in ("fp64", "fp64_df"):
        s = Solver(mesh, bc, ref, precision=prec, species=sp, **KW)
        s.set_state(q)
        s.step(3)
        out.append(s.get_state())
        s.close()
    assert rel(out[1], out[0]) <= 1e-12


def test_full_size_periodic_conservation():
    rng = np.random.default_rng(2026)
    mesh, bc, ref, q, sp = cases.gaussian_sum(1024, 1024, rng)
    s = Solver(mesh, bc, ref, precision="fp64", species=sp, flux="roe", limiter="vanalbada", rk="ssp34",
               dt="global", cfl=0.5)
    s.set_state(q)
    tot0 = cons(q).reshape(4, -1).sum(axis=1)  # uniform cells: the totals are sums of cell values
    s.step(5)
    tot = cons(s.get_state()).reshape(4, -1).sum(axis=1)
    scale = np.abs(cons(q)).reshape(4, -1).sum(axis=1)
    assert np.all(np.abs(tot - tot0) <= 1e-13 * scale), (tot - tot0) / scale
