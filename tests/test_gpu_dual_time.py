"""Dual-time stepping (hc_dual_time_run) of the CUDA path against the CPU oracle's
restatement of the same scheme: outer physical steps of BDF1 / BDF2 / the trapezium
rule (ode.h:12-82), inner pseudo-time RK steps of the dual-time residual
g0 R(u) - V (b0 Q(u) + b1 Q_n + b2 Q_{n-1}) / dt + g1 R(u_n) with the pseudo step
dtau / (1 + b0 dtau / dt).  With a fixed inner count the two runs do the same
arithmetic: FP64 bar 1e-12 relative L-inf per conserved variable."""
import numpy as np
import pytest

from hyperboliconvergence_gb300.solver import Solver
from oracle import oracle_py
from test_gpu_parity import CASES, TOL64, make_pair, prim2cons, rel_linf

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,scheme,rk,dt", [("vortex", "bdf2", "ssp34", "local"), ("vortex", "bdf1", "ssp11", "global"),
                                               ("cylinder", "bdf2", "ssp34", "local"),
                                               ("quadrant", "trapezium", "ssp22", "global"),
                                               ("cylinder", "trapezium", "ssp33", "local")])
def test_dual_time_parity(name, scheme, rk, dt):
    gpu, ora = make_pair(CASES[name], flux="roe" if name != "quadrant" else "slau", limiter="vanalbada", rk=rk,
                         dt=dt)
    st = gpu.dual_time(3, cfl_outer=2.0, scheme=scheme, inner_max=6, inner_drop=0.0)
    dto = ora.dual_time(3, cfl_outer=2.0, scheme=scheme, inner=6)
    assert st.dt == pytest.approx(dto, rel=1e-12)
    assert st.outer_steps == 3 and st.inner_steps == 18 and st.t == pytest.approx(3 * dto, rel=1e-12)
    assert rel_linf(prim2cons(gpu.get_state()), prim2cons(ora.get_state())) <= TOL64


def test_dual_time_given_dt_and_fp32():
    gpu, ora = make_pair(CASES["vortex"], flux="roe", limiter="vanleer", dt="local", precision="fp32")
    st = gpu.dual_time(2, dt=0.05, scheme="bdf2", inner_max=5)
    ora.dual_time(2, dt=0.05, scheme="bdf2", inner=5)
    assert st.dt == 0.05
    assert rel_linf(prim2cons(gpu.get_state()), prim2cons(ora.get_state())) <= 1e-4


def test_dual_time_inner_loop_converges():
    """Enough pseudo-time steps drive the dual-time residual down by the requested factor
    and stop the inner loop early."""
    mesh, bc, ref, q, species = CASES["vortex"]
    s = Solver(mesh, bc, ref, flux="roe", limiter="vanalbada", dt="local", cfl=0.8, species=species)
    s.set_state(q)
    st = s.dual_time(2, cfl_outer=1.0, scheme="bdf2", inner_max=400, inner_drop=1e-6, check_every=5)
    assert st.last_inner < 400
    assert st.res_last <= 1e-6 * st.res0_last


def test_converged_dual_time_matches_an_explicit_step():
    """A converged BDF1 step and an explicit RK step of the same physical timestep reach
    the same state to the schemes' time error (implicit Euler's O(dt^2) per step)."""
    mesh, bc, ref, q, species = CASES["vortex"]
    b = Solver(mesh, bc, ref, flux="roe", limiter="vanalbada", dt="global", cfl=0.5, species=species)
    b.set_state(q)
    dt = b.step(1).dt
    a = Solver(mesh, bc, ref, flux="roe", limiter="vanalbada", dt="local", cfl=0.8, species=species)
    a.set_state(q)
    st = a.dual_time(1, dt=dt, scheme="bdf1", inner_max=800, inner_drop=1e-11, check_every=10)
    assert st.res_last <= 1e-11 * st.res0_last
    change = rel_linf(prim2cons(b.get_state()), prim2cons(q))
    err = rel_linf(prim2cons(a.get_state()), prim2cons(b.get_state()))
    assert err <= 0.1 * change, (err, change)


def test_dual_time_conserved_basis_parity():
    from test_gpu_basis import cons_case
    mesh, bc, ref, q, species = cons_case("quadrant")
    gpu = Solver(mesh, bc, ref, flux="slau", limiter="minmod", dt="local", species=species, basis="conserved")
    gpu.set_state(q)
    ora = oracle_py.OracleSolver(mesh.ni, mesh.nj, mesh.nodes.ravel(), bc, flux="slau", limiter="minmod", dt="local",
                                 species=species, ghost_ref=ref, basis="conserved")
    ora.set_state(q)
    gpu.dual_time(2, cfl_outer=1.0, scheme="bdf1", inner_max=4)
    ora.dual_time(2, cfl_outer=1.0, scheme="bdf1", inner=4)
    assert rel_linf(gpu.get_state(), ora.get_state()) <= TOL64


def test_dual_time_rejects_bad_controls():
    mesh, bc, ref, q, species = CASES["vortex"]
    s = Solver(mesh, bc, ref, species=species)
    s.set_state(q)
    with pytest.raises(Exception, match="dual-time"):
        s.dual_time(1, dt=0.0, cfl_outer=0.0)
    with pytest.raises(Exception, match="dual-time"):
        s.dual_time(1, inner_max=0)
