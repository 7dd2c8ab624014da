"""The low-Mach flux variants of the CUDA path against the CPU oracle: RoeUnprecWS and
AUSM+up's nine (velocity, pressure) LowMachScaling pairs, each a run-time choice
(hc_set_low_mach) with the species lref and dt that the adaptive scaling reads.

FP64 bar as in test_gpu_parity: residuals within 1e-11 of the face-flux scale,
one RK step <= 1e-12 relative L-inf on the conserved variables.
"""
import numpy as np
import pytest

from hyperboliconvergence_gb300.solver import Solver
from oracle import oracle_py
from test_gpu_parity import CASES, TOL64, prim2cons, rel_linf, residual_scale

pytestmark = pytest.mark.gpu

SCALINGS = ["convective", "acoustic", "adaptive"]
# (lref, dt): the reference default (adaptive ratio 0), and a ratio lref/(as dt) of
# about 0.5 that lies between the cut-off and the local Mach numbers of the cases
LREF_DT = [(1.0, np.finfo(np.float64).max), (0.05, 0.1)]


def pair(case, vs, ps, lref, sdt, precision="fp64", flux="ausmpup", limiter="vanalbada", dt="global", rk="ssp34"):
    mesh, bc, ref, q, species = case
    gpu = Solver(mesh, bc, ref, flux=flux, limiter=limiter, rk=rk, precision=precision, dt=dt,
                 species=species, low_mach=(vs, ps, lref, sdt))
    gpu.set_state(q)
    ora = oracle_py.OracleSolver(mesh.ni, mesh.nj, mesh.nodes.ravel(), bc, flux=flux, limiter=limiter, rk=rk,
                                 dt=dt, species=species, ghost_ref=ref, low_mach=(vs, ps, lref, sdt))
    ora.set_state(q)
    return gpu, ora


def residual_err(gpu, ora):
    rg, ro = gpu.residual(), ora.residual()
    scale = np.maximum(residual_scale(ro), 1e-300)
    err = (np.abs(rg[:4] - ro[:4]).reshape(4, -1).max(axis=1) / scale).max()
    lam = np.abs(rg[4] - ro[4]).max() / np.abs(ro[4]).max()
    return err, lam


@pytest.mark.parametrize("name", ["cylinder", "quadrant"])
@pytest.mark.parametrize("lref_dt", LREF_DT)
@pytest.mark.parametrize("vs", SCALINGS)
@pytest.mark.parametrize("ps", SCALINGS)
def test_ausmpup_scaling_residual_parity(name, lref_dt, vs, ps):
    gpu, ora = pair(CASES[name], vs, ps, *lref_dt)
    err, lam = residual_err(gpu, ora)
    assert err <= 1e-11, err
    assert lam <= 1e-12, lam


def test_adaptive_scaling_changes_the_residual():
    """With lref/(as dt) ~ 0.5 the adaptive pair differs from the convective one (the
    choice reaches the kernel) and the acoustic pair differs from both."""
    case = CASES["cylinder"]
    r = {k: pair(case, k, k, 0.05, 0.1)[0].residual() for k in SCALINGS}
    assert not np.array_equal(r["adaptive"], r["convective"])
    assert not np.array_equal(r["acoustic"], r["adaptive"])


@pytest.mark.parametrize("vs,ps", [("adaptive", "adaptive"), ("acoustic", "convective"), ("convective", "adaptive")])
@pytest.mark.parametrize("dt", ["global", "local"])
def test_ausmpup_scaling_one_step_parity(vs, ps, dt):
    gpu, ora = pair(CASES["cylinder"], vs, ps, 0.05, 0.1, dt=dt)
    st = gpu.step(1)
    dto, _ = ora.step(1)
    assert rel_linf(prim2cons(gpu.get_state()), prim2cons(ora.get_state())) <= TOL64
    assert st.dt == pytest.approx(dto, rel=1e-12)


@pytest.mark.parametrize("vs,ps", [("adaptive", "adaptive"), ("acoustic", "adaptive")])
def test_ausmpup_scaling_df_residual_parity(vs, ps):
    gpu, ora = pair(CASES["quadrant"], vs, ps, 0.05, 0.1, precision="fp64_df")
    err, lam = residual_err(gpu, ora)
    assert err <= 1e-11, err
    assert lam <= 1e-12, lam


def test_ausmpup_scaling_fp32_close():
    gpu, ora = pair(CASES["cylinder"], "adaptive", "adaptive", 0.05, 0.1, precision="fp32")
    err, _ = residual_err(gpu, ora)
    assert err <= 1e-4, err


@pytest.mark.parametrize("name,dt,rk", [("vortex", "global", "ssp34"), ("cylinder", "local", "ssp33"),
                                        ("quadrant", "global", "ssp22")])
def test_roe_ws_one_step_parity(name, dt, rk):
    mesh, bc, ref, q, species = CASES[name]
    gpu = Solver(mesh, bc, ref, flux="roe_ws", limiter="vanleer", rk=rk, dt=dt, species=species)
    gpu.set_state(q)
    ora = oracle_py.OracleSolver(mesh.ni, mesh.nj, mesh.nodes.ravel(), bc, flux="roe_ws", limiter="vanleer",
                                 rk=rk, dt=dt, species=species, ghost_ref=ref)
    ora.set_state(q)
    for _ in range(3):
        st = gpu.step(1)
        dto, _ = ora.step(1)
        assert rel_linf(prim2cons(gpu.get_state()), prim2cons(ora.get_state())) <= TOL64
        assert st.dt == pytest.approx(dto, rel=1e-12)


def test_roe_ws_low_cutoff_mach():
    """RoeUnprecWS's dissipation coefficients scale with the cut-off Mach number;
    parity at minf = 0.05 on the perturbed cylinder state."""
    mesh, bc, ref, q, species = CASES["cylinder"]
    sp = (species[0], species[1], 0.05)
    gpu = Solver(mesh, bc, ref, flux="roe_ws", limiter="minmod", species=sp)
    gpu.set_state(q)
    ora = oracle_py.OracleSolver(mesh.ni, mesh.nj, mesh.nodes.ravel(), bc, flux="roe_ws", limiter="minmod",
                                 species=sp, ghost_ref=ref)
    ora.set_state(q)
    err, lam = residual_err(gpu, ora)
    assert err <= 1e-11, err
    assert lam <= 1e-12, lam


def test_set_low_mach_rejects_bad_arguments():
    mesh, bc, ref, q, species = CASES["vortex"]
    gpu = Solver(mesh, bc, ref, flux="ausmpup", species=species)
    for args in [(3, 0, 1.0, 1.0), (0, -1, 1.0, 1.0), (0, 0, 0.0, 1.0), (0, 0, 1.0, float("inf"))]:
        with pytest.raises(Exception):
            gpu.set_low_mach(*args)
