"""Parity of the double-float stage path (precision "fp64_df": FP64 state and
update, gradients/reconstruction/fluxes in pairs of FP32) with the FP64 oracle,
held to the FP64 bar: relative L-inf error per step on the conserved variables
<= 1e-12, residuals within 1e-11 of the face-flux scale.

The literal reference van Leer ratio (vanleer_ref) is left out: where its
denominator vanishes the result depends on the smallest normal number of the
arithmetic (DBL_MIN in FP64, FLT_MIN here), so the set of non-finite faces is
not the FP64 one.
"""
import numpy as np
import pytest

from hyperboliconvergence_gb300.solver import Solver
from test_gpu_parity import CASES, FLUXES, TOL64, make_pair, prim2cons, rel_linf, residual_scale

pytestmark = pytest.mark.gpu

DF_LIMITERS = ["nolimit1", "nolimit2", "nolimit3", "vanalbada", "minmod", "superbee", "mc", "vanleer", "cada3"]


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("flux", FLUXES)
def test_df_residual_parity_fluxes(name, flux):
    gpu, ora = make_pair(CASES[name], flux=flux, limiter="vanalbada", precision="fp64_df")
    rg, ro = gpu.residual(), ora.residual()
    scale = np.maximum(residual_scale(ro), 1e-300)
    err = (np.abs(rg[:4] - ro[:4]).reshape(4, -1).max(axis=1) / scale).max()
    assert err <= 1e-11, err
    assert np.abs(rg[4] - ro[4]).max() <= 1e-12 * np.abs(ro[4]).max()


@pytest.mark.parametrize("limiter", DF_LIMITERS)
def test_df_residual_parity_limiters(limiter):
    gpu, ora = make_pair(CASES["cylinder"], flux="roe", limiter=limiter, precision="fp64_df")
    rg, ro = gpu.residual(), ora.residual()
    err = (np.abs(rg[:4] - ro[:4]).reshape(4, -1).max(axis=1) / np.maximum(residual_scale(ro), 1e-300)).max()
    assert err <= 1e-11, err


@pytest.mark.parametrize("name,dt", [("vortex", "global"), ("cylinder", "local"), ("quadrant", "global"),
                                     ("cylinder", "global")])
@pytest.mark.parametrize("flux", ["roe", "slau", "ausmpup", "rusanov"])
def test_df_one_step_parity(name, dt, flux):
    gpu, ora = make_pair(CASES[name], flux=flux, limiter="vanalbada", rk="ssp34", dt=dt, precision="fp64_df")
    st = gpu.step(1)
    dto, _ = ora.step(1)
    err = rel_linf(prim2cons(gpu.get_state()), prim2cons(ora.get_state()))
    assert err <= TOL64, err
    assert st.dt == pytest.approx(dto, rel=1e-12)


def test_df_vortex_ten_steps_each_step_parity():
    gpu, ora = make_pair(CASES["vortex"], flux="roe", limiter="vanleer", precision="fp64_df")
    for _ in range(10):
        gpu.set_state(ora.get_state())
        gpu.step(1)
        ora.step(1)
        err = rel_linf(prim2cons(gpu.get_state()), prim2cons(ora.get_state()))
        assert err <= TOL64, err


@pytest.mark.parametrize("flux,limiter", [("roe", "nolimit2"), ("rusanov", "nolimit3")])
def test_df_adjoint_matches_fp64(flux, limiter):
    """Adjoint on a double-float context (forward, replayed and recomputed steps and
    the face reverse in double-float, other reverse passes in FP64) against the
    FP64 context's gradient, for smooth reconstructions.  (With a limiter, faces
    whose arguments sit at round-off level -- zero crossings, exactly uniform
    regions -- can take different branches in the two precisions, and the
    gradient at those cells differs by up to ~1%.)"""
    from test_gpu_adjoint import cylinder_case, make
    case = cylinder_case(nr=12, nth=32, seed=5)
    out = {}
    for prec in ("fp64", "fp64_df"):
        mesh, bc, ref, q = case
        s = Solver(mesh, bc, ref, flux=flux, limiter=limiter, rk="ssp34", precision=prec, dt="global", cfl=0.5,
                   species=(1.4, 287.058, 0.4))
        s.set_state(q)
        J, g, refb, rates, st = s.gradient(8, snapshots=2, kind="drag", scale=2.0)
        out[prec] = (J, g, refb[1])
    (ja, ga, ra), (jb, gb, rb) = out["fp64"], out["fp64_df"]
    assert abs(jb - ja) <= 1e-12 * abs(ja)
    assert np.abs(gb - ga).max() <= 1e-9 * np.abs(ga).max()
    assert np.abs(rb - ra).max() <= 1e-9 * np.abs(ra).max()
