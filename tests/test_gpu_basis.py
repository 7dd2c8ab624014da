"""The conserved solution basis (HC_BASIS_CONSERVED) of the CUDA path against the CPU
oracle run in the same basis: state, ghost reference layers, gradients, limiting and
reconstruction in {rho u, rho v, rho, rho E}; fluxes through set2State of the
conserved set; the RK update on the conserved set directly.

FP64 bar as in test_gpu_parity: residuals within 1e-11 of the face-flux scale, one
RK step <= 1e-12 relative L-inf per conserved variable.
"""
import numpy as np
import pytest

from hyperboliconvergence_gb300.batch import Batch
from hyperboliconvergence_gb300.solver import Solver
from oracle import oracle_py
from test_gpu_parity import CASES, GAMMA, TOL64, rel_linf, residual_scale

pytestmark = pytest.mark.gpu


def to_cons(q, gamma=GAMMA):
    u, v, r, p = q
    return np.stack([r * u, r * v, r, p / (gamma - 1) + 0.5 * r * (u * u + v * v)])


def cons_case(name):
    mesh, bc, ref, q, species = CASES[name]
    cref = None if ref is None else [None if r is None else to_cons(np.asarray(r)) for r in ref]
    return mesh, bc, cref, to_cons(q), species


def pair(name, flux="roe", limiter="vanalbada", rk="ssp34", dt="global", precision="fp64"):
    mesh, bc, ref, q, species = cons_case(name)
    gpu = Solver(mesh, bc, ref, flux=flux, limiter=limiter, rk=rk, precision=precision, dt=dt, species=species,
                 basis="conserved")
    gpu.set_state(q)
    ora = oracle_py.OracleSolver(mesh.ni, mesh.nj, mesh.nodes.ravel(), bc, flux=flux, limiter=limiter, rk=rk,
                                 dt=dt, species=species, ghost_ref=ref, basis="conserved")
    ora.set_state(q)
    return gpu, ora


def residual_err(gpu, ora):
    rg, ro = gpu.residual(), ora.residual()
    scale = np.maximum(residual_scale(ro), 1e-300)
    err = (np.abs(rg[:4] - ro[:4]).reshape(4, -1).max(axis=1) / scale).max()
    lam = np.abs(rg[4] - ro[4]).max() / np.abs(ro[4]).max()
    return err, lam


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("flux", ["roe", "slau", "ausmpup", "rusanov", "roe_ws"])
def test_conserved_residual_parity_fluxes(name, flux):
    err, lam = residual_err(*pair(name, flux=flux))
    assert err <= 1e-11, err
    assert lam <= 1e-12, lam


@pytest.mark.parametrize("limiter", ["nolimit1", "nolimit3", "minmod", "superbee", "mc", "vanleer", "cada3"])
def test_conserved_residual_parity_limiters(limiter):
    err, lam = residual_err(*pair("cylinder", limiter=limiter))
    assert err <= 1e-11, err
    assert lam <= 1e-12, lam


@pytest.mark.parametrize("name,dt,rk", [("vortex", "global", "ssp34"), ("cylinder", "local", "ssp34"),
                                        ("quadrant", "global", "ssp22"), ("cylinder", "global", "ssp33")])
def test_conserved_step_parity(name, dt, rk):
    gpu, ora = pair(name, rk=rk, dt=dt, flux="roe" if name != "quadrant" else "slau", limiter="vanleer")
    for _ in range(3):
        st = gpu.step(1)
        dto, _ = ora.step(1)
        assert rel_linf(gpu.get_state(), ora.get_state()) <= TOL64
        assert st.dt == pytest.approx(dto, rel=1e-12)


@pytest.mark.parametrize("name", ["cylinder", "quadrant"])
def test_conserved_df_residual_parity(name):
    err, lam = residual_err(*pair(name, precision="fp64_df"))
    assert err <= 1e-11, err
    assert lam <= 1e-12, lam


def test_conserved_fp32_close():
    gpu, ora = pair("vortex", precision="fp32")
    for _ in range(5):
        gpu.step(1)
        ora.step(1)
    assert rel_linf(gpu.get_state(), ora.get_state()) <= 1e-4


def test_bases_differ_but_both_conserve():
    """Reconstructing conserved instead of primitive variables changes the face states
    (so the residual differs) while a periodic run conserves the totals in both."""
    mesh, bc, ref, q, species = CASES["vortex"]
    prim = Solver(mesh, bc, ref, flux="roe", limiter="vanleer", species=species)
    prim.set_state(q)
    cons = Solver(mesh, bc, ref, flux="roe", limiter="vanleer", species=species, basis="conserved")
    cons.set_state(to_cons(q))
    assert not np.allclose(prim.residual()[:4], cons.residual()[:4], rtol=0, atol=1e-13)
    # the vortex mesh is uniform: the totals are sums of the cell values
    tot0 = to_cons(q).reshape(4, -1).sum(axis=1)
    cons.step(5)
    prim.step(5)
    tot_c = cons.get_state().reshape(4, -1).sum(axis=1)
    tot_p = to_cons(prim.get_state()).reshape(4, -1).sum(axis=1)
    assert np.allclose(tot_c, tot0, rtol=1e-12, atol=1e-11)
    assert np.allclose(tot_p, tot0, rtol=1e-12, atol=1e-11)


def test_conserved_batch_equals_single_contexts():
    names = ["quadrant", "vortex"]
    insts = [cons_case(n)[:4] for n in names]
    bt = Batch(insts, flux="roe", limiter="vanleer", precision="fp64", species=(GAMMA, 287.058, 0.5),
               basis="conserved")
    bt.step_async(2)
    bt.sync()
    for k, (mesh, bc, ref, q) in enumerate(insts):
        s = Solver(mesh, bc, ref, flux="roe", limiter="vanleer", species=(GAMMA, 287.058, 0.5), basis="conserved")
        s.set_state(q)
        s.step(2)
        assert np.array_equal(s.get_state(), bt.get_state(k))


def test_conserved_basis_rejected_where_unsupported():
    mesh, bc, ref, q, species = cons_case("vortex")
    s = Solver(mesh, bc, ref, flux="roe", limiter="vanalbada", species=species, basis="conserved")
    s.set_state(q)
    with pytest.raises(Exception, match="primitive basis"):
        s.gradient(2, kind="l2", target=q)
    with pytest.raises(Exception, match="one basis"):
        Solver(mesh, ["periodic"] * 4, None, flux="rusanov", limiter="nolimit3", law="scalar", basis="conserved")
