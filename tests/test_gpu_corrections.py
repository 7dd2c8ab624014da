"""The CUDA path with corrections of the reference's defects (hc_set_corrections, and the
face-frame Roe flux HC_FLUX_ROE_FACE) against the oracle with the same corrections, at
the FP64 bar; and what the corrections are for: the isentropic vortex (supersonic faces
in x and y) converges to the exact translated vortex at second order with SLAU and AUSM+up
once MachSplit_P1 is the 1/0 split it is meant to be (as the reference writes it their
error is O(1) at every resolution)."""
import numpy as np
import pytest

from hyperboliconvergence_gb300 import cases
from hyperboliconvergence_gb300.batch import Batch
from hyperboliconvergence_gb300.solver import Solver
from oracle import oracle_py

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
ALL = "all"


def cons(q, g=1.4):
    u, v, r, p = q
    return np.stack([r * u, r * v, r, p / (g - 1) + 0.5 * r * (u * u + v * v)])


def rel_linf(a, b):
    num = np.abs(a - b).reshape(a.shape[0], -1).max(axis=1)
    den = np.abs(b).reshape(b.shape[0], -1).max(axis=1)
    return float((num / np.maximum(den, 1e-300)).max())


def small_cases():
    rng = np.random.default_rng(17)
    vort = cases.isentropic_vortex(24)
    mesh, bc, ref, q, sp = cases.cylinder(12, 40, mach=0.5, rb=6.0)
    q = q * (1 + 0.05 * rng.standard_normal(q.shape))
    q[2:] = np.abs(q[2:])
    cyl = (mesh, bc, ref, q, sp)
    # supersonic far field: faces of both signs of normal Mach number above 1
    mesh, bc, ref, q, sp = cases.cylinder(12, 40, mach=1.6, rb=6.0)
    q = q * (1 + 0.05 * rng.standard_normal(q.shape))
    q[2:] = np.abs(q[2:])
    sup = (mesh, bc, ref, q, sp)
    quad = cases.quadrant_riemann(13, 11, rng)
    return {"vortex": vort, "cylinder": cyl, "supersonic": sup, "quadrant": quad}


CASES = small_cases()


def pair(case, flux, limiter="vanalbada", dt="global", rk="ssp34", corrections=ALL, precision="fp64"):
    mesh, bc, ref, q, sp = case
    g = Solver(mesh, bc, ref, flux=flux, limiter=limiter, rk=rk, dt=dt, cfl=0.5, species=sp, precision=precision,
               corrections=corrections)
    g.set_state(q)
    o = oracle_py.OracleSolver(mesh.ni, mesh.nj, mesh.nodes.ravel(), bc, flux=flux, limiter=limiter, rk=rk, dt=dt,
                               cfl=0.5, species=sp, ghost_ref=ref, corrections=corrections)
    o.set_state(q)
    return g, o


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("flux", ["slau", "slau_ref", "ausmpup", "roe_face", "roe"])
def test_residual_parity_with_corrections(name, flux):
    g, o = pair(CASES[name], flux)
    rg, ro = g.residual(), o.residual()
    scale = np.maximum(np.abs(ro[:4]).reshape(4, -1).max(axis=1), 1e-300)
    err = (np.abs(rg[:4] - ro[:4]).reshape(4, -1).max(axis=1) / scale).max()
    assert err <= 1e-11, err
    assert np.abs(rg[4] - ro[4]).max() <= 1e-12 * np.abs(ro[4]).max()


@pytest.mark.parametrize("name,dt", [("vortex", "global"), ("cylinder", "local"), ("supersonic", "local"),
                                     ("quadrant", "global")])
@pytest.mark.parametrize("flux", ["slau", "ausmpup", "roe_face"])
def test_three_steps_parity_with_corrections(name, dt, flux):
    g, o = pair(CASES[name], flux, dt=dt)
    for _ in range(3):
        g.set_state(o.get_state())
        g.step(1)
        o.step(1)
        err = rel_linf(cons(g.get_state()), cons(o.get_state()))
        assert err <= TOL64, (name, flux, err)


def test_corrections_change_the_results_where_they_apply():
    """P1 changes supersonic faces of SLAU/AUSM+up; the far-field test changes outflow faces;
    neither touches the literal paths (mask 0 equals the default bit for bit)."""
    for name, flux, mask in (("supersonic", "ausmpup", "mach_split_p1"), ("cylinder", "roe", "farfield_transverse")):
        mesh, bc, ref, q, sp = CASES[name]
        outs = {}
        for m in (None, 0, mask):
            g = Solver(mesh, bc, ref, flux=flux, limiter="vanalbada", dt="local", species=sp, corrections=m)
            g.set_state(q)
            outs[m] = g.residual()
        assert np.array_equal(outs[None], outs[0])
        assert not np.array_equal(outs[None], outs[mask])


def test_corrections_rejects_unknown_bits():
    mesh, bc, ref, q, sp = CASES["vortex"]
    g = Solver(mesh, bc, ref, species=sp)
    with pytest.raises(Exception, match="correction"):
        g.set_corrections(8)


@pytest.mark.parametrize("flux", ["slau", "ausmpup"])
def test_vortex_second_order_with_mach_split_fix(flux):
    """The 64^2 / 128^2 / 256^2 vortex (50 / 100 / 200 steps, van Leer, ssp34, CFL 0.5):
    corrected, the L1 error falls at second order; as written it is O(1e-2) at 64^2 and
    does not fall."""
    errs, lit = {}, {}
    for n, steps in ((64, 50), (128, 100), (256, 200)):
        mesh, bc, ref, q, sp = cases.isentropic_vortex(n)
        c = mesh.centres()
        for m, store in ((ALL, errs), (None, lit)):
            if m is None and n > 128:
                continue
            g = Solver(mesh, bc, ref, flux=flux, limiter="vanleer", rk="ssp34", dt="global", cfl=0.5, species=sp,
                       corrections=m)
            g.set_state(q)
            st = g.step(steps)
            e = np.abs(cons(g.get_state()) - cons(cases.vortex_state(c[0], c[1], 4.0 * st.t)))
            store[n] = e.reshape(4, -1).mean(axis=1)
    for a, b in ((64, 128), (128, 256)):
        order = np.log2(errs[a] / errs[b])
        print(f"{flux} {a}->{b}: L1 order {order}")
        assert (order >= 1.8).all(), (a, b, order)
    assert lit[64].max() > 10 * errs[64].max() and lit[128].max() > 0.5 * lit[64].max(), (lit, errs)


def test_fp32_with_corrections_against_fp64_oracle():
    g, o = pair(CASES["supersonic"], "ausmpup", dt="local", precision="fp32")
    g.step(3)
    o.step(3)
    assert rel_linf(cons(g.get_state()), cons(o.get_state())) < 1e-4


def test_batch_with_corrections_equals_single_mesh():
    rng = np.random.default_rng(3)
    insts = []
    for n in (24, 40):
        mesh, bc, ref, q, sp = cases.quadrant_riemann(n, n + 8, rng)
        insts.append((mesh, bc, ref, q))
    b = Batch(insts, flux="ausmpup", limiter="vanalbada", precision="fp64", species=sp, corrections=ALL)
    b.step_async(4)
    b.sync()
    for k, (mesh, bc, ref, q) in enumerate(insts):
        g = Solver(mesh, bc, ref, flux="ausmpup", limiter="vanalbada", precision="fp64", cfl=0.5, species=sp,
                   corrections=ALL)
        g.set_state(q)
        g.step(4)
        assert np.array_equal(b.get_state(k), g.get_state()), k
