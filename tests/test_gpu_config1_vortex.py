"""The isentropic-vortex configuration as stated: periodic [0,10]^2, 128 x 128 cells,
gamma 1.4, freestream rho = p = 1, (u, v) = (1, 1), strength 5 at (5, 5); Roe, MUSCL
with van Leer (the harmonic-mean slope), LSQ gradients, ssp34 at CFL 0.5 with the
global timestep, FP64, 100 steps (the reference's unsteady 2D driver,
cpp/script/euler/gresho2D.cpp:78-221: ssp34 at :151, periodic sides at :212-215).

Against the CPU oracle: one step restarted from the GPU state at steps 1, 50 and 100
(relative L-inf per conserved variable <= 1e-12), and 100 free-running steps.

Against the exact vortex translated by (t, t), t = 4 * sum(dt) (the reference's cell
volume is a quarter of the quad's area, so its sum of timesteps is a quarter of the
physical time).  The exact solution is the one pin on the restated LSQ / MUSCL / RK
glue that does not share the oracle's reading of it.  It shows a defect of the
reference's RoeDissipation (roeFlux.ipp:40-54): the jump is rotated to the face frame
while the Roe-averaged velocity stays in the global frame, so the dissipation is the
Roe matrix's only for the face normal (1, 0).  With it (HC_FLUX_ROE, kept bit-for-bit
as the reference computes it) the error at 256^2 exceeds the error at 128^2 and 512^2
goes non-physical; with the averaged velocity taken into the face frame
(HC_FLUX_ROE_FACE) the L1 error falls at second order."""
import numpy as np
import pytest

from hyperboliconvergence_gb300 import cases
from hyperboliconvergence_gb300.solver import Mesh, Solver
from oracle import oracle_py

pytestmark = pytest.mark.gpu

N, STEPS = 128, 100
TOL64 = 1e-12
# free-running: 100 steps of round-off-level differences (measured 1.6e-14 with the
# reference's Roe flux, 6.9e-15 with the face-frame one), held to the per-step bar
TOL_FREE = 1e-12


def cons(q, g=1.4):
    u, v, r, p = q
    return np.stack([r * u, r * v, r, p / (g - 1) + 0.5 * r * (u * u + v * v)])


def rel_linf(a, b):
    a, b = cons(a), cons(b)
    num = np.abs(a - b).reshape(4, -1).max(axis=1)
    den = np.abs(b).reshape(4, -1).max(axis=1)
    return float((num / den).max())


def solver(case, flux):
    mesh, bc, ref, q, sp = case
    s = Solver(mesh, bc, ref, flux=flux, limiter="vanleer", rk="ssp34", dt="global", cfl=0.5, species=sp)
    s.set_state(q)
    return s


def oracle(case, flux):
    mesh, bc, ref, q, sp = case
    o = oracle_py.OracleSolver(mesh.ni, mesh.nj, mesh.nodes.ravel(), bc, flux=flux, limiter="vanleer", rk="ssp34",
                               dt="global", cfl=0.5, species=sp)
    o.set_state(q)
    return o


def exact_errors(case, state, t):
    mesh = case[0]
    c = mesh.centres()
    e = np.abs(cons(state) - cons(cases.vortex_state(c[0], c[1], 4.0 * t)))
    return e.reshape(4, -1).mean(axis=1), e.reshape(4, -1).max(axis=1)


@pytest.mark.parametrize("flux", ["roe", "roe_face"])
def test_restart_parity_at_steps_1_50_100(flux):
    case = cases.isentropic_vortex(N)
    s = solver(case, flux)
    states = {0: s.get_state()}
    for k in range(1, STEPS + 1):
        s.step(1)
        if k in (1, 49, 50, 99, 100):
            states[k] = s.get_state()
    for k in (1, 50, 100):
        o = oracle(case, flux)
        o.set_state(states[k - 1])
        o.step(1)
        err = rel_linf(states[k], o.get_state())
        assert err <= TOL64, (flux, k, err)


@pytest.mark.parametrize("flux", ["roe", "roe_face"])
def test_branch_flips_per_step(flux):
    """The parity report's branch-flip count at steps 1, 25, 50, 75 and 100 of the run: the
    GPU and the oracle evaluate the same state (the GPU's at that step); the faces whose
    limiter or flux branches differ.  The vortex's far field is uniform to round-off, so its
    limiter arguments are noise and some may flip; every flip must be at such a round-off
    argument, and the count stays a small fraction of the faces (measured: one face at step 1
    with the reference's Roe flux, none at the other steps or with the face-frame flux)."""
    from hyperboliconvergence_gb300.solver import branch_flips
    case = cases.isentropic_vortex(N)
    s = solver(case, flux)
    counts = {}
    for k in range(1, STEPS + 1):
        s.step(1)
        if k in (1, 25, 50, 75, 100):
            o = oracle(case, flux)
            o.set_state(s.get_state())
            (oi, oj), args = o.face_signatures(with_args=True)
            f = branch_flips(s.face_signatures(), (oi, oj), args=args, limiter="vanleer")
            counts[k] = (f["faces"], f["cells"])
            assert f["faces_above_roundoff"] == 0, (flux, k, f)
            assert f["faces"] <= 0.002 * f["faces_total"], (flux, k, f)
    print(f"{flux}: branch flips (faces, cells) per step {counts}")


@pytest.mark.parametrize("flux", ["roe", "roe_face"])
def test_free_running_100_steps(flux):
    case = cases.isentropic_vortex(N)
    s = solver(case, flux)
    st = s.step(STEPS)
    o = oracle(case, flux)
    dt, t = o.step(STEPS)
    err = rel_linf(s.get_state(), o.get_state())
    print(f"{flux}: free-running relative L-inf after {STEPS} steps {err:.2e}")
    assert err <= TOL_FREE, (flux, err)
    assert abs(st.t - t) <= 1e-13 * t


def test_fp32_against_fp64_after_100_steps():
    """The configuration in FP32 (the face-frame Roe flux) against the same run in FP64: the
    single-precision round-off accumulated over 100 steps stays small against the state's
    scale (relative L-inf <= 1e-4 per conserved variable; 4.4e-6 measured, 8.4e-7 in the
    mean)."""
    mesh, bc, ref, q, sp = cases.isentropic_vortex(N)
    out = {}
    for prec in ("fp32", "fp64"):
        s = Solver(mesh, bc, ref, flux="roe_face", limiter="vanleer", rk="ssp34", dt="global", cfl=0.5,
                   species=sp, precision=prec)
        s.set_state(q)
        s.step(STEPS)
        out[prec] = s.get_state()
    err = rel_linf(out["fp32"], out["fp64"])
    print(f"fp32 vs fp64 after {STEPS} steps: relative L-inf {err:.2e}")
    assert err <= 1e-4, err


def test_exact_vortex_error_literal_roe():
    """The configuration's own comparison: Roe as the reference computes it, 100 steps of
    the 128^2 vortex against the exact translated vortex."""
    case = cases.isentropic_vortex(N)
    s = solver(case, "roe")
    st = s.step(STEPS)
    l1, linf = exact_errors(case, s.get_state(), st.t)
    print(f"roe 128^2, T = {4 * st.t:.4f}: L1 {l1}, Linf {linf}")
    assert l1.max() <= 5e-4 and linf.max() <= 3e-2, (l1, linf)


def test_exact_vortex_second_order_face_frame_roe():
    """64^2 / 128^2 / 256^2 for 50 / 100 / 200 steps (the same physical time to 0.1%): the
    L1 error of every conserved variable falls at second order (>= 1.9; about 2.1
    measured) and L-inf at >= 1.1 (van Leer clips the vortex's extrema)."""
    errs = {}
    for n, steps in ((64, 50), (128, 100), (256, 200)):
        case = cases.isentropic_vortex(n)
        s = solver(case, "roe_face")
        st = s.step(steps)
        errs[n] = exact_errors(case, s.get_state(), st.t)
    for a, b in ((64, 128), (128, 256)):
        o1 = np.log2(errs[a][0] / errs[b][0])
        oi = np.log2(errs[a][1] / errs[b][1])
        print(f"roe_face {a}->{b}: L1 order {o1}, Linf order {oi}")
        assert (o1 >= 1.9).all(), (a, b, o1)
        assert (oi >= 1.1).all(), (a, b, oi)


def test_literal_roe_error_grows_under_refinement():
    """The reference's RoeDissipation, reproduced as written: refining 128^2 -> 256^2 (100 ->
    200 steps) raises the L-inf error instead of lowering it (an instability growing at
    a fixed place near the vortex), where the face-frame flux lowers it."""
    linf = {}
    for flux in ("roe", "roe_face"):
        for n, steps in ((128, 100), (256, 200)):
            case = cases.isentropic_vortex(n)
            s = solver(case, flux)
            st = s.step(steps)
            linf[flux, n] = exact_errors(case, s.get_state(), st.t)[1].max()
    assert linf["roe", 256] > linf["roe", 128], linf
    assert linf["roe_face", 256] < 0.5 * linf["roe_face", 128], linf


def rotated_case(n):
    """The vortex case turned by 90 degrees: nodes (x, y) -> (-y, x), velocities likewise;
    cell (i, j) of the turned mesh is the turned cell (i, j)."""
    mesh, bc, ref, q, sp = cases.isentropic_vortex(n)
    nodes = mesh.nodes
    rn = np.stack([-nodes[..., 1], nodes[..., 0]], axis=-1)
    rq = np.stack([-q[1], q[0], q[2], q[3]])
    return (Mesh(rn), bc, ref, rq, sp), (mesh, bc, ref, q, sp)


@pytest.mark.parametrize("flux,equal", [("roe_face", True), ("roe", False)])
def test_quarter_turn_equivariance(flux, equal):
    """The scheme commutes with turning the problem by 90 degrees when its flux is
    rotation-invariant: the face-frame Roe gives the turned state (<= 1e-12 after 10
    steps); the reference's Roe does not (its dissipation depends on the frame)."""
    rcase, case = rotated_case(64)
    a, b = solver(case, flux), solver(rcase, flux)
    a.step(10)
    b.step(10)
    qa, qb = a.get_state(), b.get_state()
    back = np.stack([qb[1], -qb[0], qb[2], qb[3]])
    err = rel_linf(back, qa)
    if equal:
        assert err <= TOL64, err
    else:
        assert err > 1e-6, err
