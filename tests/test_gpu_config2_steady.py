"""The steady cylinder configuration: flow past a cylinder on an O-grid (radius 0.5 to 20,
radial stretching 1.01, inviscid wall, Riemann far field, periodic in theta), freestream
M 0.3, local timestepping with ssp34, run from the uniform freestream until the density
residual fell by 1e-10 -- on a 64 x 128 O-grid, where that takes tens of thousands of
steps (the 512 x 1024 grid of the benchmark needs far more; its capped runs are reported
by bench.py's steady extra).

The run uses the corrections of the reference's defects: the face-frame Roe flux and the
far field's outflow test (without the latter the outflow faces copy the interior and the
residual does not converge), and an unlimited reconstruction (NoLimit2; van Albada stalls
near a 1e-4 drop, as limited schemes do on steady problems).  Checked: convergence to
1e-10; the converged state is a steady state of the oracle's discretisation too (its
oracle residual fell by 1e-9) and one more step matches the oracle's step at the FP64 bar;
the lift vanishes by symmetry; FP32 against the FP64 converged state."""
import numpy as np
import pytest

from hyperboliconvergence_gb300 import cases
from hyperboliconvergence_gb300.solver import Solver
from oracle import oracle_py

pytestmark = pytest.mark.gpu

NR, NTH, MACH = 64, 128, 0.3
KW = dict(flux="roe_face", limiter="nolimit2", rk="ssp34", dt="local", cfl=1.5)


def cons(q, g=1.4):
    u, v, r, p = q
    return np.stack([r * u, r * v, r, p / (g - 1) + 0.5 * r * (u * u + v * v)])


@pytest.fixture(scope="module")
def converged():
    mesh, bc, ref, q, sp = cases.cylinder(NR, NTH, mach=MACH)
    s = Solver(mesh, bc, ref, species=sp, corrections="all", **KW)
    s.set_state(q)
    st, hist = s.steady(60000, residual_drop=1e-10, check_every=1000)
    return (mesh, bc, ref, q, sp), s, st, hist


def test_converges_to_1e10(converged):
    _, s, st, hist = converged
    print(f"converged in {st.steps} steps, drop {st.res / st.res0:.2e}")
    assert st.converged and st.res <= 1e-10 * st.res0


def test_converged_state_is_the_oracles_steady_state(converged):
    (mesh, bc, ref, q, sp), s, st, _ = converged
    o = oracle_py.OracleSolver(NR, NTH, mesh.nodes.ravel(), bc, species=sp, ghost_ref=ref, corrections="all", **KW)
    o.set_state(q)
    r0 = np.sqrt((o.residual()[2] ** 2).sum())
    qc = s.get_state()
    o.set_state(qc)
    r1 = np.sqrt((o.residual()[2] ** 2).sum())
    assert r1 <= 1e-9 * r0, r1 / r0
    # one more step from the converged state: GPU and oracle agree at the FP64 bar
    s.set_state(qc)
    s.step(1)
    o.step(1)
    a, b = cons(s.get_state()), cons(o.get_state())
    err = (np.abs(a - b).reshape(4, -1).max(1) / np.abs(b).reshape(4, -1).max(1)).max()
    assert err <= 1e-12, err


def test_lift_vanishes_by_symmetry(converged):
    _, s, st, _ = converged
    q = 0.5 * MACH * MACH  # rho U^2 / 2 with rho = 1, U = M (unit speed of sound); length 2 r_c = 1
    cd = s.wall_force((1.0, 0.0)) / q
    cl = s.wall_force((0.0, 1.0)) / q
    print(f"C_d {cd:.6e}, C_l {cl:.3e}")
    assert np.isfinite(cd) and abs(cl) <= 1e-8 * max(1.0, abs(cd))


def test_fp32_against_the_fp64_converged_state(converged):
    (mesh, bc, ref, q, sp), s64, _, _ = converged
    s = Solver(mesh, bc, ref, species=sp, corrections="all", precision="fp32", **KW)
    s.set_state(q)
    st, _ = s.steady(60000, residual_drop=1e-10, check_every=1000)
    a, b = cons(s.get_state()), cons(s64.get_state())
    d = np.abs(a - b).reshape(4, -1)
    scale = np.abs(b).reshape(4, -1).max(1)
    linf = (d.max(1) / scale).max()
    l1 = (d.mean(1) / scale).max()
    print(f"FP32: residual drop {st.res / st.res0:.2e} after {st.steps} steps; difference from the FP64 converged "
          f"state relative to each variable's largest magnitude: L-inf {linf:.2e}, mean {l1:.2e}")
    assert st.res <= 1e-3 * st.res0
    assert linf <= 2e-4 and l1 <= 1e-4


def test_without_the_farfield_correction_the_residual_stalls(converged):
    """The reference's far field as written (outflow faces copy the interior): the same run
    ends far from converged, where the corrected one reached 1e-10."""
    (mesh, bc, ref, q, sp), _, st_c, _ = converged
    s = Solver(mesh, bc, ref, species=sp, corrections="mach_split_p1", **KW)
    s.set_state(q)
    st, _ = s.steady(st_c.steps, residual_drop=1e-10, check_every=1000)
    print(f"uncorrected far field: drop {st.res / st.res0:.2e} after {st.steps} steps")
    assert not st.converged and st.res >= 1e3 * 1e-10 * st.res0
