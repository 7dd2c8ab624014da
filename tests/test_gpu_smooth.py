"""Residual smoothing of the legacy 1D path on the GPU (hc_smooth_1d) against the oracle
restatement (pinned in test_oracle_smooth by the iterations' closed-form amplification):
bit for bit in FP64, products and sums rounded one by one in the reference's order.  And
the 1D steady driver with use_residual_smoothing: one smoothed forward-Euler step against
the oracle's residual, smoothing and update composed here, and convergence of a smoothed
steady run."""
import numpy as np
import pytest

from hyperboliconvergence_gb300.solver import Mesh1D, Solver
from oracle import oracle_py

pytestmark = pytest.mark.gpu

SP = (1.4, 287.058, 1e-4)


def solver(nc=40, bc=("riemann", "riemann"), cfl=0.5, rk="ssp34", limiter="vanleer", seed=3):
    rng = np.random.default_rng(seed)
    x = np.cumsum(np.concatenate([[0.0], rng.uniform(0.8, 1.2, nc)]))
    c = 0.5 * (x[:-1] + x[1:])
    q = np.stack([0.3 + 0.05 * np.sin(2 * np.pi * c / x[-1]), 1.0 + 0.1 * np.sin(4 * np.pi * c / x[-1] + 0.3),
                  1.0 + 0.05 * np.cos(2 * np.pi * c / x[-1])])
    ref = None if bc[0] == "periodic" else [np.array([0.3, 1.0, 1.0]), np.array([0.3, 1.0, 1.0])]
    s = Solver(Mesh1D(x), list(bc), ref, flux="roe", limiter=limiter, rk=rk, cfl=cfl, species=SP)
    s.set_state(q)
    return s, x, q, ref


@pytest.mark.parametrize("kind", ["implicit", "explicit"])
@pytest.mark.parametrize("ends", ["p", "a", "n"])
@pytest.mark.parametrize("n", [2, 3, 17, 1000, 5003])
def test_smoothing_bit_identical_to_oracle(kind, ends, n):
    s, _, _, _ = solver()
    rng = np.random.default_rng(n)
    r0 = rng.standard_normal((3, n))
    for alpha in (1.0, 1.7, 3.0):
        got = s.smooth_1d(r0, alpha, kind, ends)
        ref = oracle_py.smooth_1d(r0, alpha, kind, ends)
        assert np.array_equal(got, ref), (alpha, np.abs(got - ref).max())


@pytest.mark.parametrize("kind", ["implicit", "explicit"])
@pytest.mark.parametrize("ends", ["p", "a", "n"])
@pytest.mark.parametrize("n", [2, 3, 1000, 300_007])
def test_smoothing_in_place_equals_out_of_place(kind, ends, n):
    """r1 == r0: the explicit kind reads neighbours (and a periodic line's ends) that other
    threads and blocks write, so the library smooths a copy; the result must equal the
    out-of-place one bit for bit, on lines long enough to span many blocks."""
    s, _, _, _ = solver()
    rng = np.random.default_rng(7 + n)
    r0 = rng.standard_normal((3, n))
    for alpha in (1.7, 3.0):
        out = s.smooth_1d(r0, alpha, kind, ends)
        inp = s.smooth_1d(r0, alpha, kind, ends, in_place=True)
        assert np.array_equal(inp, out), (alpha, np.abs(inp - out).max())


def test_smoothing_rejects_bad_arguments():
    s, _, _, _ = solver()
    with pytest.raises(Exception, match="smoothing"):
        s.smooth_1d(np.ones((1, 1)), 2.0)
    with pytest.raises(Exception, match="smoothing"):
        s.smooth_1d(np.ones((1, 8)), -1.0)


def cons1(q, g=1.4):
    u, r, p = q
    return np.stack([r * u, r, p / (g - 1) + 0.5 * r * u * u])


def prim1(c, g=1.4):
    m, r, e = c
    u = m / r
    return np.stack([u, r, (g - 1) * (e - 0.5 * r * u * u)])


def test_smoothed_step_matches_composed_oracle():
    """ssp11 with the global timestep: q1 = prim(cons(q0) + S(R(q0)) dt / V), S the implicit
    smoothing of the three flux planes, dt = cfl / max(lambda / V) of the unsmoothed R."""
    alpha = 2.0
    s, x, q, ref = solver(rk="ssp11", cfl=0.4)
    st, hist = s.steady(1, residual_drop=1e-30, check_every=1, smoothing=alpha)
    got = s.get_state()
    ora = oracle_py.OracleSolver1D(x, ["riemann", "riemann"], flux="roe", limiter="vanleer", rk="ssp11", cfl=0.4,
                                   species=SP, ref=ref)
    ora.set_state(q)
    r = ora.residual()
    vol = np.diff(x)
    dt = 0.4 / np.max(r[3] / vol)
    rs = oracle_py.smooth_1d(r[:3], alpha, "implicit", "a")
    want = prim1(cons1(q) + rs * (dt / vol))
    err = np.abs(cons1(got) - cons1(want)).max(axis=1) / np.abs(cons1(want)).max(axis=1)
    assert err.max() <= 1e-12, err


def test_smoothed_steady_run_converges():
    s, _, q, _ = solver(nc=60, cfl=0.8, limiter="vanalbada")
    st, hist = s.steady(20000, residual_drop=1e-8, check_every=200, smoothing=2.0)
    assert st.converged, (st.steps, st.res / st.res0)
    s2, _, _, _ = solver(nc=60, cfl=0.8, limiter="vanalbada")
    st2, _ = s2.steady(st.steps, residual_drop=1e-30, check_every=st.steps)
    assert not np.array_equal(s.get_state(), s2.get_state())


def test_smoothing_only_on_one_dimensional_contexts():
    from hyperboliconvergence_gb300 import cases
    mesh, bc, ref, q, sp = cases.isentropic_vortex(16)
    s = Solver(mesh, bc, ref, species=sp)
    s.set_state(q)
    with pytest.raises(Exception, match="1D path"):
        s.steady(10, smoothing=2.0)
    s1, _, _, _ = solver()
    with pytest.raises(Exception, match="smoothing factor"):
        s1.steady(10, smoothing=0.5)
