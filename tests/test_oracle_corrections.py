"""Corrections of two defects of the reference (FIX_*, hc_set_corrections), at the
pointwise level of the oracle.

FIX_MACH_SPLIT_P1: MachSplit_P1 (machSplittings.ipp:26-31) is (M1 + eps)/(|M| + eps)
with eps the largest finite value, which rounds to 1 for both signs.  As written, SLAU and
AUSM+up then add both sides' pressure on a supersonic face and F(q, q) is not the exact
flux; corrected, every flux is consistent.

FIX_FARFIELD_TRANSVERSE: the Riemann and entropy far fields (conservationLaws/euler/boundary/riemann.ipp:48-50,
entropy.ipp:47-49) copy the interior state when u_n/|u| < threshold, a test without the
absolute value, so every outflow face copies the interior; corrected, only transverse
faces do, and a subsonic outflow face takes its acoustic invariant from the far field."""
import numpy as np
import pytest

from oracle import oracle_py

SP = np.array([1.4, 287.058, 0.5])
SLAU, SLAU_REF, AUSMPUP = 1, 2, 3
RIEMANN, ENTROPY = 2, 3


@pytest.fixture(scope="module")
def o():
    return oracle_py.pointwise()


def states(rng, n, mach_max=2.5):
    """Primitive states with normal Mach numbers up to mach_max (sub- and supersonic)."""
    out = []
    for _ in range(n):
        r, p = rng.uniform(0.5, 2.0, 2)
        a = np.sqrt(1.4 * p / r)
        out.append(np.array([rng.uniform(-mach_max, mach_max) * a, rng.uniform(-1, 1) * a, r, p]))
    return out


@pytest.mark.parametrize("kind", [SLAU, SLAU_REF, AUSMPUP])
def test_mach_split_p1_makes_the_fluxes_consistent(o, kind):
    rng = np.random.default_rng(kind)
    worst_fixed, worst_ref, supersonic = 0.0, 0.0, 0
    for q in states(rng, 400):
        th = rng.uniform(-np.pi, np.pi)
        n = np.array([np.cos(th), np.sin(th)])
        face = np.array([1.0, 0.0, 0.0, n[0], n[1], -n[1], n[0]])
        exact = o.exact_flux(SP, n, q)[:4]
        scale = np.abs(exact).max() + q[3]
        fixed = o.flux_fixed(kind, "mach_split_p1", SP, face, q, q)[:4]
        lit = o.flux(kind, SP, face, q, q)[:4]
        assert np.array_equal(lit, o.flux_fixed(kind, 0, SP, face, q, q)[:4])
        worst_fixed = max(worst_fixed, np.abs(fixed - exact).max() / scale)
        a = np.sqrt(1.4 * q[3] / q[2])
        if abs(q[0] * n[0] + q[1] * n[1]) > 1.01 * a:
            supersonic += 1
        worst_ref = max(worst_ref, np.abs(lit - exact).max() / scale)
    assert supersonic > 50
    assert worst_fixed <= 1e-13, worst_fixed
    # as written, a supersonic face's normal momentum flux carries pressure of the wrong side
    assert worst_ref > 0.1, worst_ref


def test_mach_split_p1_leaves_subsonic_faces_alone(o):
    rng = np.random.default_rng(5)
    for q in states(rng, 200, mach_max=0.95):
        for ql in (q, q * np.array([1.05, 0.97, 1.02, 0.99])):
            face = np.array([1.0, 0.0, 0.0, 0.6, 0.8, -0.8, 0.6])
            for kind in (SLAU, SLAU_REF, AUSMPUP):
                if abs(0.6 * ql[0] + 0.8 * ql[1]) < 0.99 * np.sqrt(1.4 * ql[3] / ql[2]) and \
                   abs(0.6 * q[0] + 0.8 * q[1]) < 0.99 * np.sqrt(1.4 * q[3] / q[2]):
                    assert np.array_equal(o.flux(kind, SP, face, ql, q),
                                          o.flux_fixed(kind, "mach_split_p1", SP, face, ql, q))


@pytest.mark.parametrize("kind", [RIEMANN, ENTROPY])
def test_farfield_outflow_faces(o, kind):
    """Normal (1, 0) into the domain; interior and far field moving out (u < 0), subsonic."""
    face = np.array([1.0, 0.0, 0.0, 1.0, 0.0, -0.0, 1.0])
    qi = np.array([-0.3, 0.05, 1.02, 0.98 / 1.4])
    qf = np.array([-0.3, 0.0, 1.0, 1.0 / 1.4])
    lit = o.bc_update(kind, SP, face, qi, qf)
    fixed = o.bc_update_fixed(kind, "farfield_transverse", SP, face, qi, qf)
    assert np.array_equal(lit, qi)           # as written: a copy of the interior
    assert not np.array_equal(fixed, qi)     # corrected: the characteristic update
    # outflow: entropy and tangential velocity from the interior
    assert fixed[1] == qi[1]
    s_i = qi[3] / qi[2] ** 1.4
    s_b = fixed[3] / fixed[2] ** 1.4
    assert abs(s_b - s_i) <= 1e-12 * s_i
    if kind == ENTROPY:  # the pressure of the far field
        assert abs(fixed[3] - qf[3]) <= 1e-14
    # the interior equal to the far field: the update returns it
    same = o.bc_update_fixed(kind, "farfield_transverse", SP, face, qf, qf)
    assert np.allclose(same, qf, rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("kind", [RIEMANN, ENTROPY])
def test_farfield_inflow_and_transverse_faces_unchanged(o, kind):
    face = np.array([1.0, 0.0, 0.0, 1.0, 0.0, -0.0, 1.0])
    qf = np.array([0.3, 0.1, 1.0, 1.0 / 1.4])
    for qi in (np.array([0.31, 0.08, 1.01, 0.99 / 1.4]), np.array([1e-6, 0.4, 1.0, 1.0 / 1.4])):
        assert np.array_equal(o.bc_update(kind, SP, face, qi, qf),
                              o.bc_update_fixed(kind, "farfield_transverse", SP, face, qi, qf))
