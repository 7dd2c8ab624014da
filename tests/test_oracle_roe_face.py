"""The face-frame Roe flux (flux kind 7, HC_FLUX_ROE_FACE) against the reference's Roe
flux (kind 0, pinned bit for bit to the reference's own RoeFlux by the golden vectors).

The reference's RoeDissipation (conservationLaws/base/fluxes/roeFlux.ipp:40-54) rotates
the jump of conserved variables to the face frame but passes the Roe-averaged state,
whose velocity is in the global frame, to the characteristic transforms.  The result is
the Roe matrix's dissipation only when the face frame is the global frame (normal
(1, 0)).  Kind 7 takes the averaged velocity into the face frame; it must

* equal kind 0 bit for bit for the normal (1, 0), on the golden face states;
* be invariant under rotation: F(n; qL, qR) = R^T F((1, 0); R qL, R qR);

while kind 0 is not invariant (the defect this variant removes)."""
import os

import numpy as np
import pytest

from oracle import oracle_py

GOLD = os.path.join(os.path.dirname(__file__), "golden", "pointwise_golden.npz")
SP = np.array([1.4, 287.058, 0.3])


def turn(q, c, s):
    """Velocity components in the frame whose first axis is (c, s)."""
    u, v, r, p = q
    return np.array([c * u + s * v, -s * u + c * v, r, p])


def unturn(f, c, s):
    return np.array([c * f[0] - s * f[1], s * f[0] + c * f[1], f[2], f[3], f[4]])


@pytest.fixture(scope="module")
def o():
    return oracle_py.pointwise()


def test_equals_reference_roe_for_the_unit_x_normal(o):
    g = np.load(GOLD)
    face = np.array([1.3, 0.2, -0.4, 1.0, 0.0, -0.0, 1.0])
    for ql, qr in zip(g["flux_ql"], g["flux_qr"]):
        assert np.array_equal(o.flux(7, SP, face, ql, qr), o.flux(0, SP, face, ql, qr), equal_nan=True)
    ref = oracle_py.reference_pointwise()
    if ref is not None:  # the reference's own RoeFlux, where its probe was built here
        for ql, qr in zip(g["flux_ql"], g["flux_qr"]):
            assert np.array_equal(o.flux(7, SP, face, ql, qr), ref.flux(0, SP, face, ql, qr), equal_nan=True)


@pytest.mark.parametrize("theta", [np.pi / 2, np.pi, -np.pi / 2, 0.3, 1.0, -2.2])
def test_rotation_invariance(o, theta):
    rng = np.random.default_rng(11)
    c, s = np.cos(theta), np.sin(theta)
    face = np.array([1.0, 0.0, 0.0, c, s, -s, c])
    fx = np.array([1.0, 0.0, 0.0, 1.0, 0.0, -0.0, 1.0])
    worst_face, worst_ref = 0.0, 0.0
    for _ in range(300):
        ql = np.array([*rng.uniform(-1, 1, 2), *rng.uniform(0.5, 2, 2)])
        qr = np.array([*rng.uniform(-1, 1, 2), *rng.uniform(0.5, 2, 2)])
        for kind in (7, 0):
            f = o.flux(kind, SP, face, ql, qr)
            g = unturn(o.flux(kind, SP, fx, turn(ql, c, s), turn(qr, c, s)), c, s)
            d = np.abs(f - g).max() / np.abs(f).max()
            if kind == 7:
                worst_face = max(worst_face, d)
            else:
                worst_ref = max(worst_ref, d)
    assert worst_face <= 1e-14, worst_face
    assert worst_ref > 1e-3, worst_ref
