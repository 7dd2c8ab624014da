"""Residual smoothing of the reference's legacy 1D path, restated in the oracle
(oracle/hc_oracle_smooth.hpp; OLD.fieldOperations/centralImplicitSmoothing.ipp and
centralExplicitSmoothing.ipp).  The reference's headers for these functions are absent
from its tree, so the restatement is pinned by closed forms that follow from the
reference's iterations on periodic sinusoids of wavenumber k on n points (theta =
2 pi k / n):
  explicit: r1 = r0 (1 + 4 gamma sin^2(theta/2)), the amplification the reference's own
            smoothing test (script/test/testSmooth.cpp) writes as `ampe`;
  implicit: four weighted-Jacobi sweeps w <- a w + b from w = 1, a = (1 - omega) +
            omega 2 beta cos(theta) / (1 + 2 beta), b = omega / (1 + 2 beta), omega = 2/3,
            then times alpha.
"""
import numpy as np
import pytest

from oracle import oracle_py


def modes(n, ks):
    x = np.arange(n) / n
    return np.stack([np.sin(2 * np.pi * k * x + 0.3) for k in ks])


@pytest.mark.parametrize("alpha", [1.5, 2.0, 3.0])
def test_explicit_smoothing_amplification(alpha):
    n, ks = 64, [1, 3, 8, 17, 31]
    r0 = modes(n, ks)
    r1 = oracle_py.smooth_1d(r0, alpha, "explicit", "p")
    beta = 0.25 * (alpha * alpha - 1.0)
    gamma = 0.25 * ((1.0 + 4.0 * beta) / alpha - 1.0)
    for row, k in enumerate(ks):
        th = 2 * np.pi * k / n
        amp = 1.0 + 4.0 * gamma * np.sin(0.5 * th) ** 2
        assert np.allclose(r1[row], amp * r0[row], rtol=0, atol=1e-13)


@pytest.mark.parametrize("alpha", [1.5, 2.0, 3.0])
def test_implicit_smoothing_amplification(alpha):
    n, ks = 64, [1, 3, 8, 17, 31]
    r0 = modes(n, ks)
    r1 = oracle_py.smooth_1d(r0, alpha, "implicit", "p")
    beta = 0.25 * (alpha * alpha - 1.0)
    omega = 2.0 / 3.0
    for row, k in enumerate(ks):
        th = 2 * np.pi * k / n
        a = (1 - omega) + omega * 2 * beta * np.cos(th) / (1 + 2 * beta)
        b = omega / (1 + 2 * beta)
        w = 1.0
        for _ in range(4):
            w = a * w + b
        assert np.allclose(r1[row], alpha * w * r0[row], rtol=0, atol=1e-13)


def test_smoothing_ends():
    """A constant line: explicit smoothing leaves it; implicit with one-neighbour ('a') or
    periodic ends returns alpha times it; with unscaled ends the end values grow."""
    r0 = np.full((1, 20), 2.5)
    for ends in ("a", "p", "n"):
        assert np.allclose(oracle_py.smooth_1d(r0, 2.0, "explicit", ends), r0, rtol=0, atol=1e-15)
    for ends in ("a", "p"):
        assert np.allclose(oracle_py.smooth_1d(r0, 2.0, "implicit", ends), 2.0 * r0, rtol=1e-15, atol=0)
    un = oracle_py.smooth_1d(r0, 2.0, "implicit", "n")[0]
    assert np.allclose(un[1:-1][3:-3], 5.0) and un[0] > 5.0 and un[-1] > 5.0


def test_planted_change_is_detected():
    """The closed form rejects a restatement with one sweep fewer (computed here from the
    oracle's own sweeps on a shorter recurrence)."""
    n, k, alpha = 64, 5, 2.0
    r0 = modes(n, [k])
    r1 = oracle_py.smooth_1d(r0, alpha, "implicit", "p")[0]
    beta, omega, th = 0.25 * (alpha * alpha - 1.0), 2.0 / 3.0, 2 * np.pi * k / n
    a = (1 - omega) + omega * 2 * beta * np.cos(th) / (1 + 2 * beta)
    b = omega / (1 + 2 * beta)
    w3 = 1.0
    for _ in range(3):
        w3 = a * w3 + b
    assert not np.allclose(r1, alpha * w3 * r0[0], rtol=0, atol=1e-6)
