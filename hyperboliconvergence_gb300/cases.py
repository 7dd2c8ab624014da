"""Seeded synthetic workloads of the residual-and-timestep path.

The reference publishes no dataset; these generators stand in for the
workloads of its drivers (cpp/script/euler/gresho2D.cpp, cylinder2D.cpp):

* isentropic vortex on a periodic Cartesian mesh;
* steady flow past a cylinder on a stretched O-grid (wall, far field, periodic);
* four-quadrant Riemann problems with fixed ghost states;
* sums of Gaussians over a uniform base state.

All return primitive states {u, v, rho, p} as arrays of shape (4, ni, nj).
"""
from __future__ import annotations

import math

import numpy as np

from .solver import Mesh

GAMMA = 1.4
R_AIR = 287.058  # get_air_species (conservationLaws/euler/species.ipp:1-17)


def vortex_state(x, y, t=0.0, gamma=GAMMA, beta=5.0, centre=(5.0, 5.0), uinf=(1.0, 1.0), period=10.0):
    """Isentropic vortex advected by (uinf) for time t on a periodic box."""
    xc = (x - uinf[0] * t - centre[0] + period / 2) % period - period / 2
    yc = (y - uinf[1] * t - centre[1] + period / 2) % period - period / 2
    r2 = xc * xc + yc * yc
    e = np.exp(0.5 * (1.0 - r2))
    du = -beta / (2 * math.pi) * yc * e
    dv = beta / (2 * math.pi) * xc * e
    T = 1.0 - (gamma - 1.0) * beta * beta / (8.0 * gamma * math.pi ** 2) * np.exp(1.0 - r2)
    rho = T ** (1.0 / (gamma - 1.0))
    p = rho ** gamma
    return np.stack([uinf[0] + du, uinf[1] + dv, rho, p])


def isentropic_vortex(n: int = 128):
    """2D isentropic vortex, periodic [0,10]^2, n x n cells, (u,v)=(1,1), strength 5."""
    mesh = Mesh.linspace(n, n, 0.0, 10.0, 0.0, 10.0)
    c = mesh.centres()
    q = vortex_state(c[0], c[1])
    species = (GAMMA, R_AIR, math.sqrt(2.0) / math.sqrt(GAMMA))
    return mesh, ["periodic"] * 4, None, q, species


def cylinder(nr: int = 512, nth: int = 1024, mach: float = 0.3, rc: float = 0.5, rb: float = 20.0,
             stretch: float = 1.01, far="riemann"):
    """Steady cylinder flow: wall at i=0, far field at i=nr, periodic in theta.

    Freestream rho=1, p=1/gamma (unit speed of sound), velocity (mach, 0); the
    state starts uniform at the freestream.
    """
    mesh = Mesh.cylinder(nr, nth, rc, rb, stretch)
    qinf = np.array([mach, 0.0, 1.0, 1.0 / GAMMA])
    q = np.broadcast_to(qinf[:, None, None], (4, nr, nth)).copy()
    ref = [None, np.broadcast_to(qinf[:, None], (4, nth)).copy(), None, None]
    species = (GAMMA, R_AIR, mach)
    return mesh, ["wall", far, "periodic", "periodic"], ref, q, species


def _opens_vacuum(quad, gamma=GAMMA, margin=0.2):
    """True when a quadrant interface separates faster than `margin` times the
    vacuum-formation speed 2(a_L + a_R)/(gamma - 1) of its 1D Riemann problem."""
    a = np.sqrt(gamma * quad[:, 3] / quad[:, 2])
    lim = lambda l, r: margin * 2.0 * (a[l] + a[r]) / (gamma - 1.0)  # noqa: E731
    # quadrant k = 2*(x >= 0.5) + (y >= 0.5)
    for lo, hi, comp in ((0, 2, 0), (1, 3, 0), (0, 1, 1), (2, 3, 1)):
        if quad[hi, comp] - quad[lo, comp] >= lim(lo, hi):
            return True
    return False


def quadrant_riemann(ni: int, nj: int, rng: np.random.Generator):
    """Four-quadrant Riemann problem on [0,1]^2 split at (0.5, 0.5), fixed ghost states.

    Quadrant states: rho in [0.5, 2], p in [0.1, 2], |u|, |v| <= 1 (uniform draws);
    draws whose interfaces separate faster than a fifth of the 1D vacuum-formation
    speed are redrawn: where the four rarefactions meet at the centre the 2D
    expansion is stronger than any 1D one, and at half that speed MUSCL schemes
    (the CPU oracle in FP64 included) drive the pressure negative within a few
    steps.  With this bound the 256-instance batch of seed 2026 stays physical
    for 15 SLAU/van Albada ssp34 steps at CFL 0.5 in the oracle.
    """
    mesh = Mesh.linspace(ni, nj, 0.0, 1.0, 0.0, 1.0)
    quad = np.empty((4, 4))  # quadrant x (u, v, rho, p)
    while True:
        quad[:, 2] = rng.uniform(0.5, 2.0, 4)
        quad[:, 3] = rng.uniform(0.1, 2.0, 4)
        quad[:, 0:2] = rng.uniform(-1.0, 1.0, (4, 2))
        if not _opens_vacuum(quad):
            break
    c = mesh.centres()
    qi = (c[0] >= 0.5).astype(int)
    qj = (c[1] >= 0.5).astype(int)
    k = qi * 2 + qj
    q = np.moveaxis(quad[k], 2, 0).copy()
    # ghost reference = initial state of the adjacent cells (make_fixed_BCond)
    ref = [q[:, 0, :].copy(), q[:, -1, :].copy(), q[:, :, 0].copy(), q[:, :, -1].copy()]
    return mesh, ["fixed"] * 4, ref, q, (GAMMA, R_AIR, 0.5)


def gaussian_sum(ni: int, nj: int, rng: np.random.Generator, base=(0.5, 0.25, 5.0, 1.0), nbumps: int = 8):
    """Uniform base state plus 8 seeded Gaussians added to the density."""
    mesh = Mesh.linspace(ni, nj, 0.0, 1.0, 0.0, 1.0)
    c = mesh.centres()
    q = np.broadcast_to(np.asarray(base, dtype=np.float64)[:, None, None], (4, ni, nj)).copy()
    for _ in range(nbumps):
        cx, cy = rng.uniform(0, 1, 2)
        w = rng.uniform(0.02, 0.2)
        amp = rng.uniform(-0.5, 0.5)
        q[2] += amp * np.exp(-((c[0] - cx) ** 2 + (c[1] - cy) ** 2) / (2 * w * w))
    return mesh, ["periodic"] * 4, None, q, (GAMMA, R_AIR, 0.3)


def scalar_gaussian_sum(ni: int, nj: int, rng: np.random.Generator, velocity=(0.8, -0.5), base: float = 1.0,
                        nbumps: int = 8):
    """Scalar advection on the periodic unit square: a constant velocity and a scalar of
    `base` plus 8 seeded Gaussians (centres in the domain, widths in [0.02, 0.2],
    amplitudes in [-0.5, 0.5]); states {u, v, q}."""
    mesh = Mesh.linspace(ni, nj, 0.0, 1.0, 0.0, 1.0)
    c = mesh.centres()
    q = np.empty((3, ni, nj))
    q[0], q[1], q[2] = velocity[0], velocity[1], base
    for _ in range(nbumps):
        cx, cy = rng.uniform(0, 1, 2)
        w = rng.uniform(0.02, 0.2)
        amp = rng.uniform(-0.5, 0.5)
        q[2] += amp * np.exp(-((c[0] - cx) ** 2 + (c[1] - cy) ** 2) / (2 * w * w))
    return mesh, ["periodic"] * 4, None, q
