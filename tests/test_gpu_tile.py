"""Tile shape of the single-mesh stage kernels (hc_set_tile): every shape computes each
face and each cell with the same arithmetic, so FP64 states after several RK steps (and
residuals, timesteps and adjoint gradients) are bit-identical across 8x32, 4x32 and
16x16 tiles; FP32 agrees to its rounding (separate instantiations may contract
differently).  The meshes are smaller and larger than one tile and not multiples of
the tile sides.
"""
import numpy as np
import pytest

from hyperboliconvergence_gb300 import cases
from hyperboliconvergence_gb300._capi import HCError, check
from hyperboliconvergence_gb300.solver import Solver
from test_gpu_parity import CASES

pytestmark = pytest.mark.gpu

TILES = ["8x32", "4x32", "16x16", "16x16/128"]


def run(case, tile, precision="fp64", flux="roe", limiter="vanalbada", dt="local", steps=3):
    mesh, bc, ref, q, species = case
    s = Solver(mesh, bc, ref, flux=flux, limiter=limiter, precision=precision, dt=dt, species=species, tile=tile)
    s.set_state(q)
    res = s.residual()
    st = s.step(steps)
    return res, s.get_state(), st.dt


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("flux,dt", [("roe", "local"), ("slau", "global"), ("ausmpup", "local")])
def test_fp64_tiles_bit_identical(name, flux, dt):
    base = run(CASES[name], "8x32", flux=flux, dt=dt)
    for tile in TILES[1:]:
        got = run(CASES[name], tile, flux=flux, dt=dt)
        assert np.array_equal(got[0], base[0]), tile
        assert np.array_equal(got[1], base[1]), tile
        assert got[2] == base[2], tile


def test_fp64_tiles_large_mesh():
    case = cases.cylinder(70, 150, mach=0.4, rb=8.0)
    base = run(case, "8x32", steps=2)
    for tile in TILES[1:]:
        got = run(case, tile, steps=2)
        assert np.array_equal(got[1], base[1]), tile


def test_fp32_tiles_close():
    base = run(CASES["cylinder"], "8x32", precision="fp32")
    for tile in TILES[1:]:
        got = run(CASES["cylinder"], tile, precision="fp32")
        assert np.allclose(got[1], base[1], rtol=1e-5, atol=1e-6), tile


def test_adjoint_gradient_independent_of_tile():
    mesh, bc, ref, q, species = CASES["quadrant"]
    out = []
    for tile in ["8x32", "16x16"]:
        s = Solver(mesh, bc, ref, flux="roe", limiter="vanalbada", precision="fp64", species=species, tile=tile)
        s.set_state(q)
        J, qbar = s.gradient(5, snapshots=2, kind="l2", target=q * 1.01)[:2]
        out.append((J, qbar))
    assert out[0][0] == out[1][0]
    assert np.array_equal(out[0][1], out[1][1])


def test_unknown_tile_rejected():
    mesh, bc, ref, q, species = CASES["vortex"]
    s = Solver(mesh, bc, ref, species=species)
    with pytest.raises(HCError, match="tile"):
        check(s.lib.hc_set_tile(s.h, 7))
    with pytest.raises(KeyError):
        s.set_tile("32x8")
