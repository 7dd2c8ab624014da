"""The FP32 stage kernel with its tile loads staged by TMA tensor copies (the interior
tiles' state, every tile's i-face records) against the same kernel with plain per-thread
loads (hc_set_staged_loads(ctx, 0)): the same arithmetic on the same values, so residuals,
states and timesteps are bit-identical -- on walls, far fields, periodic and fixed sides,
meshes larger and smaller than a tile and not multiples of it, every limiter the staged
kernel is compiled for, both timestep modes and with the corrections on."""
import numpy as np
import pytest

from hyperboliconvergence_gb300 import cases
from hyperboliconvergence_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def meshes():
    rng = np.random.default_rng(21)
    cyl = cases.cylinder(64, 128, mach=0.5, rb=8.0)
    mesh, bc, ref, q, sp = cyl
    c = mesh.centres()
    q = q * (1 + 0.03 * np.sin(3 * c[0])[None] * np.cos(2 * c[1])[None])
    small = cases.cylinder(13, 36, mach=0.4, rb=4.0)
    return {"cylinder": (mesh, bc, ref, q, sp), "small_cylinder": small, "vortex": cases.isentropic_vortex(64),
            "quadrant": cases.quadrant_riemann(20, 44, rng)}


MESHES = meshes()


def run(case, staged, limiter, dt, flux="roe", corrections=None, steps=5):
    mesh, bc, ref, q, sp = case
    s = Solver(mesh, bc, ref, flux=flux, limiter=limiter, rk="ssp34", dt=dt, cfl=0.5, precision="fp32",
               species=sp, corrections=corrections)
    s.set_staged_loads(staged)
    s.set_state(q)
    r = s.residual()
    st = s.step(steps)
    return r, s.get_state(), st.dt


@pytest.mark.parametrize("name", list(MESHES))
@pytest.mark.parametrize("limiter", ["vanalbada", "vanleer", "minmod", "nolimit2", "nolimit3"])
def test_staged_equals_plain_loads(name, limiter):
    case = MESHES[name]
    dt = "local" if name.endswith("cylinder") else "global"
    a = run(case, True, limiter, dt)
    b = run(case, False, limiter, dt)
    assert np.array_equal(a[0], b[0])
    assert np.array_equal(a[1], b[1])
    assert a[2] == b[2]


def test_staged_equals_plain_with_corrections_and_face_frame_roe():
    case = MESHES["cylinder"]
    a = run(case, True, "vanalbada", "local", flux="roe_face", corrections="all", steps=8)
    b = run(case, False, "vanalbada", "local", flux="roe_face", corrections="all", steps=8)
    assert np.array_equal(a[1], b[1])
