"""Gnuplot text writers in the reference drivers' layout and the checkpoint
round trip (host side; the checkpoint reload runs on the GPU)."""
import numpy as np
import pytest

from hyperboliconvergence_gb300 import cases, io
from hyperboliconvergence_gb300.solver import Mesh


def test_mesh_dat_layout(tmp_path):
    mesh = Mesh.cylinder(3, 5, 0.5, 2.0, 1.01)
    p = tmp_path / "mesh.dat"
    io.write_mesh_dat(p, mesh)
    blocks = io.read_dat(p)
    assert len(blocks) == mesh.ni + 1 and all(b.shape == (mesh.nj + 1, 2) for b in blocks)
    assert np.allclose(np.stack(blocks), mesh.nodes, rtol=1e-8, atol=1e-12)


def test_cylinder_result_dat_freestream_is_zero(tmp_path):
    mesh, bc, ref, q, sp = cases.cylinder(4, 8, mach=0.3, rb=3.0)
    qinf = ref[1][:, 0]
    p = tmp_path / "result.dat"
    io.write_cylinder_result_dat(p, mesh, q, qinf)
    blocks = io.read_dat(p)
    assert len(blocks) == 4 and all(b.shape == (8, 9) for b in blocks)
    d = np.stack(blocks)
    # (rho-rho0)/rho0, v/|U0|, (p-p0)/p0, (s-s0)/s0 vanish; u/|U0| and a/a0 are one
    assert np.abs(d[..., [3, 5, 6, 7]]).max() < 1e-12
    assert np.allclose(d[..., 4], 1.0) and np.allclose(d[..., 8], 1.0)
    c = mesh.centres()
    assert np.allclose(d[..., 2], np.hypot(c[0], c[1]), rtol=1e-8)


def test_cartesian_result_dat_columns(tmp_path):
    mesh, bc, ref, q, sp = cases.isentropic_vortex(6)
    p = tmp_path / "result.dat"
    qref = np.array([0.0, 0.0, 1.0, 1.0])
    io.write_cartesian_result_dat(p, mesh, q, qref)
    d = np.stack(io.read_dat(p))
    assert d.shape == (6, 6, 9)
    assert np.allclose(d[..., 2], q[2], rtol=1e-14)
    assert np.allclose(d[..., 3], q[0], rtol=1e-14) and np.allclose(d[..., 5], q[3] - 1.0, rtol=1e-12, atol=1e-15)
    a = np.sqrt(1.4 * q[3] / q[2])
    assert np.allclose(d[..., 8], np.hypot(q[0], q[1]) / a, rtol=1e-14)


@pytest.mark.gpu
def test_checkpoint_round_trip(tmp_path):
    from hyperboliconvergence_gb300.solver import Solver
    mesh, bc, ref, q, sp = cases.cylinder(8, 24, mach=0.4, rb=4.0)
    s = Solver(mesh, bc, ref, flux="roe", limiter="vanalbada", dt="local", species=sp)
    s.set_state(q)
    s.step(3)
    io.save_checkpoint(tmp_path / "ck.npz", s)
    s.step(2)
    t = io.load_checkpoint(tmp_path / "ck.npz")
    t.step(2)
    assert np.array_equal(s.get_state(), t.get_state())
