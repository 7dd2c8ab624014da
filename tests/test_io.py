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


def _ck_sample(tmp_path):
    rng = np.random.default_rng(4)
    meta = {"format": 2, "law": "euler", "step": 17, "t": 0.125, "dt": 1e-3, "bc": ["wall", "riemann"],
            "species": [1.4, 287.058, 0.3]}
    arrays = {"nodes": rng.standard_normal((5, 7, 2)), "state": rng.standard_normal((4, 4, 6)),
              "ref1": rng.standard_normal((4, 6))}
    p = tmp_path / "ck.hcck"
    io.write_checkpoint(p, meta, arrays)
    return p, meta, arrays


def test_checkpoint_format_round_trip(tmp_path):
    p, meta, arrays = _ck_sample(tmp_path)
    m2, a2 = io.read_checkpoint(p)
    assert m2 == meta
    assert set(a2) == set(arrays) and all(np.array_equal(a2[k], arrays[k]) for k in arrays)
    assert not any(x.name.startswith("ck.hcck.tmp") for x in tmp_path.iterdir())  # written atomically


@pytest.mark.parametrize("where", ["preamble", "header", "payload", "crc"])
def test_checkpoint_flipped_byte_refused(tmp_path, where):
    """Fault injection on the host: one flipped byte anywhere is refused with a clear error."""
    p, _, _ = _ck_sample(tmp_path)
    data = bytearray(p.read_bytes())
    hlen = int.from_bytes(data[8:16], "little")
    pos = {"preamble": 3, "header": 24 + hlen // 2, "payload": 24 + hlen + 40, "crc": len(data) - 2}[where]
    data[pos] ^= 0x20
    p.write_bytes(bytes(data))
    with pytest.raises(io.CheckpointError, match="corrupted|magic|truncated"):
        io.read_checkpoint(p)


def test_checkpoint_truncated_or_foreign_refused(tmp_path):
    p, _, _ = _ck_sample(tmp_path)
    data = p.read_bytes()
    p.write_bytes(data[:-9])
    with pytest.raises(io.CheckpointError, match="truncated"):
        io.read_checkpoint(p)
    p.write_bytes(data[:10])
    with pytest.raises(io.CheckpointError, match="truncated"):
        io.read_checkpoint(p)
    p.write_bytes(data + b"\0")
    with pytest.raises(io.CheckpointError, match="truncated or padded"):
        io.read_checkpoint(p)
    np.savez(tmp_path / "old.npz", a=np.zeros(3))
    with pytest.raises(io.CheckpointError, match="magic"):
        io.read_checkpoint(tmp_path / "old.npz")


@pytest.mark.gpu
@pytest.mark.parametrize("precision,flux", [("fp64", "roe"), ("fp32", "ausmpup"), ("fp64_df", "roe")])
def test_checkpoint_resume_is_bit_exact(tmp_path, precision, flux):
    """Save after 3 steps, reload into a new context, run 2 more: the state equals the
    uninterrupted run's bit for bit, and the step count and time continue."""
    from hyperboliconvergence_gb300.solver import Solver
    mesh, bc, ref, q, sp = cases.cylinder(8, 24, mach=0.4, rb=4.0)
    s = Solver(mesh, bc, ref, flux=flux, limiter="vanalbada", dt="global", species=sp, precision=precision,
               corrections="all")
    s.set_state(q)
    s.step(3)
    io.save_checkpoint(tmp_path / "ck.hcck", s)
    st_a = s.step(2)
    t = io.load_checkpoint(tmp_path / "ck.hcck")
    assert t.steps_done == 3 and (t.precision, t.flux, t.corrections) == (precision, flux, s.corrections)
    st_b = t.step(2)
    assert np.array_equal(s.get_state(), t.get_state())
    assert st_b.t == st_a.t and t.steps_done == 5


@pytest.mark.gpu
def test_checkpoint_resume_one_dimensional(tmp_path):
    from hyperboliconvergence_gb300.solver import Mesh1D, Solver
    x = np.linspace(0.0, 1.0, 65)
    c = 0.5 * (x[:-1] + x[1:])
    q = np.stack([np.zeros_like(c), np.where(c < 0.5, 1.0, 0.125), np.where(c < 0.5, 1.0, 0.1)])
    ref = [q[:, 0], q[:, -1]]
    s = Solver(Mesh1D(x), ["fixed", "fixed"], ref, flux="roe", limiter="mc", cfl=0.8, species=(1.4, 287.058, 1e-4))
    s.set_state(q)
    s.step(10)
    io.save_checkpoint(tmp_path / "ck1d.hcck", s)
    s.step(5)
    t = io.load_checkpoint(tmp_path / "ck1d.hcck")
    t.step(5)
    assert np.array_equal(s.get_state(), t.get_state())
