"""Batched path: one persistent launch per stage over many uneven meshes must
give exactly the results of per-instance launches and of single-mesh contexts,
and match the CPU oracle at the FP64 tolerance."""
import numpy as np
import pytest

from hyperboliconvergence_gb300 import cases
from hyperboliconvergence_gb300.batch import Batch, uneven_riemann_batch
from hyperboliconvergence_gb300.solver import Solver
from oracle import oracle_py

pytestmark = pytest.mark.gpu


def small_batch(seed=3, n=5):
    return uneven_riemann_batch(n, seed, sizes=(9, 13, 24, 40, 67))


def states(b):
    return [b.get_state(k) for k in range(b.n)]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("tile", ["8x32", "4x32", "16x16"])
def test_persistent_equals_per_instance(precision, tile):
    insts = small_batch()
    a = Batch(insts, flux="slau", limiter="vanalbada", precision=precision)
    b = Batch(insts, flux="slau", limiter="vanalbada", precision=precision)
    a.set_schedule(tile=tile, ctas_per_sm=1, order="largest_first")
    b.set_schedule(tile=tile)
    a.step_async(3, "persistent")
    b.step_async(3, "per_instance")
    a.sync(), b.sync()
    for x, y in zip(states(a), states(b)):
        assert np.array_equal(x, y)


def test_persistent_tma_tile_equals_per_instance():
    """Every instance's nj a multiple of 4: the FP32 8x32 batch stages its tile loads by TMA
    with per-instance tensor maps (batch_stage_kernel_tma), the per-instance launches by the
    single-mesh TMA kernel; both equal, over several steps and with edge, interior and partial
    tiles (the single-mesh TMA kernel equals the plain-load kernel bit for bit)."""
    insts = uneven_riemann_batch(6, 17, sizes=(12, 20, 36, 44, 68, 100))
    a = Batch(insts, flux="slau", limiter="vanalbada", precision="fp32")
    b = Batch(insts, flux="slau", limiter="vanalbada", precision="fp32")
    a.set_schedule(tile="8x32", ctas_per_sm=2, order="largest_first")
    b.set_schedule(tile="8x32")
    a.step_async(4, "persistent")
    b.step_async(4, "per_instance")
    a.sync(), b.sync()
    for x, y in zip(states(a), states(b)):
        assert np.array_equal(x, y)


def test_batch_equals_single_contexts():
    insts = small_batch(seed=11, n=4)
    bt = Batch(insts, flux="roe", limiter="vanleer", precision="fp64", dt="global")
    bt.step_async(2)
    st = bt.sync()
    for k, (mesh, bc, ref, q) in enumerate(insts):
        s = Solver(mesh, bc, ref, flux="roe", limiter="vanleer", precision="fp64", dt="global",
                   species=(1.4, 287.058, 0.5))
        s.set_state(q)
        one = s.step(2)
        assert np.array_equal(s.get_state(), bt.get_state(k))
        assert one.dt == st[k].dt


def test_batch_fp64_matches_oracle():
    insts = small_batch(seed=5, n=3)
    bt = Batch(insts, flux="slau", limiter="vanalbada", precision="fp64")
    bt.step_async(2)
    bt.sync()
    for k, (mesh, bc, ref, q) in enumerate(insts):
        o = oracle_py.OracleSolver(mesh.ni, mesh.nj, mesh.nodes.ravel(), bc, flux="slau", limiter="vanalbada",
                                   species=(1.4, 287.058, 0.5), ghost_ref=ref)
        o.set_state(q)
        o.step(2)
        a, b = bt.get_state(k), o.get_state()
        err = (np.abs(a - b).reshape(4, -1).max(1) / np.abs(b).reshape(4, -1).max(1)).max()
        assert err <= 1e-12, (k, err)


def test_batch_fp64_matches_oracle_over_200_steps():
    """The batched configuration's 200 steps (SLAU + van Albada, ssp34, CFL 0.5, global dt)
    on a small four-quadrant instance, FP64 batch against the oracle free-running."""
    insts = uneven_riemann_batch(2, 2026, sizes=(24, 40))
    bt = Batch(insts, flux="slau", limiter="vanalbada", precision="fp64")
    bt.step_async(200)
    bt.sync()
    for k, (mesh, bc, ref, q) in enumerate(insts):
        o = oracle_py.OracleSolver(mesh.ni, mesh.nj, mesh.nodes.ravel(), bc, flux="slau", limiter="vanalbada",
                                   species=(1.4, 287.058, 0.5), ghost_ref=ref)
        o.set_state(q)
        o.step(200)
        a, b = bt.get_state(k), o.get_state()
        err = (np.abs(a - b).reshape(4, -1).max(1) / np.abs(b).reshape(4, -1).max(1)).max()
        assert err <= 1e-9, (k, err)


def test_graph_replay_equals_stream_steps():
    insts = small_batch(seed=8, n=4)
    a = Batch(insts, precision="fp32")
    b = Batch(insts, precision="fp32")
    a.capture(3)
    a.replay()
    a.sync()
    b.step_async(3)
    b.sync()
    for x, y in zip(states(a), states(b)):
        assert np.array_equal(x, y)
    # replay again continues from the new state
    a.replay()
    a.sync()
    b.step_async(3)
    b.sync()
    for x, y in zip(states(a), states(b)):
        assert np.array_equal(x, y)


def test_autotune_keeps_states_and_picks_a_schedule():
    insts = small_batch(seed=9, n=6)
    b = Batch(insts, precision="fp32")
    before = states(b)
    sch = b.autotune(steps=1)
    assert sch["tile"] in ("8x32", "4x32", "16x16") and sch["ms_per_step"] > 0
    for x, y in zip(before, states(b)):
        assert np.array_equal(x, y)
    b.step_async(1)
    b.sync()
