"""Batches of scalar-advection instances (law="scalar"): the persistent launch equals
per-instance launches and single-mesh contexts bit for bit (FP64 and FP32, every tile
shape), FP64 matches the scalar oracle at the parity bar, graph replay equals stream
steps, and the batched adjoint equals every instance's single-mesh adjoint (bit for
bit in FP64, to FP32 rounding in FP32)."""
import numpy as np
import pytest

from hyperboliconvergence_gb300 import cases
from hyperboliconvergence_gb300.batch import Batch
from hyperboliconvergence_gb300.solver import Mesh, Solver
from oracle import oracle_py

pytestmark = pytest.mark.gpu


def fixed_instance(ni, nj, rng):
    """A scalar instance with fixed ghost layers on all four sides and a non-uniform velocity."""
    mesh = Mesh.linspace(ni, nj, 0.0, 1.0, 0.0, 1.0)
    c = mesh.centres()
    q = np.stack([0.7 + 0.1 * np.sin(2 * np.pi * (c[1] + 0.2)), -0.4 + 0.08 * np.cos(2 * np.pi * (c[0] + 0.3)),
                  1.0 + 0.3 * np.exp(-((c[0] - rng.uniform(0.3, 0.7)) ** 2 + (c[1] - 0.45) ** 2) / 0.03)])
    ref = [q[:, 0, :].copy(), q[:, -1, :].copy(), q[:, :, 0].copy(), q[:, :, -1].copy()]
    return mesh, ["fixed"] * 4, ref, q


def riemann_instance(ni, nj):
    mesh = Mesh.linspace(ni, nj, 0.0, 1.0, 0.0, 1.0)
    c = mesh.centres()
    q = np.stack([-(c[1] - 0.5), c[0] - 0.5, 1.0 + 0.5 * np.exp(-((c[0] - 0.4) ** 2 + (c[1] - 0.55) ** 2) / 0.02)])
    ref = [None, None, np.stack([-(np.linspace(0, 1, ni) - 0.5), np.full(ni, -0.5), np.ones(ni)]),
           np.stack([-(np.linspace(0, 1, ni) - 0.5), np.full(ni, 0.5), np.full(ni, 1.2)])]
    return mesh, ["periodic", "periodic", "riemann", "riemann"], ref, q


def scalar_batch(seed=4, riemann=True):
    rng = np.random.default_rng(seed)
    insts = [cases.scalar_gaussian_sum(ni, nj, rng) for ni, nj in [(24, 17), (9, 40), (37, 31)]]
    insts.append(fixed_instance(13, 22, rng))
    if riemann:
        insts.append(riemann_instance(20, 28))
    return insts


def states(b):
    return [b.get_state(k) for k in range(b.n)]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("tile", ["8x32", "4x32", "16x16"])
@pytest.mark.parametrize("flux", ["rusanov", "central"])
def test_scalar_persistent_equals_per_instance(precision, tile, flux):
    insts = scalar_batch()
    a = Batch(insts, law="scalar", flux=flux, limiter="vanalbada", precision=precision)
    b = Batch(insts, law="scalar", flux=flux, limiter="vanalbada", precision=precision)
    a.set_schedule(tile=tile, ctas_per_sm=1, order="largest_first")
    b.set_schedule(tile=tile)
    a.step_async(3, "persistent")
    b.step_async(3, "per_instance")
    a.sync(), b.sync()
    for x, y in zip(states(a), states(b)):
        assert x.shape[0] == 3
        assert np.array_equal(x, y)


@pytest.mark.parametrize("dt", ["global", "local"])
def test_scalar_batch_equals_single_contexts(dt):
    insts = scalar_batch(seed=9)
    bt = Batch(insts, law="scalar", flux="rusanov", limiter="minmod", precision="fp64", dt=dt)
    bt.step_async(2)
    st = bt.sync()
    for k, (mesh, bc, ref, q) in enumerate(insts):
        s = Solver(mesh, bc, ref, flux="rusanov", limiter="minmod", precision="fp64", dt=dt, law="scalar",
                   tile="8x32")
        s.set_state(q)
        one = s.step(2)
        assert np.array_equal(s.get_state(), bt.get_state(k)), k
        if dt == "global":
            assert one.dt == st[k].dt


@pytest.mark.parametrize("flux", ["rusanov", "central"])
def test_scalar_batch_fp64_matches_oracle(flux):
    insts = scalar_batch(seed=5)
    bt = Batch(insts, law="scalar", flux=flux, limiter="vanleer", precision="fp64")
    bt.step_async(3)
    bt.sync()
    for k, (mesh, bc, ref, q) in enumerate(insts):
        o = oracle_py.ScalarOracleSolver(mesh.ni, mesh.nj, mesh.nodes.ravel(), bc, flux=flux, limiter="vanleer",
                                         ghost_ref=ref)
        o.set_state(q)
        o.step(3)
        ref_state = o.get_state().reshape(3, mesh.ni, mesh.nj)
        err = np.abs(bt.get_state(k) - ref_state).reshape(3, -1).max(1) / np.abs(ref_state).reshape(3, -1).max(1)
        assert err.max() <= 1e-12, (k, err)


def test_scalar_graph_replay_equals_stream_steps():
    insts = scalar_batch(seed=6)
    a = Batch(insts, law="scalar", flux="rusanov", limiter="vanalbada", precision="fp32", stream=None)
    b = Batch(insts, law="scalar", flux="rusanov", limiter="vanalbada", precision="fp32")
    a.capture(2)
    a.replay()
    a.sync()
    b.step_async(2)
    b.sync()
    for x, y in zip(states(a), states(b)):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("flux,limiter", [("rusanov", "vanalbada"), ("central", "minmod"), ("rusanov", "nolimit3")])
def test_scalar_batch_adjoint_equals_single_mesh(precision, flux, limiter):
    insts = scalar_batch(seed=12)
    rng = np.random.default_rng(3)
    targets = [q * (1 + 0.02 * rng.standard_normal(q.shape)) for (_, _, _, q) in insts]
    w = (0.5, 2.0, 1.0, 0.0)
    bt = Batch(insts, law="scalar", flux=flux, limiter=limiter, precision=precision)
    J, grads, st = bt.gradient(5, targets, snapshots=2, weight=w)
    assert st.adjoint_steps == 5
    for k, (mesh, bc, ref, q) in enumerate(insts):
        s = Solver(mesh, bc, ref, flux=flux, limiter=limiter, precision=precision, law="scalar", tile="8x32")
        s.set_state(q)
        j1, g1 = s.gradient(5, snapshots=2, kind="l2", target=targets[k], weight=w)[:2]
        assert grads[k].shape == (3, mesh.ni, mesh.nj)
        if precision == "fp64":
            assert J[k] == j1, (k, J[k], j1)
            assert np.array_equal(grads[k], g1), (k, np.abs(grads[k] - g1).max())
        else:
            assert J[k] == pytest.approx(j1, rel=1e-5)
            if limiter.startswith("nolimit"):
                assert np.abs(grads[k] - g1).max() <= 1e-4 * np.abs(g1).max()


def test_scalar_batch_rejections():
    insts = scalar_batch(seed=2, riemann=False)
    with pytest.raises(Exception, match="Rusanov or central"):
        Batch(insts, law="scalar", flux="roe")
    mesh = Mesh.linspace(10, 12, 0.0, 1.0, 0.0, 1.0)
    with pytest.raises(Exception, match="periodic, fixed or Riemann"):
        Batch([(mesh, ["wall", "wall", "periodic", "periodic"], None, np.ones((3, 10, 12)))], law="scalar",
              flux="rusanov")
    rb = Batch([riemann_instance(12, 14)], law="scalar", flux="rusanov", precision="fp64")
    with pytest.raises(Exception, match="target 0"):
        rb.gradient(2, [np.ones((4, 12, 14))])
