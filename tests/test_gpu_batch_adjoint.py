"""Batched discrete adjoint (hc_batch_adjoint_gradient): one reverse sweep over
every instance of a batch, each reverse pass one launch over all instances.

Every instance's J and gradient must equal those of the single-mesh adjoint of
the same instance (whose gradients are checked against central differences and the
dual-number FP64 reference in test_gpu_adjoint): the batch runs the same stage and
reverse bodies on each instance's slices of its pools, with the same frozen
timesteps.  In FP64 the results are bit-identical (the stage arithmetic fixes its
fused multiply-adds explicitly).  In FP32 the batched and plain stage kernels are
separate compilations whose contractions may differ: J agrees to FP32 rounding, and
the gradient too where the reconstruction is smooth (NoLimit3).
"""
import numpy as np
import pytest

from hyperboliconvergence_gb300 import cases
from hyperboliconvergence_gb300.batch import Batch
from hyperboliconvergence_gb300.solver import Solver

pytestmark = pytest.mark.gpu

SP = (1.4, 287.058, 0.5)
BASE = (0.5, 0.25, 5.0, 1.0)


def mixed_batch(seed):
    """Periodic Gaussian-sum instances of uneven sizes plus a four-quadrant Riemann
    instance with fixed boundaries; a seeded target per instance."""
    rng = np.random.default_rng(seed)
    insts, targets = [], []
    for ni, nj in [(24, 17), (9, 40), (31, 31)]:
        mesh, bc, ref, q, _ = cases.gaussian_sum(ni, nj, rng, base=BASE)
        insts.append((mesh, bc, ref, q))
        targets.append(cases.gaussian_sum(ni, nj, rng, base=BASE)[3])
    mesh, bc, ref, q, _ = cases.quadrant_riemann(13, 22, rng)
    insts.append((mesh, bc, ref, q))
    targets.append(q * (1 + 0.01 * rng.standard_normal(q.shape)))
    return insts, targets


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("flux,limiter", [("rusanov", "nolimit3"), ("roe", "vanalbada"), ("roe", "minmod"),
                                          ("slau", "vanalbada"), ("ausmpup", "nolimit3"), ("roe_ws", "minmod")])
def test_batch_adjoint_equals_single_mesh_adjoints(precision, flux, limiter):
    insts, targets = mixed_batch(41)
    nsteps, snaps = 7, 3
    w = (1.0, 0.5, 2.0, 1.0)
    bt = Batch(insts, flux=flux, limiter=limiter, precision=precision, species=SP)
    J, grads, st = bt.gradient(nsteps, targets, snapshots=snaps, weight=w)
    assert st.adjoint_steps == nsteps
    for k, (mesh, bc, ref, q) in enumerate(insts):
        s = Solver(mesh, bc, ref, flux=flux, limiter=limiter, precision=precision, species=SP)
        s.set_state(q)
        j1, g1 = s.gradient(nsteps, snapshots=snaps, kind="l2", target=targets[k], weight=w)[:2]
        if precision == "fp64":
            assert J[k] == j1, (k, J[k], j1)
            assert np.array_equal(grads[k], g1), (k, np.abs(grads[k] - g1).max())
        else:
            assert J[k] == pytest.approx(j1, rel=1e-5), (k, J[k], j1)
            if limiter.startswith("nolimit"):
                # with a limiter, rounding-level state differences flip its branches where the
                # state is uniform to round-off, and the gradients there differ by O(1)
                assert np.abs(grads[k] - g1).max() <= 1e-4 * np.abs(g1).max(), (k, np.abs(grads[k] - g1).max())
        assert np.all(np.isfinite(g1))


def test_batch_adjoint_launches_do_not_grow_with_instances():
    """The reverse sweep's launches are those of one instance: the same for a batch
    of one instance and a batch of four."""
    insts, targets = mixed_batch(7)
    one = Batch(insts[:1], flux="rusanov", limiter="nolimit3", precision="fp32", species=SP)
    four = Batch(insts, flux="rusanov", limiter="nolimit3", precision="fp32", species=SP)
    _, _, s1 = one.gradient(6, targets[:1], snapshots=2)
    _, _, s4 = four.gradient(6, targets, snapshots=2)
    assert s1.kernel_launches == s4.kernel_launches
    assert s1.forward_steps == s4.forward_steps


def test_batch_adjoint_leaves_states_and_honours_want():
    insts, targets = mixed_batch(9)
    bt = Batch(insts, flux="roe", limiter="vanalbada", precision="fp64", species=SP)
    before = [bt.get_state(k) for k in range(bt.n)]
    J, grads, _ = bt.gradient(4, targets, snapshots=1, want=[2])
    assert list(grads) == [2]
    assert J.shape == (bt.n,) and np.all(J > 0)
    for k in range(bt.n):
        assert np.array_equal(bt.get_state(k), before[k])


def test_batch_adjoint_unsupported_configurations():
    insts, targets = mixed_batch(3)
    local = Batch(insts, flux="roe", limiter="vanalbada", precision="fp64", dt="local", species=SP)
    with pytest.raises(Exception, match="global timestep"):
        local.gradient(2, targets)
    central = Batch(insts, flux="central", limiter="vanalbada", precision="fp64", species=SP)
    with pytest.raises(Exception, match="Roe, Rusanov, SLAU"):
        central.gradient(2, targets)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_adjoint_with_farfield_instances(precision):
    """Instances with Riemann and entropy far fields (the ghost update reversed by
    tangents): every instance's J and gradient equal its single-mesh adjoint's."""
    from hyperboliconvergence_gb300.solver import Mesh
    insts, targets = [], []
    rng = np.random.default_rng(21)
    for k, (nr, nth, bc1) in enumerate([(10, 32, "riemann"), (14, 24, "entropy")]):
        mesh = Mesh.cylinder(nr, nth, 0.5, 4.0, 1.05)
        qinf = np.array([0.4 * np.cos(0.1), 0.4 * np.sin(0.1), 1.0, 1.0 / 1.4])
        c = mesh.centres()
        shape = 0.5 * np.exp(-((c[0] - 1.0) ** 2 + c[1] ** 2)) + 0.1 * c[0] + 0.07 * c[1]
        q = qinf[:, None, None] + np.array([0.02, 0.02, 0.03, 0.02])[:, None, None] * shape[None]
        ref = [None, np.broadcast_to(qinf[:, None], (4, nth)).copy(), None, None]
        insts.append((mesh, ["wall", bc1, "periodic", "periodic"], ref, q))
        targets.append(q * (1 + 0.01 * rng.standard_normal(q.shape)))
    sp = (1.4, 287.058, 0.4)
    bt = Batch(insts, flux="roe", limiter="vanalbada", precision=precision, species=sp)
    J, grads, _ = bt.gradient(5, targets, snapshots=2)
    for k, (mesh, bc, ref, q) in enumerate(insts):
        s = Solver(mesh, bc, ref, flux="roe", limiter="vanalbada", precision=precision, species=sp)
        s.set_state(q)
        j1, g1 = s.gradient(5, snapshots=2, kind="l2", target=targets[k])[:2]
        if precision == "fp64":
            assert J[k] == j1
            assert np.array_equal(grads[k], g1)
        else:
            assert J[k] == pytest.approx(j1, rel=1e-5)
