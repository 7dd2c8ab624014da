"""The torch.autograd.Functions over the discrete adjoint, device-resident.

batch_l2_objective: per-instance L2 objectives of a batch from CUDA tensors;
loss.backward() runs one batched reverse sweep (hc_batch_adjoint_reverse) from the
checkpoints the forward recorded, and its gradients equal Batch.gradient's (the one-call
batched adjoint) bit for bit in FP64.  run_objective: the single-mesh Function, whose
backward no longer repeats the forward sweep, equals Solver.gradient bit for bit.
"""
import numpy as np
import pytest

from hyperboliconvergence_gb300 import cases
from hyperboliconvergence_gb300.batch import Batch
from hyperboliconvergence_gb300.solver import Solver

pytestmark = pytest.mark.gpu

SP = (1.4, 287.058, 0.5)
BASE = (0.5, 0.25, 5.0, 1.0)


def four_instances(seed=5):
    rng = np.random.default_rng(seed)
    insts, targets = [], []
    for ni, nj in [(24, 17), (9, 40), (31, 31), (16, 20)]:
        mesh, bc, ref, q, _ = cases.gaussian_sum(ni, nj, rng, base=BASE)
        insts.append((mesh, bc, ref, q))
        targets.append(cases.gaussian_sum(ni, nj, rng, base=BASE)[3])
    return insts, targets


@pytest.mark.parametrize("flux,limiter", [("roe", "vanalbada"), ("rusanov", "nolimit3")])
def test_batch_backward_equals_batch_gradient(flux, limiter):
    import torch
    from hyperboliconvergence_gb300.autograd import batch_l2_objective
    insts, targets = four_instances()
    nsteps, snaps, w = 9, 3, (1.0, 0.5, 2.0, 1.0)
    ref_b = Batch(insts, flux=flux, limiter=limiter, precision="fp64", species=SP)
    J_ref, g_ref, _ = ref_b.gradient(nsteps, targets, snapshots=snaps, weight=w)

    b = Batch(insts, flux=flux, limiter=limiter, precision="fp64", species=SP)
    q0s = [torch.tensor(q, dtype=torch.float64, device="cuda", requires_grad=True) for (_, _, _, q) in insts]
    tgs = [torch.tensor(t, dtype=torch.float64, device="cuda") for t in targets]
    J = batch_l2_objective(b, q0s, tgs, nsteps, snapshots=snaps, weight=w)
    assert J.shape == (4,) and J.is_cuda
    assert np.array_equal(J.detach().cpu().numpy(), J_ref)
    coef = torch.tensor([1.0, -2.0, 0.5, 3.0], dtype=torch.float64, device="cuda")
    (J * coef).sum().backward()
    for k in range(4):
        want = g_ref[k] * float(coef[k])
        assert np.array_equal(q0s[k].grad.cpu().numpy(), want), (k, np.abs(q0s[k].grad.cpu().numpy() - want).max())


def test_batch_backward_fp32_and_a_second_forward():
    """FP32 batch: the Function's gradients equal the one-call batched adjoint's (the same
    kernels on the same data); a second forward before backward drops the first recording."""
    import torch
    from hyperboliconvergence_gb300.autograd import batch_l2_objective
    insts, targets = four_instances(8)
    nsteps, snaps = 6, 2
    ref_b = Batch(insts, flux="rusanov", limiter="nolimit3", precision="fp32", species=SP)
    J_ref, g_ref, _ = ref_b.gradient(nsteps, targets, snapshots=snaps)
    b = Batch(insts, flux="rusanov", limiter="nolimit3", precision="fp32", species=SP)
    q0s = [torch.tensor(q, dtype=torch.float64, device="cuda", requires_grad=True) for (_, _, _, q) in insts]
    J = batch_l2_objective(b, q0s, targets, nsteps, snapshots=snaps)
    J.sum().backward()
    assert np.array_equal(J.detach().cpu().numpy(), J_ref)
    for k in range(4):
        assert np.array_equal(q0s[k].grad.cpu().numpy(), g_ref[k]), k
    # two recordings, one reverse each: the first one's backward fails cleanly
    q1 = [torch.tensor(q, dtype=torch.float64, device="cuda", requires_grad=True) for (_, _, _, q) in insts]
    J1 = batch_l2_objective(b, q1, targets, nsteps, snapshots=snaps)
    J2 = batch_l2_objective(b, q1, targets, nsteps, snapshots=snaps)
    J2.sum().backward(retain_graph=True)
    with pytest.raises(Exception, match="no recorded forward sweep"):
        J1.sum().backward()


def test_record_reverse_equals_one_call_gradient():
    """Solver.record + Solver.reverse (device outputs) equal Solver.gradient bit for bit, and
    the single-mesh Function's q0 gradient equals them too."""
    import torch
    from hyperboliconvergence_gb300.autograd import run_objective
    mesh, bc, ref, q, sp = cases.cylinder(12, 40, mach=0.4, rb=6.0)
    rng = np.random.default_rng(2)
    q = q * (1 + 0.02 * rng.standard_normal(q.shape))
    kw = dict(kind="drag", scale=1.0, direction=(1.0, 0.0))
    s = Solver(mesh, bc, ref, flux="roe", limiter="vanalbada", species=sp)
    s.set_state(q)
    J0, q0b, refb, rates, _ = s.gradient(8, snapshots=3, **kw)
    s.set_state(q)
    J1, rates1 = s.record(8, snapshots=3, **kw)
    qb = torch.empty(q.shape, dtype=torch.float64, device="cuda")
    nref = sum(4 * mesh.nface(k) for k in range(4))
    rb = torch.empty(nref, dtype=torch.float64, device="cuda")
    s.reverse(qb, rb)
    assert J1 == J0 and np.array_equal(rates1, rates)
    assert np.array_equal(qb.cpu().numpy(), q0b)
    assert np.array_equal(rb.cpu().numpy()[4 * mesh.nj:8 * mesh.nj], refb[1].ravel())
    with pytest.raises(Exception, match="no recorded forward sweep"):
        s.reverse(qb, rb)
    q0 = torch.tensor(q, dtype=torch.float64, device="cuda", requires_grad=True)
    refs = [None if r is None else torch.tensor(r, dtype=torch.float64) for r in ref]
    J = run_objective(s, q0, refs, 8, snapshots=3, **kw)
    J.backward()
    assert float(J) == J0
    assert np.array_equal(q0.grad.cpu().numpy(), q0b)
