"""Stage tapes of the adjoint's checkpointing (hc_set_adjoint_tapes).

Reversing a step needs its stage states.  Without a tape they are replayed from the
step's start state; a tape keeps them from the forward sweep or the re-advance that
computed the step last before its reversal.  The tapes change where the stage states
come from, not their values: the gradients are bit-identical to the replaying reversal's
for every tape count, with the same re-advances, and the default count (one per
snapshot and one more) replays no step."""
import numpy as np
import pytest

from hyperboliconvergence_gb300 import cases
from hyperboliconvergence_gb300.batch import Batch
from hyperboliconvergence_gb300.solver import Mesh, Solver

pytestmark = pytest.mark.gpu

SP = (1.4, 287.058, 0.4)


def cylinder(precision="fp64", seed=3):
    mesh = Mesh.cylinder(10, 32, 0.5, 4.0, 1.05)
    qinf = np.array([0.4 * np.cos(0.1), 0.4 * np.sin(0.1), 1.0, 1.0 / 1.4])
    c = mesh.centres()
    rng = np.random.default_rng(seed)
    shape = 0.5 * np.exp(-((c[0] - 1.0) ** 2 + c[1] ** 2)) + 0.1 * c[0] + 0.07 * c[1]
    q = qinf[:, None, None] + (0.02 * (1 + 0.2 * rng.random(4)))[:, None, None] * shape[None]
    ref = [None, np.broadcast_to(qinf[:, None], (4, 32)).copy(), None, None]
    s = Solver(mesh, ["wall", "fixed", "periodic", "periodic"], ref, flux="roe", limiter="vanalbada",
               rk="ssp34", precision=precision, dt="global", cfl=0.5, species=SP)
    return s, q


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("nsteps,snapshots", [(16, 2), (9, 3), (20, 4), (7, 0), (12, 11)])
def test_tapes_leave_the_gradient_bit_identical(precision, nsteps, snapshots):
    s, q = cylinder(precision)
    out = {}
    for tapes in (0, 1, 2, -1):
        s.set_adjoint_tapes(tapes)
        s.set_state(q)
        J, g, refb, rates, st = s.gradient(nsteps, snapshots=snapshots, kind="drag", scale=1.0)
        out[tapes] = (J, g, refb, st.replays, st.stage_tapes, st.forward_steps)
    J0, g0, r0, rep0, nt0, fw0 = out[0]
    assert nt0 == 0 and rep0 == nsteps
    for tapes in (1, 2, -1):
        J, g, refb, rep, nt, fw = out[tapes]
        assert J == J0 and np.array_equal(g, g0), tapes
        assert all(np.array_equal(a, b) for a, b in zip(refb, r0))
        # the same re-advances; the replays saved are the forward steps saved
        assert fw0 - fw == rep0 - rep, (tapes, fw0, fw, rep0, rep)
    assert out[-1][4] == min(snapshots + 1, nsteps)
    assert out[-1][3] == 0
    assert out[1][3] < nsteps


def test_tapes_with_record_and_reverse():
    """The recorded sweep keeps its tapes until the reverse call."""
    s, q = cylinder()
    s.set_adjoint_tapes(0)
    s.set_state(q)
    J0, g0, _, _, _ = s.gradient(14, snapshots=3, kind="drag", scale=1.0)
    s.set_adjoint_tapes(-1)
    s.set_state(q)
    import torch
    J1, _ = s.record(14, snapshots=3, kind="drag", scale=1.0)
    g1 = torch.empty(q.shape, dtype=torch.float64, device="cuda")
    st = s.reverse(g1)
    assert J1 == J0 and np.array_equal(g1.cpu().numpy(), g0)
    assert st.replays == 0 and st.stage_tapes == 4


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_tapes_leave_the_gradient_bit_identical(precision):
    rng = np.random.default_rng(11)
    insts, targets = [], []
    for ni, nj in [(24, 17), (9, 40), (31, 31)]:
        mesh, bc, ref, q0, _ = cases.gaussian_sum(ni, nj, rng, base=(0.5, 0.25, 5.0, 1.0))
        insts.append((mesh, bc, ref, q0))
        targets.append(cases.gaussian_sum(ni, nj, rng, base=(0.5, 0.25, 5.0, 1.0))[3])
    res = {}
    for tapes in (0, 2, -1):
        b = Batch(insts, flux="roe", limiter="vanalbada", precision=precision, species=(1.4, 287.058, 0.5))
        b.set_adjoint_tapes(tapes)
        J, g, st = b.gradient(15, targets, snapshots=3)
        res[tapes] = (J, g, st.replays, st.stage_tapes)
    J0, g0, rep0, _ = res[0]
    assert rep0 == 15
    for tapes in (2, -1):
        J, g, rep, nt = res[tapes]
        assert np.array_equal(J, J0)
        for k in g0:
            assert np.array_equal(g[k], g0[k]), (tapes, k)
    assert res[-1][2] == 0 and res[-1][3] == 4
