"""Branch flips in the parity report: per face, the branches (limiter pieces, flux
branches, far-field paths) that the CUDA path's evaluation of a state took, against
the oracle's evaluation of the same state (hc_face_signatures / the oracle's
hco_face_signatures share the codes).  In FP64 the two evaluations differ only by
round-off, so a flip needs a limiter argument within round-off of a breakpoint: on
states without round-off-level structure (the perturbed cylinder, the piecewise
constant quadrants) flips are rare; where the state is uniform to round-off (the far
field of the isentropic vortex) the arguments are noise and flip freely, with no
effect on the residual beyond the parity bar.  FP32 and double-float flips are
reported and bounded."""
import numpy as np
import pytest

from hyperboliconvergence_gb300.solver import branch_flips
from test_gpu_parity import CASES, make_pair

pytestmark = pytest.mark.gpu

VALID = np.uint64(1) << np.uint64(63)
COMBOS = [("roe", "vanalbada"), ("roe", "minmod"), ("slau", "superbee"), ("ausmpup", "mc"), ("rusanov", "cada3"),
          ("roe", "nolimit1")]


def flips(gpu, ora, **kw):
    return branch_flips(gpu.face_signatures(), ora.face_signatures(), **kw)


@pytest.mark.parametrize("flux,limiter", COMBOS)
def test_fp64_branch_flips_against_oracle(flux, limiter):
    """The perturbed cylinder state has no structurally zero limiter arguments."""
    gpu, ora = make_pair(CASES["cylinder"], flux=flux, limiter=limiter)
    si, sj = gpu.face_signatures()
    assert np.all(si & VALID) and np.all(sj & VALID)  # every face evaluated and recorded
    assert all(np.array_equal(x, y) for x, y in zip((si, sj), gpu.face_signatures()))  # deterministic
    f = flips(gpu, ora)
    assert f["faces"] <= 0.002 * f["faces_total"], f
    # the recorded limiter arguments are the oracle's to FP64 round-off
    (_, gargs), (_, oargs) = gpu.face_signatures(with_args=True), ora.face_signatures(with_args=True)
    for g, o in zip(gargs, oargs):
        scale = np.abs(o).max(axis=(0, 1, 3)) + 1e-300
        assert np.all(np.abs(g - o).max(axis=(0, 1, 3)) <= 1e-9 * scale)


def assert_flips_at_roundoff(gpu, ora, limiter):
    (oi, oj), args = ora.face_signatures(with_args=True)
    f = branch_flips(gpu.face_signatures(), (oi, oj), args=args, limiter=limiter)
    assert f["faces_above_roundoff"] == 0, f


@pytest.mark.parametrize("name", ["vortex", "quadrant"])
@pytest.mark.parametrize("limiter", ["vanalbada", "minmod", "superbee", "mc"])
def test_fp64_branch_flips_only_at_roundoff_arguments(name, limiter):
    """Where a limiter argument is zero (or at a breakpoint) in exact arithmetic -- a
    biased gradient whose other neighbours are uniform, a far field uniform to 1e-11 --
    its computed value is round-off and the piece is noise; the limited slope is then
    round-off either way.  Every flipped piece must be such a case: the oracle's
    arguments lie within 1e-9 of the variable's argument scale from a breakpoint."""
    gpu, ora = make_pair(CASES[name], flux="roe", limiter=limiter)
    assert_flips_at_roundoff(gpu, ora, limiter)


def test_fp64_branch_flips_after_steps():
    gpu, ora = make_pair(CASES["quadrant"], flux="slau", limiter="vanleer")
    for _ in range(3):
        gpu.step(1)
        ora.step(1)
    assert_flips_at_roundoff(gpu, ora, "vanleer")


@pytest.mark.parametrize("precision,bound", [("fp64_df", 0.002), ("fp32", 0.05)])
def test_reduced_precision_branch_flips(precision, bound):
    gpu, ora = make_pair(CASES["cylinder"], flux="roe", limiter="vanalbada", precision=precision)
    f = flips(gpu, ora)
    assert f["faces"] <= bound * f["faces_total"], f
