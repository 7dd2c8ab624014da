"""Branch flips in the parity report: per face, the branches (limiter pieces, flux
branches, far-field paths) that the CUDA path's evaluation of a state took, against
the oracle's evaluation of the same state (hc_face_signatures / the oracle's
hco_face_signatures share the codes).  In FP64 the two evaluations differ only by
round-off, so a flip needs an argument within round-off of a breakpoint; FP32 and
double-float flips are reported and bounded."""
import numpy as np
import pytest

from hyperboliconvergence_gb300.solver import branch_flips
from test_gpu_parity import CASES, make_pair

pytestmark = pytest.mark.gpu

VALID = np.uint64(1) << np.uint64(63)


def flips(gpu, ora):
    return branch_flips(gpu.face_signatures(), ora.face_signatures())


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("flux,limiter", [("roe", "vanalbada"), ("roe", "minmod"), ("slau", "superbee"),
                                          ("ausmpup", "mc"), ("rusanov", "cada3"), ("roe", "nolimit1")])
def test_fp64_branch_flips_against_oracle(name, flux, limiter):
    gpu, ora = make_pair(CASES[name], flux=flux, limiter=limiter)
    si, sj = gpu.face_signatures()
    assert np.all(si & VALID) and np.all(sj & VALID)  # every face evaluated and recorded
    f = flips(gpu, ora)
    assert f["faces"] <= 0.002 * f["faces_total"], f


def test_fp64_branch_flips_after_steps():
    gpu, ora = make_pair(CASES["quadrant"], flux="slau", limiter="vanleer")
    for _ in range(3):
        gpu.step(1)
        ora.step(1)
    f = flips(gpu, ora)
    assert f["faces"] <= 0.002 * f["faces_total"], f


@pytest.mark.parametrize("precision,bound", [("fp64_df", 0.002), ("fp32", 0.05)])
def test_reduced_precision_branch_flips(precision, bound):
    gpu, ora = make_pair(CASES["cylinder"], flux="roe", limiter="vanalbada", precision=precision)
    f = flips(gpu, ora)
    assert f["faces"] <= bound * f["faces_total"], f
