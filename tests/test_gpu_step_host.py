"""hc_step_host: a host state stepped in one call (upload, steps, download, one wait) equals
hc_state_upload + hc_step + hc_state_download bit for bit, in place or into another buffer,
FP64 and FP32, and reports the same step statistics."""
import numpy as np
import pytest

from hyperboliconvergence_gb300 import cases
from hyperboliconvergence_gb300.solver import Solver

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_step_host_equals_upload_step_download(precision):
    mesh, bc, ref, q, sp = cases.cylinder(24, 64, mach=0.4, rb=6.0)
    a = Solver(mesh, bc, ref, flux="roe", limiter="vanalbada", precision=precision, species=sp)
    a.set_state(q)
    sa = a.step(3)
    want = a.get_state()
    b = Solver(mesh, bc, ref, flux="roe", limiter="vanalbada", precision=precision, species=sp)
    out = np.empty_like(q)
    sb = b.step_host(np.ascontiguousarray(q), out, 3)
    assert np.array_equal(out, want)
    assert sb.dt == sa.dt and sb.t == sa.t and b.steps_done == 3
    inplace = np.ascontiguousarray(q).copy()
    c = Solver(mesh, bc, ref, flux="roe", limiter="vanalbada", precision=precision, species=sp)
    c.step_host(inplace, inplace, 3)
    assert np.array_equal(inplace, want)


def test_step_host_rejects_bad_buffers():
    mesh, bc, ref, q, sp = cases.cylinder(8, 16, mach=0.4, rb=4.0)
    s = Solver(mesh, bc, ref, species=sp)
    with pytest.raises(ValueError):
        s.step_host(q.astype(np.float32), np.empty_like(q))
