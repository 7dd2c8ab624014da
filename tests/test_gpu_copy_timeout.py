"""Failure detection of the TMA-staged FP32 stage kernel's copy waits, without a GPU fault.

hc_inject_stalled_copy arms the face-record barrier for 16 bytes more than the tensor copy
delivers.  Every CTA's wait on it gives up after its one-second bound, marks the step
ST_TIMEOUT, and the host returns HC_ERR_TIMEOUT.  The copy itself completes, so nothing is
left in flight and the context stays usable: cleared, the same context steps on and matches
a fresh context's run bit for bit."""
import time

import numpy as np
import pytest

from hyperboliconvergence_gb300 import cases
from hyperboliconvergence_gb300._capi import HC_ERR_TIMEOUT, HCError
from hyperboliconvergence_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def make():
    # nj = 64 (a multiple of 4): the TMA-staged kernel; 2 x 2 tiles, one wave of CTAs
    mesh, bc, ref, q, sp = cases.cylinder(16, 64, mach=0.3)
    s = Solver(mesh, bc, ref, flux="roe", limiter="vanalbada", rk="ssp34", dt="local", cfl=0.5,
               precision="fp32", species=sp)
    s.set_state(q)
    return s, q


def test_stalled_copy_times_out_and_the_context_recovers():
    s, q = make()
    s.inject_stalled_copy(True)
    t0 = time.perf_counter()
    with pytest.raises(HCError) as err:
        s.step(1)
    elapsed = time.perf_counter() - t0
    assert err.value.code == HC_ERR_TIMEOUT
    # four stage launches, each CTA giving up after one second
    assert 3.5 <= elapsed <= 60.0, elapsed
    s.inject_stalled_copy(False)
    s.set_state(q)
    s.step(3)
    fresh, _ = make()
    fresh.step(3)
    assert np.array_equal(s.get_state(), fresh.get_state())
