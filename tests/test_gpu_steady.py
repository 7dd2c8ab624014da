"""Steady-state driver (SteadyTimeControls, controls.h:31-48): convergence of the
density residual with local timestepping, the step cap, and the refusal of
residual smoothing."""
import ctypes as C

import numpy as np
import pytest

from hyperboliconvergence_gb300 import cases
from hyperboliconvergence_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def small_cylinder(**kw):
    mesh, bc, ref, q, sp = cases.cylinder(24, 48, mach=0.3, rb=8.0)
    s = Solver(mesh, bc, ref, flux="roe", limiter="vanalbada", dt="local", cfl=0.5, species=sp, **kw)
    s.set_state(q)
    return s


def bump_box(n=32):
    """A density bump in uniform M0.5 flow on [0,1]^2 with Riemann far field on every
    side: the disturbance leaves the box and the state relaxes to the freestream."""
    from hyperboliconvergence_gb300.solver import Mesh
    mesh = Mesh.linspace(n, n, 0.0, 1.0, 0.0, 1.0)
    qinf = np.array([0.5 * np.sqrt(1.4), 0.1, 1.0, 1.0])
    c = mesh.centres()
    q = np.broadcast_to(qinf[:, None, None], (4, n, n)).copy()
    q[2] += 0.05 * np.exp(-((c[0] - 0.5) ** 2 + (c[1] - 0.5) ** 2) / (2 * 0.1 ** 2))
    ref = [np.broadcast_to(qinf[:, None], (4, n)).copy() for _ in range(4)]
    s = Solver(mesh, ["riemann"] * 4, ref, flux="roe", limiter="vanalbada", dt="local", cfl=0.5,
               species=(1.4, 287.058, 0.5))
    s.set_state(q)
    return s, qinf


def test_steady_converges_to_freestream():
    s, qinf = bump_box()
    st, hist = s.steady(60000, residual_drop=1e-8, check_every=500)
    assert st.converged, (st.steps, (hist[-5:] / hist[0]).tolist())
    assert st.res <= 1e-8 * st.res0 and hist[0] == st.res0 and hist[-1] == st.res
    assert len(hist) == st.history_len
    assert np.abs(s.get_state() - qinf[:, None, None]).max() < 1e-6


def test_steady_stops_at_step_cap():
    s = small_cylinder()
    st, hist = s.steady(10, residual_drop=1e-30, check_every=4)
    assert not st.converged and st.steps == 10 and len(hist) == 4  # steps 1, 5, 9, 10


def test_steady_refuses_residual_smoothing_on_2d_contexts():
    """Residual smoothing exists only for the reference's 1D path (test_gpu_smooth covers it)."""
    from hyperboliconvergence_gb300._capi import SteadyControls, SteadyStats
    s = small_cylinder()
    ctl = SteadyControls(100, 1e-6, 10, 1, 0.5)
    st = SteadyStats()
    assert s.lib.hc_steady_run(s.h, C.byref(ctl), None, 0, C.byref(st)) == 5
