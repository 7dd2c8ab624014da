"""The C-ABI library loads and exports every function include/hc.h declares;
host-side logic that needs no GPU (mesh generators, argument checking)."""
import ctypes as C

import numpy as np
import pytest

from hyperboliconvergence_gb300 import _capi
from hyperboliconvergence_gb300.solver import Mesh
from oracle import oracle_py


def test_exports_every_declared_symbol():
    lib = _capi.load()
    names = _capi.header_symbols()
    assert len(names) >= 18
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_version_string():
    assert b"sm_103a" in _capi.load().hc_version()


def test_mesh_generators_match_oracle():
    o = oracle_py.pointwise()
    for stretch in (1.0, 1.01):
        m = Mesh.cylinder(20, 36, 0.5, 20.0, stretch)
        ref = o.cylinder_nodes(20, 36, 0.5, 20.0, stretch).reshape(21, 37, 2)
        assert np.array_equal(m.nodes, ref)
        r = np.hypot(m.nodes[..., 0], m.nodes[..., 1])
        assert r[0].min() == pytest.approx(0.5) and r[-1].max() == pytest.approx(20.0)
    m = Mesh.linspace(9, 7, 0.0, 10.0, -1.0, 3.0)
    assert np.array_equal(m.nodes, o.linspace_nodes(9, 7, 0.0, 10.0, -1.0, 3.0).reshape(10, 8, 2))


def test_stretched_radial_spacing_is_geometric():
    m = Mesh.cylinder(40, 8, 0.5, 20.0, 1.01)
    r = np.hypot(m.nodes[:, 0, 0], m.nodes[:, 0, 1])
    dr = np.diff(r)
    assert np.allclose(dr[1:] / dr[:-1], 1.01, rtol=1e-9)


def test_argument_errors_without_gpu():
    lib = _capi.load()
    cfg = _capi.Config(99, 0, 0, 0, 0, 0.5)
    h = C.c_void_p()
    assert lib.hc_context_create(C.byref(cfg), C.byref(h)) == _capi.HC_ERR_ARG
    assert b"flux" in lib.hc_last_error_string()
    cfg = _capi.Config(0, 0, 0, 0, 0, -1.0)
    assert lib.hc_context_create(C.byref(cfg), C.byref(h)) == _capi.HC_ERR_ARG
    assert lib.hc_residual(None, None) == _capi.HC_ERR_ARG
    assert lib.hc_set_low_mach(None, 0, 0, 1.0, 1.0) == _capi.HC_ERR_ARG
    bad = np.empty(4)
    assert lib.hc_mesh_cylinder_nodes(0, 4, 0.5, 1.0, 1.0, bad.ctypes.data_as(C.POINTER(C.c_double))) \
        == _capi.HC_ERR_ARG
