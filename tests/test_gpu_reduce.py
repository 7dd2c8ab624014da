"""hc_spectral_radius: max over cells of lambda/V, computed on the device from
device arrays, against numpy on the same values (exact: division is IEEE on both)."""
import ctypes as C

import numpy as np
import pytest

from hyperboliconvergence_gb300 import _capi

pytestmark = pytest.mark.gpu


def spectral_radius_host(lam, vol):
    return max(np.finfo(np.float64).tiny, float(np.max(lam / vol)))


@pytest.mark.parametrize("n", [1, 7, 2048, 2049, 524288, 1_000_003])
def test_spectral_radius_matches_numpy(n):
    import torch
    rng = np.random.default_rng(n)
    lam = rng.uniform(0.1, 10.0, n)
    vol = rng.uniform(0.01, 1.0, n)
    lam_d = torch.from_numpy(lam).cuda()
    vol_d = torch.from_numpy(vol).cuda()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    lib = _capi.load()
    stream = torch.cuda.current_stream().cuda_stream
    _capi.check(lib.hc_spectral_radius(C.c_void_p(lam_d.data_ptr()), C.c_void_p(vol_d.data_ptr()), n,
                                       C.c_void_p(out.data_ptr()), C.c_void_p(stream)))
    torch.cuda.synchronize()
    assert float(out.item()) == spectral_radius_host(lam, vol)


def test_spectral_radius_rejects_bad_arguments():
    lib = _capi.load()
    assert lib.hc_spectral_radius(None, None, 10, None, None) == _capi.HC_ERR_ARG
