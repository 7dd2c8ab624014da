"""The allocation-free spectral radius (for callers that may not call
cudaMalloc) against the regular entry point, through the C ABI, on two calls in
a row with different data, so a stale scratch array would show.  Collected last
on purpose."""
import ctypes as C

import numpy as np
import pytest

from hyperboliconvergence_gb300 import _capi

pytestmark = pytest.mark.gpu


def _run(fn_name, lam_d, vol_d, n, out, stream):
    lib = _capi.load()
    fn = getattr(lib, fn_name)
    _capi.check(fn(C.c_void_p(lam_d.data_ptr()), C.c_void_p(vol_d.data_ptr()), n, C.c_void_p(out.data_ptr()),
                   C.c_void_p(stream)))


def test_noalloc_matches_regular_on_two_calls():
    import torch
    stream = torch.cuda.current_stream().cuda_stream
    for call, n in enumerate([3_000_001, 70_000]):
        rng = np.random.default_rng(100 + call)
        lam_d = torch.from_numpy(rng.uniform(0.1, 10.0, n)).cuda()
        vol_d = torch.from_numpy(rng.uniform(0.01, 1.0, n)).cuda()
        ref = torch.zeros(1, dtype=torch.float64, device="cuda")
        got = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
        _run("hc_spectral_radius", lam_d, vol_d, n, ref, stream)
        _run("hc_spectral_radius_noalloc", lam_d, vol_d, n, got, stream)
        torch.cuda.synchronize()
        # same kernels, same order of operations: equal bit for bit
        assert float(got.item()) == float(ref.item()), (call, got.item(), ref.item())


@pytest.mark.parametrize("n", [8_388_608, 2048 * 5 + 1, 1])
def test_noalloc_edges_against_host_maximum(n):
    """The largest accepted size (every one of the 4096 scratch entries in use), a size
    one cell past a whole number of 2048-cell blocks, and a single cell: both entry points
    equal the host's maximum of lambda/V (the same quotient, the fold from DBL_MIN), on two
    calls in a row."""
    import torch
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        rng = np.random.default_rng(200 + call + n % 97)
        lam = rng.uniform(0.1, 10.0, n)
        vol = rng.uniform(0.01, 1.0, n)
        want = max(np.finfo(np.float64).tiny, float(np.max(lam / vol)))
        lam_d, vol_d = torch.from_numpy(lam).cuda(), torch.from_numpy(vol).cuda()
        ref = torch.zeros(1, dtype=torch.float64, device="cuda")
        got = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
        _run("hc_spectral_radius", lam_d, vol_d, n, ref, stream)
        _run("hc_spectral_radius_noalloc", lam_d, vol_d, n, got, stream)
        torch.cuda.synchronize()
        assert float(ref.item()) == want, (call, ref.item(), want)
        assert float(got.item()) == want, (call, got.item(), want)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    import torch
    lib = _capi.load()
    x = torch.ones(1, dtype=torch.float64, device="cuda")
    p = C.c_void_p(x.data_ptr())
    assert lib.hc_spectral_radius_noalloc(p, p, 8_388_609, p, None) == _capi.HC_ERR_ARG
    assert b"exceeds" in lib.hc_last_error_string()
