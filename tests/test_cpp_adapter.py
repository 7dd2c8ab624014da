"""The C++20 adapter (hcgpu::integrate with the reference's argument list)
compiles against include/hc.h and, on a GPU, matches the oracle."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "integrate_vortex.cpp")


def _build(tmp_path):
    from hyperboliconvergence_gb300 import _capi
    _capi.load()  # builds libhcgb300.so when missing
    libdir = os.path.join(ROOT, "hyperboliconvergence_gb300", "lib")
    exe = str(tmp_path / "integrate_vortex")
    cmd = ["g++", "-std=c++20", "-O2", "-fopenmp", "-ffp-contract=off",
           "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "hyperboliconvergence_gb300", "cpp", "inc"),
           "-I" + os.path.join(ROOT, "oracle"), SRC, "-L" + libdir, "-lhcgb300",
           "-Wl,-rpath," + libdir, "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_adapter_compiles(tmp_path):
    assert os.path.exists(_build(tmp_path))


@pytest.mark.gpu
def test_adapter_integrate_matches_oracle(tmp_path):
    r = subprocess.run([_build(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "rel_linf" in r.stdout


def _build_plugins(tmp_path):
    from hyperboliconvergence_gb300 import _capi
    _capi.load()
    libdir = os.path.join(ROOT, "hyperboliconvergence_gb300", "lib")
    exe = str(tmp_path / "adapter_plugins")
    cmd = ["g++", "-std=c++20", "-O2", "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "hyperboliconvergence_gb300", "cpp", "inc"),
           os.path.join(ROOT, "tests", "cpp", "adapter_plugins.cpp"), "-L" + libdir, "-lhcgb300",
           "-Wl,-rpath," + libdir, "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_flux_and_limiter_tags_against_reference_golden(tmp_path):
    """RoeFlux{}.flux(species, face, sl, sr) and the other flux tags, and the limiter tags'
    limit(a, b), on the reference's golden inputs (tests/golden/pointwise_golden.npz, made
    by the reference's own code): equal within 1e-13 of each vector's scale (the tags
    evaluate the library's pointwise code, whose operation order is the GPU kernels')."""
    import numpy as np
    g = np.load(os.path.join(ROOT, "tests", "golden", "pointwise_golden.npz"))
    exe = _build_plugins(tmp_path)
    sp, faces, ql, qr = g["species"], g["surface_out"], g["flux_ql"], g["flux_qr"]
    kinds = [0, 2, 3, 4, 5, 6]
    lines = [f"species 0 {float(sp[0])!r} {float(sp[1])!r} {float(sp[2])!r}"]
    for k in kinds:
        for m in range(len(faces)):
            vals = " ".join(repr(float(x)) for x in (*faces[m], *ql[m], *qr[m]))
            lines.append(f"flux {k} {vals}")
    lim_kinds = [0, 1, 2, 3, 4, 5, 6, 8, 9]
    for k in lim_kinds:
        for a, b in g["limit_ab"]:
            lines.append(f"limit {k} {float(a)!r} {float(b)!r}")
    r = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    out = r.stdout.splitlines()
    assert not any("differ" in x for x in out), [x for x in out if "differ" in x][:3]
    pos = 0
    for k in kinds:
        got = np.array([[float(x) for x in out[pos + m].split()] for m in range(len(faces))])
        pos += len(faces)
        want = g[f"flux_{k}"]
        scale = np.maximum(np.abs(want).max(axis=1, keepdims=True), 1e-300)
        assert np.all(np.abs(got - want) <= 1e-13 * scale), (k, np.abs((got - want) / scale).max())
    for k in lim_kinds:
        got = np.array([float(out[pos + m]) for m in range(len(g["limit_ab"]))])
        pos += len(g["limit_ab"])
        want = g[f"limit_{k}"]
        fin = np.isfinite(want)
        assert np.array_equal(np.isfinite(got), fin), k
        scale = np.maximum(np.abs(g["limit_ab"]).max(axis=1), 1e-300)
        assert np.all(np.abs(got[fin] - want[fin]) <= 1e-15 * scale[fin]), (k, np.abs(got - want)[fin].max())


@pytest.mark.gpu
def test_cylinder2d_shaped_driver_with_bc_tuple(tmp_path):
    """A driver shaped like the reference's cylinder2D.cpp, BC tuple included, runs through
    hcgpu::integrate; a tuple without a condition for one side's type is refused."""
    r = subprocess.run([_build_plugins(tmp_path), "--run"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "refused 1" in r.stdout
