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
