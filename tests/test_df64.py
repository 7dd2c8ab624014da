"""Double-float arithmetic (hc_df64.cuh) against double on the host: every
operation within 2^-45 relative (operand-relative for additions)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_df64_arithmetic_accuracy(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "df64_check")
    subprocess.run([nvcc, "-std=c++17", "-O2", "-o", exe, os.path.join(ROOT, "tests", "cpp", "df64_check.cu")],
                   check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr


def test_adjoint_pointwise_derivatives(tmp_path):
    """Reverse pointwise functions (hc_adjoint.cuh) against central differences of
    the forward ones on the host: limiter derivatives away from their kinks and
    the Roe and Rusanov face-flux adjoints, within 1e-6."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "adjoint_pointwise_check")
    subprocess.run([nvcc, "-std=c++17", "-O2", "-o", exe,
                    os.path.join(ROOT, "tests", "cpp", "adjoint_pointwise_check.cu")], check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
