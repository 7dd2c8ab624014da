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
