"""Host check of the float-float arithmetic the momentum kernels compute in (csrc/ff.cuh): the same
source compiled for the host with nvcc (FMA contraction off) and checked against exact long-double
results with the error bounds stated in tests/host/ff_check.cu (no GPU needed)."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_float_float_operations_within_stated_bounds():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "ff_check")
        subprocess.run([nvcc, "-std=c++17", "-O2", "-Xcompiler", "-ffp-contract=off", "-o", exe,
                        os.path.join(HERE, "host", "ff_check.cu")], check=True, capture_output=True, timeout=300)
        r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
