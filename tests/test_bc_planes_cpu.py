"""Host check of the boundary-plane enumeration (ia_bc.cuh::bc_plane_cell) that the velocity BC,
the periodic pressure ghosts and the VOF ghost fills launch over: compiled for the host with nvcc
and run (no GPU needed)."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_boundary_plane_enumeration_covers_exactly_the_planes():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "bc_planes_check")
        subprocess.run([nvcc, "-std=c++17", "-O1", "-o", exe, os.path.join(HERE, "host", "bc_planes_check.cu")],
                       check=True, capture_output=True, timeout=300)
        r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stdout + r.stderr
