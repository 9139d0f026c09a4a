"""The state-table Hilbert encoder of the key kernels (iHilbertByTable with the compile-time table) equals the
per-level encoder (iHilbert), checked on the host with nvcc (no GPU): 4M random coordinates and a lattice."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")


@pytest.mark.skipif(not (os.path.exists(NVCC) or shutil.which("nvcc")), reason="nvcc not available")
def test_table_encoder_equals_level_encoder(tmp_path):
    exe = str(tmp_path / "hilbert_table_check")
    nvcc = NVCC if os.path.exists(NVCC) else shutil.which("nvcc")
    r = subprocess.run([nvcc, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-I",
                        os.path.join(ROOT, "cornerstone-octree_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "hilbert_table_check.cu"), "-o", exe],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0" in r.stdout
