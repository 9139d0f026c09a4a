"""Host checks with nvcc (no GPU) of two FP64-free forms of FP64 arithmetic: the integer form of the key quantisation
(quantizeAxis) against the reference's expression int(floor(x m) - o), on boxes with integer, near-integer and
arbitrary offsets and points on, beside and between cell boundaries, inside and outside the box; and the float split
of a double (splitDouble) against RN_float(x) and RN_float(x - hi), on every exponent, rounding ties and carries."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")


@pytest.mark.skipif(not (os.path.exists(NVCC) or shutil.which("nvcc")), reason="nvcc not available")
def test_integer_quantisation_equals_fp64_expression(tmp_path):
    exe = str(tmp_path / "quantize_check")
    nvcc = NVCC if os.path.exists(NVCC) else shutil.which("nvcc")
    r = subprocess.run([nvcc, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-I",
                        os.path.join(ROOT, "cornerstone-octree_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "quantize_check.cu"), "-o", exe],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "checked" in r.stdout and r.stdout.count("mismatches 0") == 2
