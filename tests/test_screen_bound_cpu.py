"""Host check with nvcc (no GPU) of the error bound behind the FP32 screen of the FP64 search boxes: truncEstimate's
accuracy and range, the bound |RN32(pt -+ rt) - RN64(p -+ r)| <= 24 u (|pt| + |rt|) + 2^-98 for double and float h,
shadow and truncated estimates over all exponents, and the leaf-centre bound (tests/screen_bound_check.cu)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")


@pytest.mark.skipif(not (os.path.exists(NVCC) or shutil.which("nvcc")), reason="nvcc not available")
def test_search_box_screen_bound(tmp_path):
    exe = str(tmp_path / "screen_bound_check")
    nvcc = NVCC if os.path.exists(NVCC) else shutil.which("nvcc")
    r = subprocess.run([nvcc, "-O2", "-std=c++17", "-Xcompiler", "-ffp-contract=off", "-I",
                        os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "cornerstone-octree_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "screen_bound_check.cu"), "-o", exe],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("mismatches 0") == 3, r.stdout
