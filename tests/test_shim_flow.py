"""The cstone:: shim run as a user of the reference would: tests/shim/reference_flow.cu is written against the
reference's GPU API and drives libcstone_gb300 only through it (keys, sortByKey, gather, updateOctreeGpu to
convergence, buildOctreeGpu, computeGeoCentersGpu, computeBoundingBoxGpu, findHalosGpu, and a NeighborhoodBuilder's
build().ijLoop()).

- CPU: the program compiles against the reference's own headers (their declarations check the shim), where present.
- GPU: the same program, built with -DCSTONE_GB300_STANDALONE (no reference headers on the GPU host), runs and its
  outputs equal the oracle's, bit for bit (the program is compiled without fused multiply-add, so its density
  interaction evaluates the oracle's expression).
"""
import os
import subprocess
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "shim", "reference_flow.cu")
LIBDIR = os.path.join(ROOT, "cornerstone-octree_gb300", "cstone_gb300")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
FLAGS = ["-std=c++20", "--expt-relaxed-constexpr", "--extended-lambda", "-gencode", "arch=compute_103a,code=sm_103a",
         "-fmad=false", "-I", os.path.join(ROOT, "include")]


def test_flow_compiles_against_reference_headers(tmp_path):
    ref = "/root/reference/include"
    if not os.path.isdir(ref):
        pytest.skip("reference headers not present")
    r = subprocess.run([NVCC, *FLAGS, "-I", ref, "-c", SRC, "-o", str(tmp_path / "flow.o")], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr[-4000:]


def test_flow_compiles_standalone(tmp_path):
    r = subprocess.run([NVCC, *FLAGS, "-DCSTONE_GB300_STANDALONE", "-c", SRC, "-o", str(tmp_path / "flow.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


@pytest.mark.gpu
def test_flow_runs_on_gpu_and_matches_oracle(cs, O):
    n, bucket = 30_000, 16
    x, y, z = O.plummer(41, n)
    lo, hi = (x.min(), y.min(), z.min()), (x.max(), y.max(), z.max())
    r = np.sqrt(x * x + y * y + z * z)
    h = 0.05 + 0.1 * r
    m = np.random.default_rng(2).uniform(0.5, 1.5, n)
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "flow")
        b = subprocess.run([NVCC, *FLAGS, "-DCSTONE_GB300_STANDALONE", SRC, "-o", exe, "-L", LIBDIR,
                            "-lcstone_gb300", f"-Xlinker=-rpath,{LIBDIR}"], capture_output=True, text=True)
        assert b.returncode == 0, b.stderr[-4000:]
        inp = os.path.join(d, "in.bin")
        with open(inp, "wb") as f:
            f.write(np.int64(n).tobytes())
            f.write(np.array(lo, np.float64).tobytes())
            f.write(np.array(hi, np.float64).tobytes())
            f.write(np.array([bucket, 0], np.int32).tobytes())
            for a in (x, y, z, h, m):
                f.write(np.ascontiguousarray(a, np.float64).tobytes())
        run = subprocess.run([exe, inp, d], capture_output=True, text=True, timeout=300)
        assert run.returncode == 0, run.stderr[-4000:]

        def rd(name, dt):
            return np.fromfile(os.path.join(d, name), dt)

        L, N, iters, first, last = (int(v) for v in open(os.path.join(d, "meta.txt")).read().split())
        obox = O.make_box(lo, hi)
        ref = O.pipeline(x, y, z, h, obox, bucket, 0, with_neighbors=False)
        assert np.array_equal(rd("keys", np.uint64), ref["sorted_keys"])
        assert np.array_equal(rd("order", np.uint32), ref["perm"])
        assert np.array_equal(rd("leaves", np.uint64), ref["leaves"])
        assert np.array_equal(rd("counts", np.uint32), ref["counts"])
        assert iters == ref["iterations"]
        tr = ref["tree"]
        assert (L, N) == (tr.num_leaves, tr.num_nodes)
        assert np.array_equal(rd("prefixes", np.uint64), tr.prefixes)
        assert np.array_equal(rd("child_offsets", np.int32), tr.child_offsets)
        assert np.array_equal(rd("centers", np.float64).reshape(N, 3), ref["centers"])
        assert np.array_equal(rd("sizes", np.float64).reshape(N, 3), ref["sizes"])
        l2i = tr.leaf_to_internal[tr.num_internal:]
        xs, ys, zs, hs, ms = (a[ref["perm"]] for a in (x, y, z, h, m))
        sc, ss = O.search_boxes(xs, ys, zs, hs, ref["layout"], first, last, 2.0, l2i, ref["centers"])
        flags = O.find_halos(tr, ref["centers"], ref["sizes"], sc, ss, obox, first, last)
        assert np.array_equal(rd("flags", np.uint8), flags)
        rho = O.ijloop_density_all(xs, ys, zs, hs, ms, obox)
        assert np.array_equal(rd("rho", np.float64), rho)
