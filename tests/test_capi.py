"""The C-ABI library loads (no GPU needed) and exports every entry point that include/cstone_gb300.h declares; the
C++ shim compiles against the reference headers where they exist. CPU only: no compute calls."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "cstone_gb300.h")
LIB = os.path.join(ROOT, "cornerstone-octree_gb300", "cstone_gb300", "libcstone_gb300.so")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(cs_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB):
        import sys

        sys.path.insert(0, os.path.join(ROOT, "cornerstone-octree_gb300"))
        import build

        build.build()
    return ctypes.CDLL(LIB)


def test_header_declares_entry_points():
    names = declared_functions()
    assert len(names) > 40
    for expected in ("cs_sfc_keys_hilbert_u64_f64", "cs_sort_pairs_u64", "cs_compute_octree_u64",
                     "cs_build_octree_u64", "cs_find_halos_u64_f64", "cs_find_neighbors_f64", "cs_pipeline_run"):
        assert expected in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_error_string_without_gpu(lib):
    lib.cs_last_error.restype = ctypes.c_char_p
    assert isinstance(lib.cs_last_error(), bytes)
    assert lib.cs_version() >= 100


def test_invalid_arguments_are_rejected_without_gpu(lib):
    lib.cs_last_error.restype = ctypes.c_char_p
    # null box
    rc = lib.cs_sfc_keys_hilbert_u64_f64(None, None, None, None, None, ctypes.c_size_t(10), None, 0)
    assert rc == 1 and b"box" in lib.cs_last_error()
    # pipeline with a zero bucket size
    p = ctypes.c_void_p()

    class Cfg(ctypes.Structure):
        _fields_ = [("sfc_kind", ctypes.c_int), ("bucket_size", ctypes.c_uint), ("max_count", ctypes.c_uint32),
                    ("ngmax", ctypes.c_uint), ("search_ext", ctypes.c_float), ("halo_search_ext", ctypes.c_float),
                    ("do_halos", ctypes.c_int), ("do_neighbors", ctypes.c_int)]

    assert lib.cs_pipeline_create(ctypes.byref(p), 64, 64, ctypes.byref(Cfg(1, 0, 0xFFFFFFFF, 10, 1, 1, 0, 1))) == 1
    # no-alloc sort beyond its fixed limit
    assert lib.cs_sort_pairs_noalloc_u64(None, None, None, ctypes.c_size_t(1 << 20), 0, 64, 1) == 1
    assert b"exceeds" in lib.cs_last_error()


def test_cpp_shim_compiles_and_links_against_reference_headers(tmp_path, lib):
    """the header-only shim defines the reference's own declarations (checked by its headers) and every C-ABI call
    it makes resolves in the library"""
    ref = "/root/reference/include"
    if not os.path.isdir(ref):
        pytest.skip("reference headers not present")
    src = tmp_path / "main.cpp"
    src.write_text('''#include "cstone_gb300/cstone_gpu_shim.hpp"
int main(int argc, char**)
{
    if (argc > 5)
    {
        auto e = cstone::execution::gpuStream(0);
        cstone::Box<double> b(0, 1);
        cstone::computeSfcKeys(e, (double*)0, (double*)0, (double*)0, (cstone::HilbertKey<uint64_t>*)0, 0, b);
        cstone::computeNodeOpsGpu(e, (uint64_t*)0, 0, (unsigned*)0, 64u, (int*)0);
    }
    return 0;
}
''')
    obj, exe = tmp_path / "main.o", tmp_path / "a.out"
    inc = ["-I", ref, "-I", os.path.join(ROOT, "include"), "-I", "/usr/local/cuda/include"]
    r = subprocess.run(["g++", "-std=c++20", "-c", str(src), "-o", str(obj), *inc], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run(["g++", str(obj), "-o", str(exe), "-L", os.path.dirname(LIB), "-lcstone_gb300",
                        "-L", "/usr/local/cuda/lib64", "-lcudart"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    syms = subprocess.run(["nm", "-C", str(obj)], capture_output=True, text=True).stdout
    for name in ("cstone::computeSfcKeys", "cstone::sortByKey", "cstone::computeNodeCountsGpu",
                 "cstone::computeNodeOpsGpu", "cstone::rebalanceTreeGpu", "cstone::buildOctreeGpu",
                 "cstone::computeGeoCentersGpu", "cstone::computeBoundingBoxGpu", "cstone::findHalosGpu",
                 "cstone::exclusiveScan"):
        assert name in syms, name
