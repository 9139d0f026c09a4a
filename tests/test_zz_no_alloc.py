"""The allocation-free sort entry point (cs_sort_pairs_noalloc_u64) against the allocating one (cs_sort_pairs_u64).

cs_sort_pairs_noalloc_u64 serves callers that cannot allocate device memory when they sort (device memory reserved
up front by their own pool, or a loop that cannot take cudaMalloc's implicit synchronisation): its temporaries live in
a fixed device array inside the library. This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _noalloc_sort(cs, keys, values, iota):
    fn = cs.lib.cs_sort_pairs_noalloc_u64
    return fn(C.c_void_p(torch.cuda.current_stream().cuda_stream), C.c_void_p(keys.data_ptr()),
              C.c_void_p(values.data_ptr()), C.c_size_t(keys.numel()), 0, 64, int(iota))


@pytest.mark.parametrize("iota", [True, False])
def test_noalloc_sort_matches_allocating_sort_twice(cs, iota):
    rng = np.random.default_rng(123)
    max_n = 262144  # CS_SORT_NOALLOC_MAX_N
    for call, n in enumerate((max_n, 100003)):  # two calls in a row on the shared scratch array
        keys = rng.integers(0, 1 << 63, size=n, dtype=np.uint64)
        keys[rng.integers(0, n, size=n // 4)] = keys[rng.integers(0, n, size=n // 4)]  # duplicates: stability
        vals = rng.integers(0, 1 << 31, size=n, dtype=np.int64).astype(np.int32)
        dk = torch.from_numpy(keys.view(np.int64)).cuda()
        dv = torch.from_numpy(vals).cuda()

        ref_k, ref_v = cs.sort_pairs(dk.clone(), dv.clone(), iota=iota)
        k2, v2 = dk.clone(), dv.clone()
        rc = _noalloc_sort(cs, k2, v2, iota)
        assert rc == 0, cs.lib.cs_last_error().decode()
        torch.cuda.synchronize()
        # integer work: the results must be identical, bit for bit
        assert torch.equal(k2, ref_k), f"keys differ on call {call}"
        assert torch.equal(v2, ref_v), f"values differ on call {call}"


def test_noalloc_sort_allocates_no_device_memory(cs):
    """After warm-up calls (n = 0, which loads the fixed array and the sort kernels, then one full-size sort, which
    also settles the kernels' per-thread stack reservation), a second full-size call on new inputs leaves the device's
    free memory unchanged."""
    assert _noalloc_sort(cs, torch.empty(0, dtype=torch.int64, device="cuda"),
                         torch.empty(0, dtype=torch.int32, device="cuda"), True) == 0, cs.lib.cs_last_error().decode()
    rng = np.random.default_rng(7)
    n = 262144
    wk = torch.from_numpy(rng.integers(0, 1 << 63, size=n, dtype=np.uint64).view(np.int64)).cuda()
    wv = torch.empty(n, dtype=torch.int32, device="cuda")
    assert _noalloc_sort(cs, wk, wv, True) == 0, cs.lib.cs_last_error().decode()
    keys = rng.integers(0, 1 << 63, size=n, dtype=np.uint64)
    dk = torch.from_numpy(keys.view(np.int64)).cuda()
    dv = torch.empty(n, dtype=torch.int32, device="cuda")
    ref_k = torch.from_numpy(np.sort(keys).view(np.int64)).cuda()
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    rc = _noalloc_sort(cs, dk, dv, True)
    assert rc == 0, cs.lib.cs_last_error().decode()
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before, f"device free memory changed by {free_before - free_after} bytes"
    assert torch.equal(dk, ref_k)


def test_noalloc_sort_refuses_a_capturing_stream(cs):
    n = 1024
    k = torch.zeros(n, dtype=torch.int64, device="cuda")
    v = torch.zeros(n, dtype=torch.int32, device="cuda")
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    rc = None
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            rc = _noalloc_sort(cs, k, v, True)
    assert rc == cs.CS_ERR_INVALID
    assert "captured" in cs.lib.cs_last_error().decode()


def test_noalloc_sort_rejects_sizes_beyond_limit(cs):
    n = 262144 + 1
    k = torch.zeros(n, dtype=torch.int64, device="cuda")
    v = torch.zeros(n, dtype=torch.int32, device="cuda")
    rc = _noalloc_sort(cs, k, v, True)
    assert rc == cs.CS_ERR_INVALID
    assert "exceeds" in cs.lib.cs_last_error().decode()
