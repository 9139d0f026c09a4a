"""Bounded device-side waits end with CS_ERR_TIMEOUT, not a hang, and leave the library usable.

The sort's decoupled look-back and the cooperative build's grid barrier spin on flags that other blocks publish; each
wait gives up after a bounded number of polls. cs_set_wait_limits makes a wait run out on an ordinary input: a small
poll limit and a wait on a flag that nothing sets (tile 1 of each sort pass waits for an entry that is never
published; block 0 of the build never arrives at its first barrier). Nothing here faults or hangs the GPU: the stalled
waits end after a few hundred polls, and a wait that gives up reads and writes only inside its call's buffers.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from gpu_util import neighbor_lists_equal, u32, u64, uniform

pytestmark = pytest.mark.gpu

STALL_SORT, STALL_BARRIER = 1, 2


@pytest.fixture
def limits(cs):
    def set_limits(sort_spins=0, barrier_spins=0, stall=0):
        rc = cs.lib.cs_set_wait_limits(C.c_uint32(sort_spins), C.c_uint32(barrier_spins), C.c_int(stall))
        assert rc == 0, cs.lib.cs_last_error().decode()

    yield set_limits
    set_limits()


def test_unknown_stall_mode_is_rejected(cs):
    assert cs.lib.cs_set_wait_limits(C.c_uint32(0), C.c_uint32(0), C.c_int(7)) == cs.CS_ERR_INVALID


def test_sort_lookback_timeout_then_normal_sort(cs, limits):
    rng = np.random.default_rng(5)
    n = 200_000  # 49 tiles of 4096 keys per pass
    keys = rng.integers(0, 1 << 63, size=n, dtype=np.uint64)
    dk = torch.from_numpy(keys.view(np.int64)).cuda()
    limits(sort_spins=256, stall=STALL_SORT)
    with pytest.raises(cs.CsError) as e:
        cs.sort_pairs(dk.clone())
    assert e.value.code == cs.CS_ERR_TIMEOUT
    assert "timed out" in str(e.value)
    limits()
    k, v = cs.sort_pairs(dk.clone())
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(u64(k), keys[order])
    assert np.array_equal(u32(v), order.astype(np.uint32))


def test_build_barrier_timeout_then_normal_build(cs, O, limits):
    x, y, z = uniform(O, 11, 100_000, -1.0, 1.0)
    box = O.make_box(-1.0, 1.0)
    keys = np.sort(O.sfc_keys(x, y, z, box))
    dk = torch.from_numpy(keys.view(np.int64)).cuda()
    limits(barrier_spins=512, stall=STALL_BARRIER)
    with pytest.raises(cs.CsError) as e:
        cs.compute_octree(dk, 16)
    assert e.value.code == cs.CS_ERR_TIMEOUT
    limits()
    tree, counts, _, iters = cs.compute_octree(dk, 16)
    rtree, rcounts, riters = O.compute_octree(keys, 16)
    assert np.array_equal(u64(tree), rtree)
    assert np.array_equal(u32(counts), rcounts)
    assert iters == riters


def test_pipeline_barrier_timeout_then_normal_run(cs, O, limits):
    n, bucket, ngmax = 60_000, 32, 64
    x, y, z = uniform(O, 12, n, -1.0, 1.0)
    h = np.full(n, 0.04)
    obox = O.make_box(-1.0, 1.0)
    ref = O.pipeline(x, y, z, h, obox, bucket, ngmax)
    tx, ty, tz, th = (torch.from_numpy(a).cuda() for a in (x, y, z, h))
    pipe = cs.Pipeline(64, 64, cs.HILBERT, bucket, ngmax, 1.0, 1.0, False, True)
    box = cs.make_box(-1.0, 1.0)
    limits(barrier_spins=512, stall=STALL_BARRIER)
    with pytest.raises(cs.CsError) as e:
        pipe.run(tx, ty, tz, th, box)
    assert e.value.code == cs.CS_ERR_TIMEOUT
    limits()
    r = pipe.run(tx, ty, tz, th, box)
    torch.cuda.synchronize()
    out = pipe.outputs()
    assert r.num_leaves == ref["leaves"].size - 1
    assert np.array_equal(u64(out["leaves"]), ref["leaves"])
    nb = u32(out["neighbors"]).reshape(n, ngmax)
    neighbor_lists_equal(nb, u32(out["neighbor_counts"]), ref["nb"], ref["nc"], ngmax)
