"""Neighbour lists returned in compressed sparse row form, against the oracle's ngmax-strided rows.

findNeighbors (findneighbors.hpp:156-177) stores particle i's first min(nc_i, ngmax) neighbours in row i of an
n x ngmax array. cs_neighbors_csr compacts those rows on the device; cs_pipeline_run_host_csr runs the whole path from
host buffers and writes the compacted lists straight into pinned host memory. Both must reproduce the oracle's rows
exactly (integer work: bit for bit), including truncated rows (nc > ngmax) and empty ones.
"""
import numpy as np
import pytest
import torch

from gpu_util import u32, uniform

pytestmark = pytest.mark.gpu


def _oracle_csr(nb, nc, ngmax):
    m = np.minimum(nc, ngmax).astype(np.int64)
    off = np.zeros(nc.size + 1, np.int64)
    np.cumsum(m, out=off[1:])
    lst = np.concatenate([nb[i, : m[i]] for i in range(nc.size)]) if nc.size else np.zeros(0, np.uint32)
    return off, lst.astype(np.uint32)


def _case(O, n, ngmax, h, seed):
    x, y, z = uniform(O, seed, n, -1.0, 1.0)
    hh = np.full(n, h)
    # a few isolated particles (empty rows) and a dense clump (rows truncated at ngmax)
    x[:5] = 50.0 + np.arange(5)
    y[:5] = 50.0
    z[:5] = 50.0
    x[5:400] = 0.001 * np.arange(395) / 395
    y[5:400] = 0.0
    z[5:400] = 0.0
    box = O.make_box(-1.0, 60.0)
    ref = O.pipeline(x, y, z, hh, box, 16, ngmax)
    return x, y, z, hh, ref


def test_neighbors_csr_on_device_matches_oracle(cs, O):
    n, ngmax = 30_000, 48
    x, y, z, h, ref = _case(O, n, ngmax, 0.05, 3)
    assert (ref["nc"] > ngmax).any() and (ref["nc"] == 0).any()
    nb = torch.from_numpy(ref["nb"].astype(np.int64).astype(np.int32)).cuda()
    nc = torch.from_numpy(ref["nc"].astype(np.int32)).cuda()
    off, lst = cs.neighbors_csr(nb, nc, ngmax)
    torch.cuda.synchronize()
    roff, rlst = _oracle_csr(ref["nb"], ref["nc"], ngmax)
    assert np.array_equal(off.cpu().numpy(), roff)
    assert np.array_equal(u32(lst[: roff[-1]]), rlst)


def test_pipeline_run_host_csr_matches_oracle(cs, O):
    n, ngmax = 30_000, 48
    x, y, z, h, ref = _case(O, n, ngmax, 0.05, 4)
    roff, rlst = _oracle_csr(ref["nb"], ref["nc"], ngmax)
    hx, hy, hz, hh = (torch.from_numpy(a).pin_memory() for a in (x, y, z, h))
    off = torch.empty(n + 1, dtype=torch.int64).pin_memory()
    lst = torch.empty(int(roff[-1]) + 7, dtype=torch.int32).pin_memory()
    nc = torch.empty(n, dtype=torch.int32).pin_memory()
    pipe = cs.Pipeline(64, 64, cs.HILBERT, 16, ngmax, 1.0, 1.0, False, True)
    box = cs.make_box(-1.0, 60.0)
    for asynchronous in (False, True, True):  # the async calls reuse the same host buffers
        pipe.run_host_csr(hx, hy, hz, hh, box, (0, 0), off, lst, nc_out=nc, asynchronous=asynchronous)
    pipe.wait()
    assert np.array_equal(nc.numpy().view(np.uint32), ref["nc"])
    assert np.array_equal(off.numpy(), roff)
    assert np.array_equal(lst.numpy()[: roff[-1]].view(np.uint32), rlst)


def test_pipeline_run_host_csr_reports_a_small_list_buffer(cs, O):
    n, ngmax = 30_000, 48
    x, y, z, h, ref = _case(O, n, ngmax, 0.05, 5)
    roff, _ = _oracle_csr(ref["nb"], ref["nc"], ngmax)
    hx, hy, hz, hh = (torch.from_numpy(a).pin_memory() for a in (x, y, z, h))
    off = torch.empty(n + 1, dtype=torch.int64).pin_memory()
    lst = torch.empty(int(roff[-1]) // 2, dtype=torch.int32).pin_memory()
    pipe = cs.Pipeline(64, 64, cs.HILBERT, 16, ngmax, 1.0, 1.0, False, True)
    box = cs.make_box(-1.0, 60.0)
    with pytest.raises(cs.CsError) as e:
        pipe.run_host_csr(hx, hy, hz, hh, box, (0, 0), off, lst)
    assert e.value.code == cs.CS_ERR_CAPACITY
    assert int(off[-1]) == int(roff[-1])
    # the flag is cleared by the wait that reported it: a large enough buffer works again
    big = torch.empty(int(roff[-1]), dtype=torch.int32).pin_memory()
    pipe.run_host_csr(hx, hy, hz, hh, box, (0, 0), off, big)
    assert np.array_equal(off.numpy(), roff)


@pytest.mark.parametrize("shift", [1, 2, 3])
def test_pipeline_run_host_csr_unaligned_list_buffer(cs, O, shift):
    """a list buffer that does not start on a 16-byte boundary (the lists are written with 16-byte stores from the
    first aligned entry): every entry lands in place, nothing outside the buffer is touched"""
    n, ngmax = 30_000, 48
    x, y, z, h, ref = _case(O, n, ngmax, 0.05, 6 + shift)
    roff, rlst = _oracle_csr(ref["nb"], ref["nc"], ngmax)
    assert roff[-1] > 3 * 4096
    hx, hy, hz, hh = (torch.from_numpy(a).pin_memory() for a in (x, y, z, h))
    off = torch.empty(n + 1, dtype=torch.int64).pin_memory()
    raw = torch.full((int(roff[-1]) + 16,), -7, dtype=torch.int32).pin_memory()
    lst = raw[shift:]
    pipe = cs.Pipeline(64, 64, cs.HILBERT, 16, ngmax, 1.0, 1.0, False, True)
    pipe.run_host_csr(hx, hy, hz, hh, cs.make_box(-1.0, 60.0), (0, 0), off, lst)
    assert np.array_equal(off.numpy(), roff)
    assert np.array_equal(lst.numpy()[: roff[-1]].view(np.uint32), rlst)
    assert (raw.numpy()[:shift] == -7).all() and (raw.numpy()[shift + roff[-1]:] == -7).all()


def test_list_copy_survives_the_next_runs(cs, O):
    """an asynchronous call's lists are still being copied to host memory when the next runs (or a step) start: the
    copy reads the compacted lists, in buffers of their own, so the host lists are those of the first call"""
    n, ngmax = 30_000, 48
    xa, ya, za, ha, refa = _case(O, n, ngmax, 0.05, 11)
    xb, yb, zb, hb, refb = _case(O, n, ngmax, 0.05, 12)
    roff, rlst = _oracle_csr(refa["nb"], refa["nc"], ngmax)
    hx, hy, hz, hh = (torch.from_numpy(a).pin_memory() for a in (xa, ya, za, ha))
    dx, dy, dz, dh = (torch.from_numpy(a).cuda() for a in (xb, yb, zb, hb))
    box = cs.make_box(-1.0, 60.0)
    pipe = cs.Pipeline(64, 64, cs.HILBERT, 16, ngmax, 1.0, 1.0, False, True)
    for follow in ("run", "run2", "step"):
        off = torch.empty(n + 1, dtype=torch.int64).pin_memory()
        lst = torch.empty(int(roff[-1]) + 5, dtype=torch.int32).pin_memory()
        pipe.run_host_csr(hx, hy, hz, hh, box, (0, 0), off, lst, asynchronous=True)
        if follow == "step":
            pipe.step(dx, dy, dz, dh, box)
        else:
            for _ in range(1 if follow == "run" else 2):
                pipe.run(dx, dy, dz, dh, box)
        pipe.wait()
        torch.cuda.synchronize()
        assert np.array_equal(off.numpy(), roff), follow
        assert np.array_equal(lst.numpy()[: roff[-1]].view(np.uint32), rlst), follow
        out = pipe.outputs()
        assert np.array_equal(u32(out["neighbor_counts"]), refb["nc"]), follow


def test_pipeline_run_host_with_pageable_outputs(cs, O):
    """counts, flags and lists into ordinary (pageable) host memory: the copies that a kernel makes into pinned buffers
    go through the copy engine instead, with the same results"""
    n, ngmax = 30_000, 48
    x, y, z, h, ref = _case(O, n, ngmax, 0.05, 21)
    roff, rlst = _oracle_csr(ref["nb"], ref["nc"], ngmax)
    hx, hy, hz, hh = (torch.from_numpy(a).pin_memory() for a in (x, y, z, h))
    off = torch.empty(n + 1, dtype=torch.int64)
    lst = torch.empty(int(roff[-1]) + 3, dtype=torch.int32)
    nc = torch.empty(n, dtype=torch.int32)
    assert not (off.is_pinned() or lst.is_pinned() or nc.is_pinned())
    pipe = cs.Pipeline(64, 64, cs.HILBERT, 16, ngmax, 1.0, 1.0, False, True)
    pipe.run_host_csr(hx, hy, hz, hh, cs.make_box(-1.0, 60.0), (0, 0), off, lst, nc_out=nc)
    assert np.array_equal(nc.numpy().view(np.uint32), ref["nc"])
    assert np.array_equal(off.numpy(), roff)
    assert np.array_equal(lst.numpy()[: roff[-1]].view(np.uint32), rlst)
