"""GPU parity of the whole path (cs_pipeline_*) against the CPU oracle run stage by stage on the same inputs."""
import numpy as np
import pytest
import torch

from gpu_util import keys_u, neighbor_lists_equal, to_dev, u32

pytestmark = pytest.mark.gpu


def _check_against_oracle(cs, O, x, y, z, h, lo, hi, bnd, bucket, ngmax, focus, coord_bits=64, key_bits=64):
    obox = O.make_box(lo, hi, bnd)
    t, ref = O.timed_pipeline(x, y, z, h, obox, bucket, ngmax, focus, key_bits=key_bits)
    pipe = cs.Pipeline(coord_bits, key_bits, cs.HILBERT, bucket, ngmax, 1.0, 1.0, focus[1] > focus[0], True)
    tx, ty, tz, th = to_dev(x, y, z, h)
    res = pipe.run(tx, ty, tz, th, cs.make_box(lo, hi, bnd), focus)
    out = pipe.outputs()
    torch.cuda.synchronize()
    assert np.array_equal(keys_u(out["sorted_keys"]), ref["sorted_keys"])
    assert np.array_equal(u32(out["order"]), ref["perm"])
    assert np.array_equal(keys_u(out["leaves"]), ref["leaves"])
    assert np.array_equal(u32(out["counts"]), ref["counts"])
    assert res.iterations == ref["iterations"]
    tree = ref["tree"]
    assert np.array_equal(keys_u(out["prefixes"]), tree.prefixes)
    assert np.array_equal(out["child_offsets"].cpu().numpy(), tree.child_offsets)
    assert np.array_equal(out["parents"].cpu().numpy(), tree.parents)
    assert np.array_equal(out["internal_to_leaf"].cpu().numpy(), tree.internal_to_leaf)
    assert np.array_equal(out["leaf_to_internal"].cpu().numpy(), tree.leaf_to_internal)
    assert np.array_equal(out["centers"].cpu().numpy(), ref["centers"])
    assert np.array_equal(out["sizes"].cpu().numpy(), ref["sizes"])
    if ref["flags"] is not None:
        first, last, rsc, rss = ref["search_boxes"]
        assert np.array_equal(out["search_centers"][first:last].cpu().numpy(), rsc[first:last])
        assert np.array_equal(out["search_sizes"][first:last].cpu().numpy(), rss[first:last])
        assert np.array_equal(out["halo_flags"].cpu().numpy(), ref["flags"])
    neighbor_lists_equal(u32(out["neighbors"]), u32(out["neighbor_counts"]), ref["nb"], ref["nc"], ngmax)
    return res


def test_pipeline_uniform_cube(cs, O):
    """the uniform-cube workload at reduced size: U[-1,1]^3, constant h, Hilbert64, bucket 64, ngmax 150"""
    n = 1 << 17
    x, y, z = (O.philox_uniform(1, s, n, -1.0, 1.0) for s in range(3))
    h = np.full(n, 0.028 * (2 ** 20 / n) ** (1 / 3))  # ~93 neighbours, as h = 0.028 at N = 2^20
    res = _check_against_oracle(cs, O, x, y, z, h, -1.0, 1.0, 0, 64, 150, (0, 0))
    assert res.num_leaves > 0


def test_pipeline_uniform_cube_full_size(cs, O):
    """the CPU-runnable plain build at its full size: N = 2^20 FP64 U[-1,1]^3, h = 0.028, Hilbert64, stable sort,
    bucket 64 from the root to convergence, link, neighbours with ngmax 150; everything bit-exact against the oracle"""
    n = 1 << 20
    x, y, z = (O.philox_uniform(20, s, n, -1.0, 1.0) for s in range(3))
    h = np.full(n, 0.028)
    res = _check_against_oracle(cs, O, x, y, z, h, -1.0, 1.0, 0, 64, 150, (0, 0))
    assert res.num_leaves > 0


def test_pipeline_plummer(cs, O):
    """the 16M Plummer workload at reduced size: Plummer, tight box, adaptive h (~100 neighbours), halos in the first
    quarter of the key space, ngmax 200"""
    n = 1 << 17
    x, y, z = O.plummer(5, n)
    lo, hi = (x.min(), y.min(), z.min()), (x.max(), y.max(), z.max())
    h = O.h_for_k_neighbors_cpu(x, y, z, O.make_box(lo, hi), 100)
    res = _check_against_oracle(cs, O, x, y, z, h, lo, hi, 0, 64, 200, (0, 1 << 61))
    assert res.focus_last > res.focus_first


def test_pipeline_periodic_f64(cs, O):
    n = 1 << 16
    x, y, z = (O.philox_uniform(3, s, n, 0.0, 1.0) for s in range(3))
    h = np.full(n, 1.2 * n ** (-1 / 3))
    _check_against_oracle(cs, O, x, y, z, h, 0.0, 1.0, 1, 32, 150, (0, 1 << 61))


@pytest.mark.parametrize("key_bits, focus", [(64, (0, 1 << 61)), (32, (0, 1 << 28))])
def test_pipeline_plummer_f32_halos(cs, O, key_bits, focus):
    """FP32 coordinates with halos: the plain search boxes and the list-driven halo walks without the FP64 filter,
    64- and 32-bit keys"""
    n = 1 << 16
    x, y, z = (a.astype(np.float32) for a in O.plummer(11, n))
    lo, hi = (float(x.min()), float(y.min()), float(z.min())), (float(x.max()), float(y.max()), float(z.max()))
    h = O.h_for_k_neighbors_cpu(x.astype(np.float64), y.astype(np.float64), z.astype(np.float64),
                                O.make_box(lo, hi), 60).astype(np.float32)
    res = _check_against_oracle(cs, O, x, y, z, h, lo, hi, 0, 32, 100, focus, coord_bits=32, key_bits=key_bits)
    assert res.focus_last > res.focus_first


def test_pipeline_host_call_matches_device_call(cs, O):
    n = 1 << 16
    x, y, z = O.plummer(8, n)
    lo, hi = (x.min(), y.min(), z.min()), (x.max(), y.max(), z.max())
    h = O.h_for_k_neighbors_cpu(x, y, z, O.make_box(lo, hi), 50)
    box = cs.make_box(lo, hi)
    pipe = cs.Pipeline(64, 64, cs.HILBERT, 64, 100, 1.0, 1.0, True, True)
    tx, ty, tz, th = to_dev(x, y, z, h)
    pipe.run(tx, ty, tz, th, box, (0, 1 << 61))
    nc_dev = pipe.outputs()["neighbor_counts"].clone()
    flags_dev = pipe.outputs()["halo_flags"].clone()
    hx, hy, hz, hh = (torch.from_numpy(a).pin_memory() for a in (x, y, z, h))
    nc_host = torch.empty(n, dtype=torch.int32).pin_memory()
    flags_host = torch.empty(flags_dev.numel(), dtype=torch.uint8).pin_memory()
    pipe.run_host(hx, hy, hz, hh, box, (0, 1 << 61), nc_host, flags_host)
    assert torch.equal(nc_host, nc_dev.cpu())
    assert torch.equal(flags_host, flags_dev.cpu())


def test_pipeline_host_calls_pipelined(cs, O):
    """cs_pipeline_run_host_async: successive calls on different inputs (the two device input sets in turn, each
    call's copies overlapping the previous call's computation), one wait at the end; every call's counts and flags
    equal those of a device-input run on the same inputs, and so does a synchronous call after them"""
    n = 1 << 15
    box_lo, box_hi = (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0)
    box = cs.make_box(box_lo, box_hi)
    focus = (0, 1 << 61)
    inputs = []
    for seed in (11, 12, 13):
        x, y, z = (O.philox_uniform(seed, a, n, -1.0, 1.0) for a in range(3))
        inputs.append((x, y, z, np.full(n, 0.03 + 0.01 * (seed - 11))))
    pipe = cs.Pipeline(64, 64, cs.HILBERT, 64, 100, 1.0, 1.0, True, True)
    ref = []
    for x, y, z, h in inputs:
        pipe.run(*to_dev(x, y, z, h), box, focus)
        o = pipe.outputs()
        ref.append((o["neighbor_counts"].cpu().clone(), o["halo_flags"].cpu().clone()))
    hosts = [tuple(torch.from_numpy(a).pin_memory() for a in t) for t in inputs]
    order = [0, 1, 2, 0, 1]
    fcap = max(r[1].numel() for r in ref)
    outs = [(torch.empty(n, dtype=torch.int32).pin_memory(), torch.empty(fcap, dtype=torch.uint8).pin_memory())
            for k in order]
    for k, (nc_h, fl_h) in zip(order, outs):
        pipe.run_host_async(*hosts[k], box, focus, nc_h, fl_h)
    pipe.wait()
    for k, (nc_h, fl_h) in zip(order, outs):
        assert torch.equal(nc_h, ref[k][0]), k
        assert torch.equal(fl_h[:ref[k][1].numel()], ref[k][1]), k
    nc_h, fl_h = outs[0]
    pipe.run_host(*hosts[2], box, focus, nc_h, fl_h)
    assert torch.equal(nc_h, ref[2][0])


def test_pipeline_repeated_runs_reuse_buffers(cs, O):
    """a second run on different inputs (smaller, then larger) gives the same results as fresh objects"""
    pipe = cs.Pipeline(64, 64, cs.HILBERT, 32, 64, 1.0, 1.0, False, True)
    for n, seed in ((40000, 1), (20000, 2), (70000, 3)):
        x, y, z = (O.philox_uniform(seed, s, n, -1.0, 1.0) for s in range(3))
        h = np.full(n, 0.05)
        tx, ty, tz, th = to_dev(x, y, z, h)
        pipe.run(tx, ty, tz, th, cs.make_box(-1.0, 1.0))
        fresh = cs.Pipeline(64, 64, cs.HILBERT, 32, 64, 1.0, 1.0, False, True)
        fresh.run(tx, ty, tz, th, cs.make_box(-1.0, 1.0))
        a, b = pipe.outputs(), fresh.outputs()
        torch.cuda.synchronize()
        for k in ("sorted_keys", "leaves", "counts", "neighbor_counts"):
            assert torch.equal(a[k], b[k]), (n, k)


@pytest.mark.parametrize("use_graph", [False, True])
def test_pipeline_incremental_steps(cs, O, use_graph):
    """incremental time steps as in the 64M FP32 workload at reduced size: uniform [0,1]^3 periodic, Morton64,
    bucket 32, every step displaces each particle by N(0, 0.1 * spacing) with periodic wrap, then one updateOctree
    step from the previous tree, relink, geometry and neighbours (h = 1.2 * spacing, ngmax 150). Each step equals the
    oracle's keys -> sort -> updateOctree -> link -> geometry -> neighbours on the same positions."""
    n, bucket, ngmax, steps = 1 << 16, 32, 150, 5
    spacing = n ** (-1 / 3)
    x, y, z = (O.philox_uniform(11, s, n, 0.0, 1.0).astype(np.float32) for s in range(3))
    h = np.full(n, 1.2 * spacing, np.float32)
    obox = O.make_box(0.0, 1.0, 1)
    box = cs.make_box(0.0, 1.0, cs.PERIODIC)
    pipe = cs.Pipeline(32, 64, cs.MORTON, bucket, ngmax, 1.0, 1.0, False, True)
    tx, ty, tz, th = to_dev(x, y, z, h)
    rng = np.random.default_rng(5)
    tree = counts = None
    for step in range(steps):
        if step:
            for a in (x, y, z):
                a += rng.normal(0.0, 0.1 * spacing, n).astype(np.float32)
                a[a < 0] += np.float32(1.0)
                a[a >= 1] -= np.float32(1.0)
            for t, a in ((tx, x), (ty, y), (tz, z)):
                t.copy_(torch.from_numpy(a))
        res = pipe.step(tx, ty, tz, th, box, use_graph)
        out = pipe.outputs()
        torch.cuda.synchronize()
        st = pipe.stage_times()  # the stage events are recorded inside replayed graphs too
        assert all(v >= 0 for v in st.values()) and st["neighbors"] > 0, st
        keys = O.sfc_keys(x, y, z, obox, 0, 64)
        sk, perm = O.sort_by_key(keys)
        if step == 0:
            tree, counts, _ = O.compute_octree(sk, bucket, 64)
        else:
            tree, counts, _ = O.update_octree(sk, bucket, tree, counts, 64)
        assert np.array_equal(keys_u(out["sorted_keys"]), sk), step
        assert np.array_equal(u32(out["order"]), perm), step
        assert np.array_equal(keys_u(out["leaves"]), tree), step
        assert np.array_equal(u32(out["counts"]), counts), step
        otree = O.build_octree(tree, 64)
        assert np.array_equal(keys_u(out["prefixes"]), otree.prefixes), step
        assert np.array_equal(out["child_offsets"].cpu().numpy(), otree.child_offsets), step
        cen, siz = O.node_fp_centers(otree.prefixes, obox, np.float32, 0, 64)
        assert np.array_equal(out["centers"].cpu().numpy(), cen), step
        xs, ys, zs = x[perm], y[perm], z[perm]
        nb, nc = O.find_neighbors(xs, ys, zs, h, 0, n, obox, otree, O.layout_from_counts(counts), cen, siz, ngmax)
        neighbor_lists_equal(u32(out["neighbors"]), u32(out["neighbor_counts"]), nb, nc, ngmax)
    assert pipe.graph_replays() == (steps - 1 if use_graph else 0)
