"""Parity at the benchmark configurations' real sizes, bit for bit against the oracle on the same inputs.

- 16M FP64 Plummer keys -> neighbours, exactly as the benchmark runs it (same generator and seed, tight box, Hilbert64,
  bucket 64, halos for the leaves in [0, 2^61), ngmax 200, h for 100 neighbours): keys, permutation, leaves, counts,
  iterations, the linked tree, node centres and sizes, halo flags, neighbour counts and lists.
- 64M FP32 uniform periodic time steps (Morton64, bucket 32): the root build and two graph-replayed updateOctree steps
  against the oracle's computeOctree -> updateOctree chain, neighbour lists of the last step.
- The 4096-set batched workload: the whole batch in chunks, and 64 of its sets (the largest among them) against the
  oracle's single-set pipeline.

The oracle's neighbour search runs in chunks of particles (findNeighbors over [first, last)), so host memory stays
bounded; the device rows of the same chunk are copied for the comparison.
"""
import os
import sys

import numpy as np
import pytest
import torch

from gpu_util import keys_u, neighbor_lists_equal, u32

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "cornerstone-octree_gb300"))
import cstone_synth as S  # noqa: E402

CHUNK = 1 << 21


def compare_neighbors_chunked(O, xs, ys, zs, hs, obox, otree, layout, centers, sizes, ngmax, nb_dev, nc_dev):
    n = xs.size
    for first in range(0, n, CHUNK):
        last = min(n, first + CHUNK)
        rnb, rnc = O.find_neighbors(xs, ys, zs, hs, first, last, obox, otree, layout, centers, sizes, ngmax)
        gnb = u32(nb_dev[first:last])
        gnc = u32(nc_dev[first:last])
        neighbor_lists_equal(gnb, gnc, rnb, rnc, ngmax)


def test_plummer_16m_headline_config(cs, O):
    from cstone_gb300 import workloads as W

    n, bucket, ngmax, focus = 16 * 1024 * 1024, 64, 200, (0, 1 << 61)
    x, y, z = S.plummer(n, 2024)
    lo, hi = S.tight_box(x, y, z)
    box = cs.make_box(lo, hi)
    tx, ty, tz = (torch.from_numpy(a).cuda() for a in (x, y, z))
    th, hnc = W.h_for_k_neighbors(tx, ty, tz, box, 100, bucket)
    assert float((hnc == 100).double().mean()) > 0.999
    h = th.cpu().numpy()

    pipe = cs.Pipeline(64, 64, cs.HILBERT, bucket, ngmax, 1.0, 1.0, True, True)
    res = pipe.run(tx, ty, tz, th, box, focus)
    out = pipe.outputs()
    torch.cuda.synchronize()

    obox = O.make_box(lo, hi)
    keys = O.sfc_keys(x, y, z, obox, O.HILBERT, 64)
    sk, perm = O.sort_by_key(keys)
    assert np.array_equal(keys_u(out["sorted_keys"]), sk)
    assert np.array_equal(u32(out["order"]), perm)
    del keys
    xs, ys, zs, hs = x[perm], y[perm], z[perm], h[perm]
    leaves, counts, iters = O.compute_octree(sk, bucket, 64)
    del sk
    assert np.array_equal(keys_u(out["leaves"]), leaves)
    assert np.array_equal(u32(out["counts"]), counts)
    assert res.iterations == iters
    otree = O.build_octree(leaves, 64)
    assert np.array_equal(keys_u(out["prefixes"]), otree.prefixes)
    for k in ("child_offsets", "parents", "level_range", "internal_to_leaf", "leaf_to_internal"):
        assert np.array_equal(out[k].cpu().numpy(), getattr(otree, k)[: out[k].numel()]), k
    centers, sizes = O.node_fp_centers(otree.prefixes, obox, np.float64, O.HILBERT, 64)
    assert np.array_equal(out["centers"].cpu().numpy(), centers)
    assert np.array_equal(out["sizes"].cpu().numpy(), sizes)
    layout = O.layout_from_counts(counts)
    first = int(np.searchsorted(leaves, np.uint64(focus[0])))
    last = int(np.searchsorted(leaves, np.uint64(focus[1])))
    assert (res.focus_first, res.focus_last) == (first, last)
    sc, ss = O.search_boxes(xs, ys, zs, hs, layout, first, last, 2.0, otree.leaf_to_internal[otree.num_internal:],
                            centers)
    assert np.array_equal(out["search_centers"][first:last].cpu().numpy(), sc[first:last])
    assert np.array_equal(out["search_sizes"][first:last].cpu().numpy(), ss[first:last])
    flags = O.find_halos(otree, centers, sizes, sc, ss, obox, first, last, 64)
    assert np.array_equal(out["halo_flags"].cpu().numpy(), flags)
    compare_neighbors_chunked(O, xs, ys, zs, hs, obox, otree, layout, centers, sizes, ngmax, out["neighbors"],
                              out["neighbor_counts"])


def test_incremental_64m_fp32_root_and_two_graph_steps(cs, O):
    n, bucket, ngmax = 64 * 1024 * 1024, 32, 150
    spacing = n ** (-1.0 / 3)
    rng = np.random.default_rng(64)
    x, y, z = (rng.random(n, dtype=np.float32) for _ in range(3))
    h = np.full(n, 1.2 * spacing, np.float32)
    obox = O.make_box(0.0, 1.0, 1)
    box = cs.make_box(0.0, 1.0, cs.PERIODIC)
    pipe = cs.Pipeline(32, 64, cs.MORTON, bucket, ngmax, 1.0, 1.0, False, True)
    tx, ty, tz, th = (torch.from_numpy(a).cuda() for a in (x, y, z, h))
    tree = counts = None
    steps = 3
    for step in range(steps):
        if step:
            for a in (x, y, z):
                a += (rng.standard_normal(n, dtype=np.float32) * np.float32(0.1 * spacing)).astype(np.float32)
                a[a < 0] += np.float32(1.0)
                a[a >= 1] -= np.float32(1.0)
            for t, a in ((tx, x), (ty, y), (tz, z)):
                t.copy_(torch.from_numpy(a))
        pipe.step(tx, ty, tz, th, box, True)
        out = pipe.outputs()
        torch.cuda.synchronize()
        keys = O.sfc_keys(x, y, z, obox, O.MORTON, 64)
        sk, perm = O.sort_by_key(keys)
        del keys
        if step == 0:
            tree, counts, _ = O.compute_octree(sk, bucket, 64)
        else:
            tree, counts, _ = O.update_octree(sk, bucket, tree, counts, 64)
        assert np.array_equal(keys_u(out["sorted_keys"]), sk), step
        assert np.array_equal(u32(out["order"]), perm), step
        assert np.array_equal(keys_u(out["leaves"]), tree), step
        assert np.array_equal(u32(out["counts"]), counts), step
        del sk
        otree = O.build_octree(tree, 64)
        assert np.array_equal(keys_u(out["prefixes"]), otree.prefixes), step
        assert np.array_equal(out["child_offsets"].cpu().numpy(), otree.child_offsets), step
        if step == steps - 1:
            cen, siz = O.node_fp_centers(otree.prefixes, obox, np.float32, O.MORTON, 64)
            assert np.array_equal(out["centers"].cpu().numpy(), cen)
            xs, ys, zs = x[perm], y[perm], z[perm]
            compare_neighbors_chunked(O, xs, ys, zs, h, obox, otree, O.layout_from_counts(counts), cen, siz, ngmax,
                                      out["neighbors"], out["neighbor_counts"])
    assert pipe.graph_replays() == steps - 1


def test_batched_4096_sets_against_single_set_oracle(cs, O):
    from cstone_gb300 import workloads as W

    ngmax = 100
    dev = torch.device("cuda:0")
    sets = W.batched_sets(4096, 2024, dev)
    sizes = np.array([st["n"] for st in sets])
    rng = np.random.default_rng(1)
    sample = set(rng.choice(len(sets), 63, replace=False).tolist()) | {int(np.argmax(sizes))}
    batch = cs.Batch(32, cs.MORTON, ngmax)
    checked = 0
    for ch, offs, (x, y, z, h) in W.chunk_sets(sets):
        boxes = [cs.make_box(sets[s]["lo"], sets[s]["hi"]) for s in ch]
        batch.run(x, y, z, h, offs, boxes, [sets[s]["bucket"] for s in ch])
        out = batch.outputs()
        torch.cuda.synchronize()
        assert batch.result.num_sets == len(ch) and batch.result.num_particles == offs[-1]
        lb = out["set_leaf_begin"].cpu().numpy()
        for j, s in enumerate(ch):
            if s not in sample:
                continue
            st = sets[s]
            a, e = int(offs[j]), int(offs[j + 1])
            sx, sy, sz, sh = (t.cpu().numpy() for t in (st["x"], st["y"], st["z"], st["h"]))
            ref = O.pipeline(sx, sy, sz, sh, O.make_box(st["lo"], st["hi"]), st["bucket"], ngmax, O.MORTON, 32)
            assert np.array_equal(u32(out["order"][a:e]) - a, ref["perm"]), s
            leaves = keys_u(out["leaves"][lb[j]: lb[j + 1] + 1]) - (np.uint64(j) << np.uint64(30))
            assert np.array_equal(leaves, ref["leaves"]), s
            assert np.array_equal(u32(out["counts"][lb[j]: lb[j + 1]]), ref["counts"]), s
            nc = u32(out["neighbor_counts"][a:e])
            nb = (u32(out["neighbors"][a:e]).astype(np.int64) - a).astype(np.uint32)
            neighbor_lists_equal(nb, nc, ref["nb"], ref["nc"], ngmax)
            checked += 1
    assert checked == len(sample)
