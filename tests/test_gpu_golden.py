"""GPU parity against the golden fixtures produced by the reference's own CPU code (tests/golden/): the CUDA path
reproduces the reference's keys, permutation, leaves, counts, iterations, linked tree, node geometry, search boxes,
halo flags and neighbour lists bit for bit, with no oracle in the loop."""
import os

import numpy as np
import pytest
import torch

from gpu_util import dev, keys_u, to_dev, u32

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def test_keys(cs):
    g = load("keys")
    for dname in ("f64", "f32"):
        for bi in (0, 1):
            box = cs.make_box(tuple(g[f"lo_{bi}"]), tuple(g[f"hi_{bi}"]), int(g[f"bnd_{bi}"]))
            tx, ty, tz = to_dev(*[g[f"{c}_{dname}_{bi}"] for c in "xyz"])
            for kind in (0, 1):
                for bits in (32, 64):
                    k = cs.sfc_keys(tx, ty, tz, box, kind, bits)
                    torch.cuda.synchronize()
                    assert np.array_equal(keys_u(k), g[f"keys_{dname}_{bi}_{kind}_{bits}"]), (dname, bi, kind, bits)


def test_sort(cs):
    g = load("sort")
    sk, perm = cs.sort_pairs(torch.from_numpy(g["keys"].view(np.int64)).to(dev()))
    torch.cuda.synchronize()
    assert np.array_equal(keys_u(sk), g["sorted_keys"]) and np.array_equal(u32(perm), g["perm"])


def test_plummer_pipeline_stages(cs):
    g = load("plummer_tree")
    box = cs.make_box(tuple(g["lo"]), tuple(g["hi"]))
    tx, ty, tz = to_dev(g["x"], g["y"], g["z"])
    keys, perm = cs.sort_pairs(cs.sfc_keys(tx, ty, tz, box, cs.HILBERT, 64))
    assert np.array_equal(keys_u(keys), g["sorted_keys"]) and np.array_equal(u32(perm), g["perm"])
    for bucket in (8, 64):
        t, c, layout, it = cs.compute_octree(keys, bucket)
        torch.cuda.synchronize()
        assert np.array_equal(keys_u(t), g[f"leaves_b{bucket}"]) and np.array_equal(u32(c), g[f"counts_b{bucket}"])
        assert it == int(g[f"iterations_b{bucket}"])
    t, c, layout, _ = cs.compute_octree(keys, 8)
    o = cs.build_octree(t)
    torch.cuda.synchronize()
    assert np.array_equal(keys_u(o.prefixes), g["prefixes"])
    for f in ("child_offsets", "parents", "level_range", "internal_to_leaf", "leaf_to_internal"):
        a = getattr(o, f).cpu().numpy()
        assert np.array_equal(a[: g[f].size], g[f]), f
    cen, siz = cs.geo_centers(o.prefixes, box, torch.float64)
    assert np.array_equal(cen.cpu().numpy(), g["centers"]) and np.array_equal(siz.cpu().numpy(), g["sizes"])
    xs, ys, zs = cs.gather(perm, tx), cs.gather(perm, ty), cs.gather(perm, tz)
    (hs,) = to_dev(g["h_sorted"])
    first, last = (int(v) for v in g["focus"])
    l2i = o.leaf_to_internal[o.num_internal:]
    sc, ss = cs.search_boxes(xs, ys, zs, hs, layout, first, last, 2.0, l2i, cen)
    flags = cs.find_halos(o, cen, siz, sc, ss, box, first, last)
    torch.cuda.synchronize()
    assert np.array_equal(sc[first:last].cpu().numpy(), g["search_centers"])
    assert np.array_equal(ss[first:last].cpu().numpy(), g["search_sizes"])
    assert np.array_equal(flags.cpu().numpy(), g["halo_flags"])
    ngmax = int(g["ngmax"])
    nb, nc = cs.find_neighbors(xs, ys, zs, hs, 0, xs.numel(), box, o, layout, cen, siz, ngmax)
    torch.cuda.synchronize()
    assert np.array_equal(u32(nc), g["nc"])
    mask = np.arange(ngmax)[None, :] < np.minimum(g["nc"], ngmax)[:, None]
    assert np.array_equal(u32(nb)[mask], g["nb_flat"])


def test_periodic_f32(cs):
    g = load("periodic_f32")
    box = cs.make_box(0.0, 1.0, cs.PERIODIC)
    tx, ty, tz = to_dev(g["x"], g["y"], g["z"])
    keys, perm = cs.sort_pairs(cs.sfc_keys(tx, ty, tz, box, cs.HILBERT, 32))
    t, c, layout, it = cs.compute_octree(keys, 16)
    o = cs.build_octree(t)
    cen, siz = cs.geo_centers(o.prefixes, box, torch.float32)
    xs, ys, zs = cs.gather(perm, tx), cs.gather(perm, ty), cs.gather(perm, tz)
    (hs,) = to_dev(g["h_sorted"])
    ngmax = int(g["ngmax"])
    nb, nc = cs.find_neighbors(xs, ys, zs, hs, 0, xs.numel(), box, o, layout, cen, siz, ngmax)
    torch.cuda.synchronize()
    assert np.array_equal(keys_u(keys), g["sorted_keys"]) and np.array_equal(u32(perm), g["perm"])
    assert np.array_equal(keys_u(t), g["leaves"]) and np.array_equal(u32(c), g["counts"])
    assert it == int(g["iterations"])
    assert np.array_equal(keys_u(o.prefixes), g["prefixes"])
    assert np.array_equal(cen.cpu().numpy(), g["centers"]) and np.array_equal(siz.cpu().numpy(), g["sizes"])
    assert np.array_equal(u32(nc), g["nc"])
    mask = np.arange(ngmax)[None, :] < np.minimum(g["nc"], ngmax)[:, None]
    assert np.array_equal(u32(nb)[mask], g["nb_flat"])
