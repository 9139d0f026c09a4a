"""The oracle against golden fixtures produced by the reference's own CPU code (tests/golden/gen_golden.py). CPU."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def test_keys(O):
    g = load("keys")
    for dname in ("f64", "f32"):
        for bi in (0, 1):
            box = O.make_box(tuple(g[f"lo_{bi}"]), tuple(g[f"hi_{bi}"]), int(g[f"bnd_{bi}"]))
            xyz = [g[f"{c}_{dname}_{bi}"] for c in "xyz"]
            for kind in (0, 1):
                for bits in (32, 64):
                    assert np.array_equal(O.sfc_keys(*xyz, box, kind, bits), g[f"keys_{dname}_{bi}_{kind}_{bits}"]), (
                        dname, bi, kind, bits)


def test_sort_stable(O):
    g = load("sort")
    sk, perm = O.sort_by_key(g["keys"])
    assert np.array_equal(sk, g["sorted_keys"]) and np.array_equal(perm, g["perm"])


def test_plummer_tree(O):
    g = load("plummer_tree")
    box = O.make_box(tuple(g["lo"]), tuple(g["hi"]))
    keys = O.sfc_keys(g["x"], g["y"], g["z"], box)
    sk, perm = O.sort_by_key(keys)
    assert np.array_equal(sk, g["sorted_keys"]) and np.array_equal(perm, g["perm"])
    for bucket in (8, 64):
        t, c, it = O.compute_octree(sk, bucket)
        assert np.array_equal(t, g[f"leaves_b{bucket}"]) and np.array_equal(c, g[f"counts_b{bucket}"])
        assert it == int(g[f"iterations_b{bucket}"])
    tr = O.build_octree(g["leaves_b8"])
    for f in ("prefixes", "child_offsets", "parents", "level_range", "internal_to_leaf", "leaf_to_internal"):
        assert np.array_equal(getattr(tr, f), g[f]), f
    cen, siz = O.node_fp_centers(tr.prefixes, box)
    assert np.array_equal(cen, g["centers"]) and np.array_equal(siz, g["sizes"])
    xs, ys, zs = g["x"][perm], g["y"][perm], g["z"][perm]
    hs = g["h_sorted"]
    layout = O.layout_from_counts(g["counts_b8"])
    first, last = (int(v) for v in g["focus"])
    l2i = tr.leaf_to_internal[tr.num_internal:]
    sc, ss = O.search_boxes(xs, ys, zs, hs, layout, first, last, 2.0, l2i, cen)
    assert np.array_equal(sc[first:last], g["search_centers"]) and np.array_equal(ss[first:last], g["search_sizes"])
    flags = O.find_halos(tr, cen, siz, sc, ss, box, first, last)
    assert np.array_equal(flags, g["halo_flags"])
    ngmax = int(g["ngmax"])
    nb, nc = O.find_neighbors(xs, ys, zs, hs, 0, xs.size, box, tr, layout, cen, siz, ngmax)
    assert np.array_equal(nc, g["nc"])
    mask = np.arange(ngmax)[None, :] < np.minimum(nc, ngmax)[:, None]
    assert np.array_equal(nb[mask], g["nb_flat"])


def test_periodic_f32(O):
    g = load("periodic_f32")
    box = O.make_box(0.0, 1.0, 1)
    keys = O.sfc_keys(g["x"], g["y"], g["z"], box, 1, 32)
    sk, perm = O.sort_by_key(keys)
    assert np.array_equal(sk, g["sorted_keys"]) and np.array_equal(perm, g["perm"])
    t, c, it = O.compute_octree(sk, 16, 32)
    assert np.array_equal(t, g["leaves"]) and np.array_equal(c, g["counts"]) and it == int(g["iterations"])
    tr = O.build_octree(t, 32)
    assert np.array_equal(tr.prefixes, g["prefixes"]) and np.array_equal(tr.child_offsets, g["child_offsets"])
    cen, siz = O.node_fp_centers(tr.prefixes, box, np.float32, 1, 32)
    assert np.array_equal(cen, g["centers"]) and np.array_equal(siz, g["sizes"])
    xs, ys, zs = g["x"][perm], g["y"][perm], g["z"][perm]
    ngmax = int(g["ngmax"])
    nb, nc = O.find_neighbors(xs, ys, zs, g["h_sorted"], 0, xs.size, box, tr, O.layout_from_counts(c), cen, siz,
                              ngmax)
    assert np.array_equal(nc, g["nc"])
    mask = np.arange(ngmax)[None, :] < np.minimum(nc, ngmax)[:, None]
    assert np.array_equal(nb[mask], g["nb_flat"])


def test_restatement_matches_reference_build_here(O):
    """where the reference sources exist (the build container), the restatement equals the reference's own code on
    fresh random inputs too; elsewhere the committed fixtures above carry the pin"""
    if O.ref() is None:
        pytest.skip("reference sources not present")
    rng = np.random.default_rng(99)
    n = 20000
    x, y, z = (rng.normal(0, 1, n) for _ in range(3))
    box = O.make_box((x.min(), y.min(), z.min()), (x.max(), y.max(), z.max()))
    keys = O.sfc_keys(x, y, z, box)
    assert np.array_equal(keys, O.ref_sfc_keys(x, y, z, box))
    sk, perm = O.sort_by_key(keys)
    rk, rp = O.ref_sort_by_key(keys)
    assert np.array_equal(sk, rk) and np.array_equal(perm, rp)
    t, c, it = O.compute_octree(sk, 32)
    rt, rc, rit = O.ref_compute_octree(sk, 32)
    assert np.array_equal(t, rt) and np.array_equal(c, rc) and it == rit
    tr, rtr = O.build_octree(t), O.ref_build_octree(t)
    assert np.array_equal(tr.prefixes, rtr.prefixes) and np.array_equal(tr.child_offsets, rtr.child_offsets)
    cen, siz = O.node_fp_centers(tr.prefixes, box)
    rcen, rsiz = O.ref_node_fp_centers(tr.prefixes, box)
    assert np.array_equal(cen, rcen) and np.array_equal(siz, rsiz)
    xs, ys, zs = x[perm], y[perm], z[perm]
    hs = np.full(n, 0.04)
    layout = O.layout_from_counts(c)
    nb, nc = O.find_neighbors(xs, ys, zs, hs, 0, n, box, tr, layout, cen, siz, 40)
    rnb, rnc = O.ref_find_neighbors(xs, ys, zs, hs, 0, n, box, tr, layout, cen, siz, 40)
    assert np.array_equal(nc, rnc)
    mask = np.arange(40)[None, :] < np.minimum(nc, 40)[:, None]
    assert np.array_equal(np.where(mask, nb, 0), np.where(mask, rnb, 0))
