"""The oracle's restatement of the functions around the path (upsweeps, source centres, spanning trees, focus-tree
rebalance helpers, target groups) against golden fixtures made by the reference's own CPU code
(tests/golden/gen_golden_next.py), and against that code itself where it can be built (this container). CPU only."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def g():
    return np.load(os.path.join(GOLDEN, "tree_ops.npz"))


@pytest.fixture(scope="module")
def ref(O):
    if O.ref() is None:
        pytest.skip("the reference's own CPU code is not built here")
    return O


def _leaf_l2i(g):
    L = g["leaves"].size - 1
    return g["leaf_to_internal"][g["prefixes"].size - L:]


def test_upsweep_counts(O, g):
    nc = np.zeros(g["prefixes"].size, np.uint32)
    nc[_leaf_l2i(g)] = g["leaf_counts"]
    assert np.array_equal(O.upsweep_sum(g["level_range"], g["child_offsets"], nc), g["node_counts"])
    assert g["node_counts"][0] == g["x"].size


@pytest.mark.parametrize("dt", ["f64", "f32"])
def test_source_centers(O, g, dt):
    t = np.float64 if dt == "f64" else np.float32
    x, y, z, m = (g[c].astype(t) for c in "xyzm")
    c = O.leaf_mass_centers(x, y, z, m, _leaf_l2i(g), O.layout_from_counts(g["leaf_counts"]), g["prefixes"].size)
    c = O.upsweep_centers(g["level_range"], g["child_offsets"], c)
    assert np.array_equal(c, g[f"centers_{dt}"])


@pytest.mark.parametrize("bits", [64, 32])
def test_spanning_tree(O, g, bits):
    k = g[f"span_keys_{bits}"]
    assert np.array_equal(O.fill_sfc_gaps(k, bits), g[f"span_tree_{bits}"])


def test_span_sfc_range_known_answers(O):
    # between siblings at one level: just the start; across levels: every enclosing step (sfc/common.hpp:400-460)
    assert list(O.span_sfc_range(0, 1 << 60)) == [0]
    assert list(O.span_sfc_range(0, 1 << 63)) == [0]
    r = O.span_sfc_range(1 << 57, 1 << 63)
    assert r[0] == 1 << 57 and r.size == 7 + 7
    assert np.all(np.diff(r.astype(np.float64)) > 0)


def test_focus_rebalance(O, g):
    focus = tuple(int(v) for v in g["focus"])
    ops = O.rebalance_decision_essential(g["prefixes"], g["child_offsets"], g["parents"], g["node_counts"], g["macs"],
                                         focus, 16)
    assert np.array_equal(ops, g["ops_essential"])
    cops = O.rebalance_decision_essential(g["coarse_prefixes"], g["coarse_child_offsets"], g["coarse_parents"],
                                          g["coarse_counts"], g["coarse_macs"],
                                          tuple(int(v) for v in g["coarse_focus"]), 1)
    assert np.array_equal(cops, g["coarse_ops"])
    pops, conv = O.protect_ancestors(g["prefixes"], g["parents"], ops)
    assert np.array_equal(pops, g["ops_protected"]) and conv == bool(g["protect_converged"])
    eops, st = O.enforce_keys(g["forced_keys"], g["prefixes"], g["child_offsets"], g["parents"], pops)
    assert np.array_equal(eops, g["ops_enforced"]) and st == int(g["enforce_status"])
    f0, f1 = (int(v) for v in g["focus_leaf_range"])
    mr = O.mac_refine_decision(g["prefixes"], g["macs"], _leaf_l2i(g), f0, f1)
    assert np.array_equal(mr, g["mac_refine"])
    rc = O.range_count(g["global_leaves"], g["global_counts"], g["leaves"], g["range_idx"])
    assert np.array_equal(rc[g["range_idx"]], g["range_counts"][g["range_idx"]])
    lay = O.node_layout(g["leaf_counts"], g["layout_flags"], _leaf_l2i(g), f0, f1)
    assert np.array_equal(lay, g["node_layout"])


def _random_tree(O, rng, n, bucket, bits=64):
    x, y, z = (rng.random(n) for _ in range(3))
    box = O.make_box(0.0, 1.0)
    sk, perm = O.sort_by_key(O.sfc_keys(x, y, z, box, O.HILBERT, bits))
    leaves, counts, _ = O.compute_octree(sk, bucket, bits)
    return x[perm], y[perm], z[perm], sk, leaves, counts, O.build_octree(leaves, bits)


@pytest.mark.parametrize("bits", [64, 32])
def test_against_reference_random_trees(ref, bits):
    O = ref
    rng = np.random.default_rng(bits)
    for n, bucket in ((3000, 8), (20000, 64)):
        x, y, z, sk, leaves, counts, tr = _random_tree(O, rng, n, bucket, bits)
        N, L = tr.num_nodes, tr.num_leaves
        l2i = tr.leaf_to_internal[tr.num_internal:]
        nc = np.zeros(N, np.uint32)
        nc[l2i] = counts
        a = O.upsweep_sum(tr.level_range, tr.child_offsets, nc)
        assert np.array_equal(a, O.upsweep_sum(tr.level_range, tr.child_offsets, nc, use_ref=True))
        macs = (rng.random(N) < 0.4).astype(np.uint8)
        focus = (int(leaves[L // 4]), int(leaves[L // 2]))
        for b in (1, 4, bucket):
            o1 = O.rebalance_decision_essential(tr.prefixes, tr.child_offsets, tr.parents, a, macs, focus, b, bits)
            o2 = O.rebalance_decision_essential(tr.prefixes, tr.child_offsets, tr.parents, a, macs, focus, b, bits,
                                                use_ref=True)
            assert np.array_equal(o1, o2), b
            p1 = O.protect_ancestors(tr.prefixes, tr.parents, o1, bits)
            p2 = O.protect_ancestors(tr.prefixes, tr.parents, o1, bits, use_ref=True)
            assert np.array_equal(p1[0], p2[0]) and p1[1] == p2[1]
            keys = np.sort(rng.choice(sk, 30, replace=False)).astype(np.uint64)
            e1 = O.enforce_keys(keys, tr.prefixes, tr.child_offsets, tr.parents, p1[0], bits)
            e2 = O.enforce_keys(keys, tr.prefixes, tr.child_offsets, tr.parents, p1[0], bits, use_ref=True)
            assert np.array_equal(e1[0], e2[0]) and e1[1] == e2[1]
        m = rng.uniform(0.1, 1.0, n)
        lay = O.layout_from_counts(counts)
        c1 = O.upsweep_centers(tr.level_range, tr.child_offsets, O.leaf_mass_centers(x, y, z, m, l2i, lay, N))
        c2 = O.upsweep_centers(tr.level_range, tr.child_offsets,
                               O.leaf_mass_centers(x, y, z, m, l2i, lay, N, use_ref=True), use_ref=True)
        assert np.array_equal(c1, c2)
        k = np.unique(np.concatenate([[0], rng.choice(sk, 50), [sk.max()]]))
        top = np.uint64(1 << (63 if bits == 64 else 30))
        k = np.unique(np.concatenate([k, [top]])).astype(np.uint64)
        assert np.array_equal(O.fill_sfc_gaps(k, bits), O.ref_spanning_tree(k, bits))


@pytest.mark.parametrize("group_size", [32, 64])
def test_group_splits_structure(O, g, group_size):
    """groups cover [first, last) in order, none longer than the fixed size, cuts only where the criterion holds"""
    x, y, z = g["x"], g["y"], g["z"]
    n = x.size
    h = np.full(n, 0.02)
    layout = O.layout_from_counts(g["leaf_counts"])
    first, last = 100, n - 37
    grp = O.group_splits(first, last, x, y, z, h, g["leaves"], layout, g["lo"], g["hi"], group_size, 8.0)
    assert grp[0] == first and grp[-1] == last
    d = np.diff(grp.astype(np.int64))
    assert np.all(d > 0) and np.all(d <= group_size)
    assert grp.size - 1 > (last - first + group_size - 1) // group_size  # some groups were cut
    # every fixed-group start is a group start
    assert set(range(first, last, group_size)) <= set(grp.tolist())


@pytest.mark.parametrize("bnd", [0, 1])
def test_float_h_with_double_coordinates_against_reference(ref, bnd):
    """findNeighbors and computeBoundingBox with Tc = double, Th = float: radii rounded to float"""
    O = ref
    rng = np.random.default_rng(11 + bnd)
    n = 20000
    x, y, z = (rng.random(n) for _ in range(3))
    h = (0.02 + 0.02 * rng.random(n)).astype(np.float32)
    box = O.make_box(0.0, 1.0, bnd)
    sk, perm = O.sort_by_key(O.sfc_keys(x, y, z, box))
    xs, ys, zs, hs = x[perm], y[perm], z[perm], h[perm]
    lv, ct, _ = O.compute_octree(sk, 16)
    tr = O.build_octree(lv)
    cen, siz = O.node_fp_centers(tr.prefixes, box)
    lay = O.layout_from_counts(ct)
    a = O.find_neighbors(xs, ys, zs, hs, 0, n, box, tr, lay, cen, siz, 80)
    b = O.ref_find_neighbors(xs, ys, zs, hs, 0, n, box, tr, lay, cen, siz, 80)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    # the float radius differs from the double one: some pair must change side for the test to mean something
    d = O.find_neighbors(xs, ys, zs, hs.astype(np.float64), 0, n, box, tr, lay, cen, siz, 80)
    assert a[1].sum() > 0 and d[1].sum() > 0
    l2i = tr.leaf_to_internal[tr.num_internal:]
    s1 = O.search_boxes(xs, ys, zs, hs, lay, 0, tr.num_leaves, 2.0, l2i, cen)
    s2 = O.search_boxes(xs, ys, zs, hs, lay, 0, tr.num_leaves, 2.0, l2i, cen, use_ref=True)
    assert np.array_equal(s1[0], s2[0]) and np.array_equal(s1[1], s2[1])
