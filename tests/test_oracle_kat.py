"""The oracle against the known answers of the reference's own unit tests (ported as expectations):
test/unit/sfc/{morton,hilbert}.cpp, test/unit/tree/{csarray,octree}.cpp, test/unit/neighbors/findneighbors.cpp,
test/unit/traversal/collisions_a2a.cpp. CPU only."""
import zlib

import numpy as np
import pytest

from kat_util import (OctreeMaker, brute_force_neighbors, check_connectivity, max_level, outside_leaf_box, pad, top,
                      uniform_level_tree)


@pytest.mark.parametrize("bits", [32, 64])
def test_imorton3d(O, bits):
    # test/unit/sfc/morton.cpp:25-39: iMorton(5, 3, 6) at level 3 == pad(0b101011110, 9)
    shift = max_level(bits) - 3
    assert O.imorton(5 << shift, 3 << shift, 6 << shift, bits) == pad(0b101011110, 9, bits)


def test_decode_morton(O):
    # test/unit/sfc/morton.cpp:41-75
    assert O.decode_morton(340, 32) == (5, 2, 4)
    m21 = (1 << 21) - 1
    assert O.decode_morton(0x7FFFFFFFFFFFFFFF, 64) == (m21, m21, m21)
    assert O.decode_morton(0x1249249241249249, 64)[2] == (1 << 21) - 512 - 1
    assert O.decode_morton(0b0111 << 60, 64) == (1 << 20, 1 << 20, 1 << 20)
    assert O.decode_morton(0b0011 << 60, 64) == (0, 1 << 20, 1 << 20)


@pytest.mark.parametrize("bits", [32, 64])
def test_hilbert_first_order_curve(O, bits):
    # test/unit/sfc/hilbert.cpp:90-120: the first level octant order
    h2m = [0, 1, 3, 2, 6, 7, 5, 4]
    half = (1 << max_level(bits)) // 2
    for xi in range(2):
        for yi in range(2):
            for zi in range(2):
                morton_octant = 4 * xi + 2 * yi + zi
                for off in (0, half - 1):
                    k = O.ihilbert(half * xi + off, half * yi + off, half * zi + off, bits)
                    oct_ = (k >> (3 * (max_level(bits) - 1))) & 7
                    assert h2m[oct_] == morton_octant


@pytest.mark.parametrize("bits", [32, 64])
def test_hilbert_continuity(O, bits):
    # test/unit/sfc/hilbert.cpp:122-160: consecutive keys across octant boundaries are neighbouring cells
    L = max_level(bits)
    for level in range(1, L):
        for octant in range(8 if level > 1 else 7):
            last = (octant + 1) * (1 << (3 * (L - level))) - 1
            a = O.decode_hilbert(last, bits)
            b = O.decode_hilbert(last + 1, bits)
            assert sum(abs(int(p) - int(q)) for p, q in zip(a, b)) == 1


@pytest.mark.parametrize("bits", [32, 64])
def test_hilbert_inversion(O, bits):
    rng = np.random.default_rng(0)
    m = (1 << max_level(bits)) - 1
    for _ in range(2000):
        p = [int(v) for v in rng.integers(0, m + 1, 3)]
        assert O.decode_hilbert(O.ihilbert(*p, bits), bits) == tuple(p)


SEARCH_BOUNDS = [  # test/unit/tree/csarray.cpp:28-54: (guess, key, expected range)
    (3, 14, (2, 3)), (3, 15, (3, 4)), (3, 16, (3, 7)), (4, 16, (3, 4)), (0, 17, (0, 8)), (4, 12, (2, 4)),
    (4, 11, (0, 4)), (4, 10, (0, 4)), (8, 16, (0, 8)), (6, 16, (2, 6)), (9, 21, (8, 9)), (12, 16, (0, 12)),
    (8, 1 << 63, (10, 13))]


@pytest.mark.parametrize("guess,key,ref", SEARCH_BOUNDS)
def test_search_bounds(O, guess, key, ref):
    e = 1 << 63
    codes = np.array([3, 10, 11, 14, 16, 16, 16, 18, 19, 21, e, e, e], np.uint64)
    assert O.find_search_bounds(guess, key, codes) == ref


@pytest.mark.parametrize("bits", [32, 64])
def test_count_tree_nodes(O, bits):
    # test/unit/tree/csarray.cpp:56-80
    t = [int(v) for v in OctreeMaker(bits).divide().divide(0).make_tree()]
    keys = np.array([t[1], t[1], t[1] + 10, t[1] + 100, t[2] - 1, t[2] + 1, t[11], t[11] + 2, t[12], t[12] + 1000,
                     t[12] + 2000, t[13] - 10, t[13], t[13] + 1], np.uint64)
    ref = [0, 5, 1, 0, 0, 0, 0, 0, 0, 0, 0, 2, 4, 2, 0]
    tree = np.array(t, np.uint64)
    assert list(O.node_counts(tree, keys, bits)) == ref
    assert list(O.node_counts(tree, keys, bits, guess_counts=np.ones(len(ref), np.uint32))) == ref


@pytest.mark.parametrize("bits", [32, 64])
def test_rebalance_decision(O, bits):
    # test/unit/tree/csarray.cpp:108-128
    tree = OctreeMaker(bits).divide().divide(0).make_tree()
    counts = np.array([1, 1, 1, 0, 0, 0, 0, 0, 2, 3, 4, 5, 6, 7, 8], np.uint32)
    ops, conv = O.rebalance_decision(tree, counts, 4, bits)
    assert list(ops) == [1, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 8, 8, 8, 8] and not conv
    ops, conv = O.rebalance_decision(OctreeMaker(bits).make_tree(), np.array([1], np.uint32), 4, bits)
    assert list(ops) == [1] and conv


@pytest.mark.parametrize("bits", [32, 64])
def test_rebalance_insufficient_resolution(O, bits):
    # test/unit/tree/csarray.cpp:152-190: a max-depth leaf over the bucket size cannot be split further
    m = OctreeMaker(bits)
    for level in range(max_level(bits)):
        m.divide(level=level)
    tree = m.make_tree()
    counts = np.ones(tree.size - 1, np.uint32)
    counts[0] = 2
    ops, conv = O.rebalance_decision(tree, counts, 1, bits)
    assert (ops == 1).all() and conv


@pytest.mark.parametrize("bits", [32, 64])
def test_rebalance_tree(O, bits):
    # test/unit/tree/csarray.cpp:192-212
    tree = OctreeMaker(bits).divide().divide(0).make_tree()
    ops = np.array([1, 0, 0, 0, 0, 0, 0, 0, 1, 8, 1, 1, 1, 1, 8], np.int32)
    ref = OctreeMaker(bits).divide().divide(2).divide(7).make_tree()
    assert np.array_equal(O.rebalance_tree(tree, ops, bits), ref)


@pytest.mark.parametrize("bits", [32, 64])
@pytest.mark.parametrize("bucket", [64, 1024, 10000])
def test_compute_octree_counts_match_searches(O, bits, bucket):
    # test/unit/tree/csarray.cpp:269-348: counts of the converged tree equal lower_bound differences
    from gpu_util import gaussian_keys

    keys = gaussian_keys(100000, bits, 42)
    tree, counts, _ = O.compute_octree(keys, bucket, bits)
    lb = np.searchsorted(keys, tree, side="left")
    assert np.array_equal(counts, np.diff(lb).astype(np.uint32))
    assert tree[0] == 0 and tree[-1] == top(bits)
    # every leaf at most bucket particles unless at the deepest level
    L = max_level(bits)
    levels = L - (np.log2(np.diff(tree).astype(np.float64)) / 3).round().astype(int)
    assert ((counts <= bucket) | (levels == L)).all()


@pytest.mark.parametrize("bits", [32, 64])
def test_internal_octree_shapes(O, bits):
    # test/unit/tree/octree.cpp:76-195
    t = O.build_octree(OctreeMaker(bits).make_tree(), bits)
    assert (t.num_leaves, t.num_nodes, t.num_internal) == (1, 1, 0)

    t = O.build_octree(uniform_level_tree(2, bits), bits)
    assert t.num_internal == (64 - 1) // 7 and t.num_leaves == 64 and t.level_range[-1] == 73
    assert list(np.diff(t.level_range[:4])) == [1, 8, 64]
    check_connectivity(t, bits)

    t = O.build_octree(OctreeMaker(bits).divide().divide(0).make_tree(), bits)
    assert t.num_leaves == 15 and t.num_internal == 2
    assert list(np.diff(t.level_range[:4])) == [1, 8, 8]
    check_connectivity(t, bits)

    t = O.build_octree(OctreeMaker(bits).divide().divide(0).divide(0, 2).divide(3).make_tree(), bits)
    assert (t.num_nodes, t.num_leaves, t.num_internal) == (33, 29, 4)
    assert list(np.diff(t.level_range[:5])) == [1, 8, 16, 8]
    check_connectivity(t, bits)


@pytest.mark.parametrize("bits", [32, 64])
def test_binary_key_weight_maps_to_internal_nodes(O, bits):
    # tree/octree.hpp:41-65: (j + binaryKeyWeight) / 7 enumerates the internal nodes exactly once
    tree = OctreeMaker(bits).divide().divide(0).divide(0, 2).divide(3).divide(7).divide(7, 7).make_tree()
    L = tree.size - 1
    I = (L - 1) // 7
    seen = []
    for j in range(L - 1):
        a, b = int(tree[j]), int(tree[j + 1])
        cpr = ((a ^ b).bit_length() and (bits - (a ^ b).bit_length())) - (2 if bits == 32 else 1)
        if cpr % 3 == 0:
            seen.append((j + O.binary_key_weight(a, cpr // 3, bits)) // 7)
    assert sorted(seen) == list(range(I))


def test_distance_sq_pbc_kat(O):
    # test/unit/neighbors/findneighbors.cpp:27-41 through the full neighbour search (2 particles each)
    for bnd, d2 in ((0, 64.0), (1, 4.0)):
        x = np.array([1.0, 9.0])
        y = np.zeros(2)
        z = np.zeros(2)
        r = np.sqrt(d2)
        for h, expect in ((0.5 * r * 1.0001, 1), (0.5 * r * 0.9999, 0)):
            res = O.pipeline(x, y, z, np.full(2, h), O.make_box(0.0, 10.0, bnd), 1, 4)
            assert list(res["nc"]) == [expect, expect], (bnd, h)


BOXES = [((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)), ((-1.2, -0.213, -5.1), (0.23, 3.213, 1.23))]


@pytest.mark.parametrize("radius,n", [(0.124, 2500), (0.0624, 2500), (3.0, 500)])
@pytest.mark.parametrize("box", BOXES)
@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("bits", [32, 64])
@pytest.mark.parametrize("dist", ["uniform", "gaussian"])
def test_find_neighbors_vs_all_to_all(O, radius, n, box, periodic, bits, dist):
    """test/unit/neighbors/findneighbors.cpp:43-136: tree search == brute force, lists compared in order.

    The reference's key of a point and the box it decodes for the point's leaf can disagree: by up to about half a
    finest cell with 32-bit Hilbert keys (e.g. quantised (354, 256, 773) in a node whose y cells are [0, 256)), by a
    few hundredths of a cell with 64-bit keys. Its traversal then prunes such a particle although it lies within the
    radius. The oracle reproduces that bit for bit (it equals the reference's build on these inputs), so a
    brute-force pair may be missing only when its candidate lies outside its own leaf's box."""
    lo, hi = np.array(box[0]), np.array(box[1])
    rng = np.random.default_rng(zlib.crc32(repr((radius, n, periodic, bits, dist)).encode()))
    if dist == "uniform":
        pts = [rng.uniform(lo[k], hi[k], n) for k in range(3)]
    else:
        pts = []
        for k in range(3):
            v = rng.normal((lo[k] + hi[k]) / 2, (hi[k] - lo[k]) / 5, 4 * n)
            pts.append(v[(v >= lo[k]) & (v < hi[k])][:n])
    x, y, z = pts
    h = np.full(n, radius / 2)
    obox = O.make_box(tuple(lo), tuple(hi), int(periodic))
    res = O.pipeline(x, y, z, h, obox, 64, n, 1, bits)
    lists, counts = brute_force_neighbors(res["x"], res["y"], res["z"], res["h"], lo, hi, periodic)
    outside = outside_leaf_box(res)
    for i in range(n):
        got = res["nb"][i, : res["nc"][i]]
        want = lists[i]
        assert np.all(np.isin(got, want)), i
        missing = np.setdiff1d(want, got)
        assert np.all(outside[missing]), (i, missing)
        assert np.array_equal(got, want[~np.isin(want, missing)]), i


@pytest.mark.parametrize("periodic", [False, True])
def test_find_halos_vs_all_to_all(O, periodic):
    # test/unit/traversal/collisions_a2a.cpp:60-114 in spirit: a node is flagged iff its box and every ancestor's
    # box overlap some focus leaf's search box and the node is not inside the focus key range
    n = 3000
    rng = np.random.default_rng(7)
    x, y, z = (rng.uniform(0, 1, n) for _ in range(3))
    h = rng.uniform(0.005, 0.05, n)
    obox = O.make_box(0.0, 1.0, int(periodic))
    res = O.pipeline(x, y, z, h, obox, 16, 1, with_neighbors=False)
    t = res["tree"]
    leaves = res["leaves"]
    first, last = 0, int(np.searchsorted(leaves, np.uint64(1) << np.uint64(61)))
    l2i = t.leaf_to_internal[t.num_internal:]
    sc, ss = O.search_boxes(res["x"], res["y"], res["z"], res["h"], res["layout"], first, last, 2.0, l2i,
                            res["centers"])
    flags = O.find_halos(t, res["centers"], res["sizes"], sc, ss, obox, first, last)
    lowest, highest = int(leaves[first]), int(leaves[last])
    L = 21

    def key_range(p):
        p = int(p)
        plen = p.bit_length() - 1
        k1 = (p ^ (1 << plen)) << (3 * L - plen)
        return k1, k1 + (1 << (3 * L - plen))

    def contained_in(c, s):
        # containedIn(codeStart, codeEnd, center, size, box), traversal/boxoverlap.hpp:127-152 (Hilbert keys)
        bmin, bmax = c - s, c + s
        if (bmin - 0.0).min() < 0 or (bmax - 1.0).max() > 0:
            return lowest == 0 and highest == 1 << 63
        bmax = bmax + 1.0 * (1.0 / 2 ** 21)
        k1 = int(O.sfc_keys(bmin[:1].copy(), bmin[1:2].copy(), bmin[2:3].copy(), obox)[0])
        k2 = int(O.sfc_keys(bmax[:1].copy(), bmax[1:2].copy(), bmax[2:3].copy(), obox)[0])
        level = ((64 - (k1 ^ k2).bit_length()) - 1) // 3
        rng_ = 1 << (3 * (L - level))
        start = k1 & ~(rng_ - 1)
        return start >= lowest and start + rng_ <= highest

    outside = np.array([not (lambda k: lowest <= k[0] and k[1] <= highest)(key_range(p)) for p in t.prefixes])
    parent = np.full(t.num_nodes, -1)
    for i in range(t.num_nodes):
        c = t.child_offsets[i]
        if c:
            parent[c:c + 8] = i
    ref = np.zeros(t.num_nodes, np.uint8)
    for leaf in range(first, last):
        if contained_in(sc[leaf], ss[leaf]):
            continue
        d = sc[leaf][None, :] - res["centers"]
        if periodic:
            d = d - 1.0 * np.rint(d * 1.0)
        ov = ((np.abs(d) - res["sizes"] - ss[leaf][None, :]) < 0).all(axis=1) & outside
        path = np.zeros(t.num_nodes, bool)
        for i in range(t.num_nodes):  # level-major order: parents come before children
            path[i] = ov[i] and (parent[i] < 0 or path[parent[i]])
        ref[path] = 1
    assert flags.sum() > 0
    assert np.array_equal(flags, ref)
