"""GPU parity: halo search boxes + collision flags and neighbour search, bit-exact against the oracle."""
import numpy as np
import pytest
import torch

from gpu_util import dev, neighbor_lists_equal, to_dev, u32, uniform

pytestmark = pytest.mark.gpu


def _setup(O, cs, x, y, z, h, box_lo, box_hi, bnd, bucket, kind=1, bits=64):
    obox = O.make_box(box_lo, box_hi, bnd)
    ref = O.pipeline(x, y, z, h, obox, bucket, 1, kind, bits, with_neighbors=False)
    tx, ty, tz, th = to_dev(ref["x"], ref["y"], ref["z"], ref["h"])
    if bits == 32:
        leaves = torch.from_numpy(ref["leaves"].astype(np.uint32).view(np.int32)).to(dev())
    else:
        leaves = torch.from_numpy(ref["leaves"].view(np.int64)).to(dev())
    o = cs.build_octree(leaves)
    layout = torch.from_numpy(ref["layout"].view(np.int32)).to(dev())
    box = cs.make_box(box_lo, box_hi, bnd)
    c, s = cs.geo_centers(o.prefixes, box, tx.dtype, kind)
    return ref, obox, box, o, layout, c, s, (tx, ty, tz, th)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("bnd", [0, 1])
@pytest.mark.parametrize("focus", ["quarter", "middle", "all"])
def test_halos(cs, O, dtype, bnd, focus):
    n = 40000
    x, y, z = uniform(O, 31, n, -1.0, 1.0, dtype)
    h = (0.02 + 0.03 * O.philox_uniform(32, 0, n, 0, 1)).astype(dtype)
    ref, obox, box, o, layout, c, s, (tx, ty, tz, th) = _setup(O, cs, x, y, z, h, -1.0, 1.0, bnd, 32)
    L = o.num_leaves
    leaves = ref["leaves"]
    if focus == "quarter":
        first, last = 0, int(np.searchsorted(leaves, np.uint64(1) << np.uint64(61)))
    elif focus == "middle":
        first, last = L // 3, 2 * L // 3
    else:
        first, last = 0, L
    tree = ref["tree"]
    l2i = tree.leaf_to_internal[tree.num_internal:]
    rsc, rss = O.search_boxes(ref["x"], ref["y"], ref["z"], ref["h"], ref["layout"], first, last, 2.0, l2i,
                              ref["centers"])
    rflags = O.find_halos(tree, ref["centers"], ref["sizes"], rsc, rss, obox, first, last)
    tl2i = o.leaf_to_internal[o.num_internal:]
    sc, ss = cs.search_boxes(tx, ty, tz, th, layout, first, last, 2.0, tl2i, c)
    flags = cs.find_halos(o, c, s, sc, ss, box, first, last)
    torch.cuda.synchronize()
    assert np.array_equal(sc[first:last].cpu().numpy(), rsc[first:last])
    assert np.array_equal(ss[first:last].cpu().numpy(), rss[first:last])
    assert np.array_equal(flags.cpu().numpy(), rflags)
    # computeBoundingBoxGpu's own contract: the caller fills the leaves' centres, the call updates them in place
    init = c.view(-1, 3)[tl2i.long()]
    sc2, ss2 = cs.search_boxes(tx, ty, tz, th, layout, first, last, 2.0, None, None, init=init)
    torch.cuda.synchronize()
    assert torch.equal(sc2[first:last], sc[first:last]) and torch.equal(ss2[first:last], ss[first:last])


@pytest.mark.parametrize("hkind", ["f64", "f32"])
@pytest.mark.parametrize("scale", [2.0, 0.75, 2.0 ** -20, 40.0])
def test_search_boxes_fp64_screen_edges(cs, O, hkind, scale):
    """FP64 search boxes, whose particles go through an FP32 screen before the exact FP64 min/max: exact ties of
    x - r across a leaf, a leaf of 700 particles at one point (every particle a candidate on every side), empty
    leaves, coordinates and h at or beyond the screen's range (2^120), subnormal, zero and negative-zero values,
    centres outside the screen's range; scale 40 takes the unscreened kernel. Against the oracle, leaf by leaf."""
    rng = np.random.default_rng(5)
    sizes = rng.integers(0, 60, 400)
    sizes[[3, 50, 51]] = 0
    sizes[7], sizes[8] = 700, 257
    L = sizes.size
    layout = np.zeros(L + 1, np.uint32)
    layout[1:] = np.cumsum(sizes)
    n = int(layout[-1])
    x, y, z = (rng.uniform(-1.0, 1.0, n) for _ in range(3))
    h = rng.uniform(0.001, 0.05, n)

    def seg(leaf):
        return slice(int(layout[leaf]), int(layout[leaf + 1]))

    s = seg(7)  # one point, one h
    x[s], y[s], z[s], h[s] = 0.3, -0.2, 0.1, 0.01
    s = seg(8)  # x - 2h = 0.5 and y + 2h = -0.25 for every particle
    k = np.arange(sizes[8], dtype=np.float64)
    x[s], h[s] = 0.5 + k * 2.0 ** -20, k * 2.0 ** -21
    y[s] = -0.25 - k * 2.0 ** -20
    s = seg(9)  # magnitudes at and beyond 2^120
    m = sizes[9]
    x[s] = np.resize([2.0 ** 120, -2.0 ** 121, 3e300, 1e37, -1e36], m)
    z[s] = np.resize([-2.0 ** 119.99, 1e200, -0.5], m)
    s = seg(10)  # zeros, negative zeros, subnormals, h = 0
    m = sizes[10]
    x[s] = np.resize([0.0, -0.0, 5e-324, -1e-310, 2.0 ** -121, -(2.0 ** -120)], m)
    y[s] = np.resize([-0.0, 1e-300, 0.0], m)
    h[s] = np.resize([0.0, 1e-310, 2.0 ** -121, 0.0, 1e-30], m)
    s = seg(11)  # h beyond the screen's range
    h[s] = np.resize([1e36, 2.0 ** 120, 0.01], sizes[11])
    if hkind == "f32":
        h = h.astype(np.float32)  # 1e-310 and 2^-121 become float zeros or subnormals
    init = rng.uniform(-1.0, 1.0, (L, 3))
    init[12] = (1e200, -3e299, 2.0 ** 120)
    init[13] = (-0.0, 5e-324, 0.0)
    init[[3, 50]] = (0.25, -0.125, 1e-300)  # empty leaves keep their centre
    init[8] = (0.6, -0.3, 0.0)  # so that the tied values are the extrema

    first, last = 2, L - 3
    rsc, rss = O.search_boxes(x, y, z, h, layout, first, last, scale, np.arange(L, dtype=np.int32), init)
    tx, ty, tz, th = to_dev(x, y, z, h)
    tlayout = torch.from_numpy(layout.view(np.int32)).to(dev())
    sc, ss = cs.search_boxes(tx, ty, tz, th, tlayout, first, last, scale, None, None,
                             init=torch.from_numpy(init).to(dev()))
    torch.cuda.synchronize()
    assert np.array_equal(sc[first:last].cpu().numpy(), rsc[first:last])
    assert np.array_equal(ss[first:last].cpu().numpy(), rss[first:last])
    assert np.isfinite(rsc[first:last]).all() and np.isfinite(rss[first:last]).all()


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("bnd", [0, 1])
@pytest.mark.parametrize("hmode", ["const", "variable"])
def test_neighbors_uniform(cs, O, dtype, bnd, hmode):
    n = 60000
    x, y, z = uniform(O, 41, n, -1.0, 1.0, dtype)
    if hmode == "const":
        h = np.full(n, 0.04, dtype)
    else:
        h = (0.01 + 0.11 * O.philox_uniform(42, 0, n, 0, 1)).astype(dtype)  # up to ~500 neighbours
    ngmax = 100
    ref, obox, box, o, layout, c, s, (tx, ty, tz, th) = _setup(O, cs, x, y, z, h, -1.0, 1.0, bnd, 32)
    rnb, rnc = O.find_neighbors(ref["x"], ref["y"], ref["z"], ref["h"], 0, n, obox, ref["tree"], ref["layout"],
                                ref["centers"], ref["sizes"], ngmax)
    nb, nc = cs.find_neighbors(tx, ty, tz, th, 0, n, box, o, layout, c, s, ngmax)
    torch.cuda.synchronize()
    neighbor_lists_equal(u32(nb), u32(nc), rnb, rnc, ngmax)
    assert (rnc > ngmax).any() or hmode == "const"  # truncation is exercised


def test_neighbors_subrange_and_ext(cs, O):
    n = 30000
    x, y, z = uniform(O, 51, n, -0.5, 0.5)
    h = np.full(n, 0.03)
    ngmax = 64
    ref, obox, box, o, layout, c, s, (tx, ty, tz, th) = _setup(O, cs, x, y, z, h, -0.5, 0.5, 0, 16)
    first, last = 1234, 23456
    rnb, rnc = O.find_neighbors(ref["x"], ref["y"], ref["z"], ref["h"], first, last, obox, ref["tree"],
                                ref["layout"], ref["centers"], ref["sizes"], ngmax, search_ext=1.25)
    nb, nc = cs.find_neighbors(tx, ty, tz, th, first, last, box, o, layout, c, s, ngmax, search_ext=1.25)
    torch.cuda.synchronize()
    neighbor_lists_equal(u32(nb), u32(nc), rnb, rnc, ngmax)


def test_neighbors_plummer(cs, O):
    n = 80000
    x, y, z = O.plummer(17, n)
    lo = (x.min(), y.min(), z.min())
    hi = (x.max(), y.max(), z.max())
    # adaptive h: from the distance to the 5th next particle in SFC order (as estimateH in the reference tests)
    obox = O.make_box(lo, hi)
    keys = O.sfc_keys(x, y, z, obox, 1, 64)
    _, perm = O.sort_by_key(keys)
    xs, ys, zs = x[perm], y[perm], z[perm]
    j = np.minimum(np.arange(n) + 5, n - 1)
    hs = 0.5001 * np.sqrt((xs - xs[j]) ** 2 + (ys - ys[j]) ** 2 + (zs - zs[j]) ** 2) + 1e-6
    h = np.empty(n)
    h[perm] = hs
    ngmax = 200
    ref, obox, box, o, layout, c, s, (tx, ty, tz, th) = _setup(O, cs, x, y, z, h, lo, hi, 0, 64)
    rnb, rnc = O.find_neighbors(ref["x"], ref["y"], ref["z"], ref["h"], 0, n, obox, ref["tree"], ref["layout"],
                                ref["centers"], ref["sizes"], ngmax)
    nb, nc = cs.find_neighbors(tx, ty, tz, th, 0, n, box, o, layout, c, s, ngmax)
    torch.cuda.synchronize()
    neighbor_lists_equal(u32(nb), u32(nc), rnb, rnc, ngmax)


def test_neighbors_duplicates(cs, O):
    """coincident particles: j == i is excluded, coincident j != i are neighbours (CPU semantics)"""
    n = 20000
    x, y, z = uniform(O, 61, n // 2, -1.0, 1.0)
    x, y, z = (np.concatenate([a, a]) for a in (x, y, z))
    h = np.full(n, 0.05)
    ngmax = 128
    ref, obox, box, o, layout, c, s, (tx, ty, tz, th) = _setup(O, cs, x, y, z, h, -1.0, 1.0, 0, 8)
    rnb, rnc = O.find_neighbors(ref["x"], ref["y"], ref["z"], ref["h"], 0, n, obox, ref["tree"], ref["layout"],
                                ref["centers"], ref["sizes"], ngmax)
    nb, nc = cs.find_neighbors(tx, ty, tz, th, 0, n, box, o, layout, c, s, ngmax)
    torch.cuda.synchronize()
    neighbor_lists_equal(u32(nb), u32(nc), rnb, rnc, ngmax)


@pytest.mark.parametrize("bits", [32, 64])
def test_neighbors_particles_outside_their_leaf_box(cs, O, bits):
    """The reference quantises int(floor(x * m) - xmin * m), which can key a point into the finest cell below its
    geometric one, so the point lies outside its leaf's box and the reference's traversal rejects some pairs within
    the radius. The GPU search rejects the same pairs. With 32-bit keys this input (the brute-force test's gaussian
    generator) holds such a pair."""
    import sys, os
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from kat_util import brute_force_neighbors

    radius, n = 0.0624, 2500
    lo, hi = np.array((-1.2, -0.213, -5.1)), np.array((0.23, 3.213, 1.23))
    rng = np.random.default_rng(713159802)
    pts = []
    for k in range(3):
        v = rng.normal((lo[k] + hi[k]) / 2, (hi[k] - lo[k]) / 5, 4 * n)
        pts.append(v[(v >= lo[k]) & (v < hi[k])][:n])
    x, y, z = pts
    h = np.full(n, radius / 2)
    ngmax = n
    ref, obox, box, o, layout, c, s, (tx, ty, tz, th) = _setup(O, cs, x, y, z, h, tuple(lo), tuple(hi), 0, 64, 1,
                                                                bits)
    rnb, rnc = O.find_neighbors(ref["x"], ref["y"], ref["z"], ref["h"], 0, n, obox, ref["tree"], ref["layout"],
                                ref["centers"], ref["sizes"], ngmax)
    nb, nc = cs.find_neighbors(tx, ty, tz, th, 0, n, box, o, layout, c, s, ngmax)
    torch.cuda.synchronize()
    neighbor_lists_equal(u32(nb), u32(nc), rnb, rnc, ngmax)
    if bits == 32:
        _, counts = brute_force_neighbors(ref["x"], ref["y"], ref["z"], ref["h"], lo, hi, False)
        assert (counts != rnc).any()  # the case is exercised: the reference drops a pair within the radius


def test_fp32_pair_at_the_radius_is_not_a_neighbour(cs, O):
    """FP32 coordinates: a candidate whose squared distance RN(RN(RN(dx dx) + RN(dy dy)) + RN(dz dz)) equals r2 exactly
    is not a neighbour (d2 < r2 is false), although the same sum with the first product fused into the add lies one
    ulp below r2. Forty coincident targets make every lane of the warp need the candidate's leaf, so the per-lane
    candidate loop decides it (the pair came from a 783k-particle uniform set of the batched workload)."""
    f = np.float32
    xi = (float.fromhex("0x1.f91c64p-3"), float.fromhex("0x1.388148p-5"), float.fromhex("0x1.2841eap-1"))
    xc = (float.fromhex("0x1.423806p-2"), float.fromhex("0x1.b76b46p-5"), float.fromhex("0x1.26c99cp-1"))
    hv = f(float.fromhex("0x1.1e079p-5"))
    d = [f(f(a) - f(b)) for a, b in zip(xc, xi)]
    assert f(f(f(d[0] * d[0]) + f(d[1] * d[1])) + f(d[2] * d[2])) == f(f(f(4) * hv) * hv)  # exactly at the radius
    rng = np.random.default_rng(23)
    fill = rng.random((3, 3000)).astype(f)
    x, y, z = (np.concatenate([np.full(40, a, f), [f(b)], fill[k]]) for k, (a, b) in enumerate(zip(xi, xc)))
    n = x.size
    h = np.full(n, hv, f)
    ngmax = 100
    ref, obox, box, o, layout, c, s, (tx, ty, tz, th) = _setup(O, cs, x, y, z, h, 0.0, 1.0, 0, 16, 0, 32)
    rnb, rnc = O.find_neighbors(ref["x"], ref["y"], ref["z"], ref["h"], 0, n, obox, ref["tree"], ref["layout"],
                                ref["centers"], ref["sizes"], ngmax)
    nb, nc = cs.find_neighbors(tx, ty, tz, th, 0, n, box, o, layout, c, s, ngmax)
    torch.cuda.synchronize()
    neighbor_lists_equal(u32(nb), u32(nc), rnb, rnc, ngmax)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("bucket", [4, 8])
def test_neighbors_lattice_at_the_radius_small_leaves(cs, O, dtype, bucket):
    """A cubic lattice whose face neighbours lie at the search radius up to the rounding of the coordinates (spacing
    2^-6, origin off the binary grid, h = spacing / 2): nearly every face pair falls in the band of the FP32 filter and
    is decided exactly, and the small buckets make the traversal merge adjoining leaves into one candidate batch, so
    the exact decisions also look up the leaf of a candidate inside a merged batch."""
    a = 1.0 / 64
    g = np.arange(24, dtype=np.float64)
    X, Y, Z = (v.ravel() for v in np.meshgrid(g, g, g, indexing="ij"))
    x = (0.3 + a * X).astype(dtype)
    y = (0.1 + a * Y).astype(dtype)
    z = (0.7 + a * Z).astype(dtype)
    n = x.size
    h = np.full(n, a / 2, dtype)
    lo = (0.3 - a, 0.1 - a, 0.7 - a)
    hi = (0.3 + 25 * a, 0.1 + 25 * a, 0.7 + 25 * a)
    ngmax = 32
    ref, obox, box, o, layout, c, s, (tx, ty, tz, th) = _setup(O, cs, x, y, z, h, lo, hi, 0, bucket)
    rnb, rnc = O.find_neighbors(ref["x"], ref["y"], ref["z"], ref["h"], 0, n, obox, ref["tree"], ref["layout"],
                                ref["centers"], ref["sizes"], ngmax)
    nb, nc = cs.find_neighbors(tx, ty, tz, th, 0, n, box, o, layout, c, s, ngmax)
    torch.cuda.synchronize()
    neighbor_lists_equal(u32(nb), u32(nc), rnb, rnc, ngmax)
    # the rounding of the coordinates puts some face pairs inside the radius and some outside
    assert 0 < rnc.sum() < 6 * n
