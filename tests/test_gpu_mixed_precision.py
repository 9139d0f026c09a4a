"""GPU parity of the double-coordinate / float-h entry points (the reference's findNeighbors and
computeBoundingBoxGpu instantiated with Tc = double, Th = float) against the oracle, bit for bit."""
import numpy as np
import pytest
import torch

from gpu_util import neighbor_lists_equal, to_dev, u32

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("bnd", [0, 1])
def test_find_neighbors_and_search_boxes_f64_coordinates_f32_h(cs, O, bnd):
    rng = np.random.default_rng(31 + bnd)
    n, ngmax = 60_000, 96
    x, y, z = (rng.random(n) for _ in range(3))
    h = (0.012 + 0.01 * rng.random(n)).astype(np.float32)
    obox = O.make_box(0.0, 1.0, bnd)
    sk, perm = O.sort_by_key(O.sfc_keys(x, y, z, obox))
    xs, ys, zs, hs = x[perm], y[perm], z[perm], h[perm]
    lv, ct, _ = O.compute_octree(sk, 16)
    tr = O.build_octree(lv)
    cen, siz = O.node_fp_centers(tr.prefixes, obox)
    lay = O.layout_from_counts(ct)
    rnb, rnc = O.find_neighbors(xs, ys, zs, hs, 0, n, obox, tr, lay, cen, siz, ngmax)

    box = cs.make_box(0.0, 1.0, bnd)
    tlv = torch.from_numpy(lv.view(np.int64)).cuda()
    o = cs.build_octree(tlv)
    tx, ty, tz = to_dev(xs, ys, zs)
    th = torch.from_numpy(hs).cuda()
    tl = torch.from_numpy(lay.astype(np.int32)).cuda()
    tc, tsz = to_dev(cen, siz)
    nb, nc = cs.find_neighbors(tx, ty, tz, th, 0, n, box, o, tl, tc, tsz, ngmax)
    torch.cuda.synchronize()
    neighbor_lists_equal(u32(nb), u32(nc), rnb, rnc, ngmax)

    l2i = tr.leaf_to_internal[tr.num_internal:]
    rsc, rss = O.search_boxes(xs, ys, zs, hs, lay, 0, tr.num_leaves, 2.0, l2i, cen)
    sc, ss = cs.search_boxes(tx, ty, tz, th, tl, 0, tr.num_leaves, 2.0, torch.from_numpy(l2i).cuda(), tc)
    assert np.array_equal(sc.cpu().numpy(), rsc) and np.array_equal(ss.cpu().numpy(), rss)
