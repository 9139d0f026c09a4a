"""GPU parity of the neighbour-list consumers (ijLoop with an SPH density interaction).

- Over the stored neighbour lists: equals the oracle's loop over the CPU full lists (the reference's
  CpuFullNbListNeighborhood::jLoop, traversal/ijloop/cpu_fullnblist.hpp:94-112) bit for bit, open and periodic boxes.
- Over cluster-pair lists: equals the oracle's brute-force sum over every pair within 2 h_i, in ascending j, bit for
  bit (the lists cover every neighbour; the loop adds them in ascending j).
"""
import types

import numpy as np
import pytest
import torch

from gpu_util import to_dev, uniform

pytestmark = pytest.mark.gpu


def _gpu_tree(cs, x, y, z, h, box, bucket, ngmax, coord_bits):
    pipe = cs.Pipeline(coord_bits, 64, cs.HILBERT, bucket, ngmax, 1.0, 1.0, False, ngmax > 0)
    tx, ty, tz, th = to_dev(x, y, z, h)
    r = pipe.run(tx, ty, tz, th, box)
    out = {k: v.clone() for k, v in pipe.outputs().items()}
    torch.cuda.synchronize()
    tree = types.SimpleNamespace(num_leaves=r.num_leaves, num_nodes=r.num_nodes, child_offsets=out["child_offsets"],
                                 parents=out["parents"], internal_to_leaf=out["internal_to_leaf"])
    return out, tree


@pytest.mark.parametrize("case", ["plummer_f64", "uniform_periodic_f32"])
def test_density_over_stored_lists(cs, O, case):
    n, ngmax = 1 << 16, 128
    if case == "plummer_f64":
        x, y, z = O.plummer(21, n)
        lo, hi = (x.min(), y.min(), z.min()), (x.max(), y.max(), z.max())
        bnd = 0
        h = O.h_for_k_neighbors_cpu(x, y, z, O.make_box(lo, hi), 60)
        dt = np.float64
    else:
        x, y, z = uniform(O, 22, n, 0.0, 1.0, np.float32)
        lo, hi, bnd = (0.0,) * 3, (1.0,) * 3, 1
        h = np.full(n, 1.2 * n ** (-1 / 3), np.float32)
        dt = np.float32
    m = np.random.default_rng(3).uniform(0.5, 1.5, n).astype(dt)
    obox = O.make_box(lo, hi, bnd)
    ref = O.pipeline(x, y, z, h, obox, 32, ngmax)
    rho_ref = O.ijloop_density_list(ref["x"], ref["y"], ref["z"], ref["h"], m[ref["perm"]], 0, n, obox, ref["nb"],
                                    ref["nc"], ngmax)
    out, _ = _gpu_tree(cs, x, y, z, h, cs.make_box(lo, hi, bnd), 32, ngmax, 64 if dt == np.float64 else 32)
    tm = torch.from_numpy(m).cuda()[out["order"].long()]
    rho = cs.ijloop_density_list(out["x"], out["y"], out["z"], out["h"], tm, cs.make_box(lo, hi, bnd),
                                 out["neighbors"], out["neighbor_counts"])
    assert np.array_equal(rho.cpu().numpy(), rho_ref)


@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_density_over_cluster_lists(cs, O, dt):
    n = 30_000
    x, y, z = (a.astype(dt) for a in O.plummer(23, n))
    lo, hi = (float(x.min()), float(y.min()), float(z.min())), (float(x.max()), float(y.max()), float(z.max()))
    # a spread of smoothing lengths: small in the core, large outside
    r = np.sqrt(x.astype(np.float64) ** 2 + y ** 2 + z ** 2)
    h = (0.05 + 0.1 * r).astype(dt)
    m = np.random.default_rng(4).uniform(0.5, 1.5, n).astype(dt)
    out, tree = _gpu_tree(cs, x, y, z, h, cs.make_box(lo, hi), 16, 0, 64 if dt == np.float64 else 32)
    box = cs.make_box(lo, hi)
    lists, counts = cs.cluster_nblist(out["x"], out["y"], out["z"], out["h"], box, tree, out["layout"],
                                      out["centers"].reshape(-1), out["sizes"].reshape(-1), 64, 64)
    tm = torch.from_numpy(m).cuda()[out["order"].long()]
    rho = cs.ijloop_density_clusters(out["x"], out["y"], out["z"], out["h"], tm, lists, counts)
    ref = O.ijloop_density_all(*(out[c].cpu().numpy() for c in ("x", "y", "z", "h")), tm.cpu().numpy(),
                               O.make_box(lo, hi))
    assert np.array_equal(rho.cpu().numpy(), ref)
    # the lists are ascending and without repeats
    c = counts.cpu().numpy()
    L = lists.cpu().numpy()
    for k in range(0, c.size, 97):
        row = L[k, : c[k]]
        assert np.all(np.diff(row) > 0)


def test_cluster_lists_reject_periodic_boxes(cs, O):
    n = 4096
    x, y, z = uniform(O, 5, n, 0.0, 1.0)
    h = np.full(n, 0.05)
    out, tree = _gpu_tree(cs, x, y, z, h, cs.make_box(0.0, 1.0), 16, 0, 64)
    with pytest.raises(cs.CsError) as e:
        cs.cluster_nblist(out["x"], out["y"], out["z"], out["h"], cs.make_box(0.0, 1.0, cs.PERIODIC), tree,
                          out["layout"], out["centers"].reshape(-1), out["sizes"].reshape(-1))
    assert e.value.code == cs.CS_ERR_INVALID


@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_cluster_density_screen_edge_cases(cs, O, dt):
    """Pairs at 2 h_i to within a few ulps, far from the origin (where float coordinates carry an error of a tenth of
    the lattice spacing): the loop's float screen may keep extra pairs but drops none that the exact test keeps."""
    rng = np.random.default_rng(77)
    s, off = 0.01, 3000.0
    g = np.stack(np.meshgrid(np.arange(16), np.arange(16), np.arange(32), indexing="ij"), -1).reshape(-1, 3)
    n = g.shape[0]
    pos = off + s * g + rng.normal(0.0, 1e-13, g.shape)
    x, y, z = (np.ascontiguousarray(pos[:, k]).astype(dt) for k in range(3))
    # 2 h at a lattice distance (1, sqrt 2, sqrt 3, 2 spacings), nudged by a few ulps either way
    base = s * np.sqrt(rng.choice([1.0, 2.0, 3.0, 4.0], n)) / 2
    ulp = np.spacing(base.astype(dt)).astype(np.float64)
    h = (base + rng.integers(-3, 4, n) * ulp).astype(dt)
    m = rng.uniform(0.5, 1.5, n).astype(dt)
    lo = (float(x.min()), float(y.min()), float(z.min()))
    hi = (float(x.max()), float(y.max()), float(z.max()))
    out, tree = _gpu_tree(cs, x, y, z, h, cs.make_box(lo, hi), 16, 0, 64 if dt == np.float64 else 32)
    box = cs.make_box(lo, hi)
    lists, counts = cs.cluster_nblist(out["x"], out["y"], out["z"], out["h"], box, tree, out["layout"],
                                      out["centers"].reshape(-1), out["sizes"].reshape(-1), 64, 64)
    tm = torch.from_numpy(m).cuda()[out["order"].long()]
    rho = cs.ijloop_density_clusters(out["x"], out["y"], out["z"], out["h"], tm, lists, counts)
    ref = O.ijloop_density_all(*(out[c].cpu().numpy() for c in ("x", "y", "z", "h")), tm.cpu().numpy(),
                               O.make_box(lo, hi))
    assert np.array_equal(rho.cpu().numpy(), ref)
