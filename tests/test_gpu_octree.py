"""GPU parity: cornerstone leaf array (counts, decisions, computeOctree, updateOctree) and the linked internal tree
with node geometry, bit-exact against the oracle."""
import numpy as np
import pytest
import torch

from gpu_util import dev, gaussian_keys, keys_u, u32, uniform

pytestmark = pytest.mark.gpu


def _tkeys(keys, bits):
    return torch.from_numpy(keys.astype(np.uint64).view(np.int64) if bits == 64 else keys.astype(np.uint32).view(
        np.int32)).to(dev())


def _sorted_uniform_keys(O, n, bits, seed, kind=1):
    x, y, z = uniform(O, seed, n, -1.0, 1.0)
    return np.sort(O.sfc_keys(x, y, z, O.make_box(-1, 1), kind, bits))


def _plummer_keys(O, n, bits, seed=3):
    x, y, z = O.plummer(seed, n)
    box = O.make_box((x.min(), y.min(), z.min()), (x.max(), y.max(), z.max()))
    return np.sort(O.sfc_keys(x, y, z, box, 1, bits))


@pytest.mark.parametrize("bits", [32, 64])
@pytest.mark.parametrize("bucket", [1, 8, 16, 64, 1024])
@pytest.mark.parametrize("dist", ["uniform", "gaussian", "plummer"])
def test_compute_octree(cs, O, bits, bucket, dist):
    n = 60000
    if dist == "uniform":
        keys = _sorted_uniform_keys(O, n, bits, 1)
    elif dist == "gaussian":
        keys = gaussian_keys(n, bits, 4)
    else:
        keys = _plummer_keys(O, n, bits)
    rt, rc, rit = O.compute_octree(keys, bucket, bits)
    t, c, layout, it = cs.compute_octree(_tkeys(keys, bits), bucket)
    torch.cuda.synchronize()
    assert np.array_equal(keys_u(t), rt)
    assert np.array_equal(u32(c), rc)
    assert it == rit
    assert np.array_equal(u32(layout), O.layout_from_counts(rc))


@pytest.mark.parametrize("bits", [32, 64])
def test_compute_octree_edge_cases(cs, O, bits):
    top = 1 << (30 if bits == 32 else 63)
    cases = {
        "empty": np.zeros(0, np.uint64),
        "one": np.array([5], np.uint64),
        "all_equal": np.full(5000, 77, np.uint64),
        "max_depth": np.concatenate([np.zeros(300, np.uint64), np.arange(1, 200, dtype=np.uint64)]),
        "extremes": np.sort(np.array([0, 0, 1, top - 1, top - 1, top // 2] * 50, np.uint64)),
    }
    for name, keys in cases.items():
        for bucket in (1, 4, 64):
            rt, rc, rit = O.compute_octree(keys, bucket, bits)
            t, c, layout, it = cs.compute_octree(_tkeys(keys, bits), bucket)
            torch.cuda.synchronize()
            assert np.array_equal(keys_u(t), rt), (name, bucket)
            assert np.array_equal(u32(c), rc), (name, bucket)
            assert it == rit, (name, bucket)


def test_compute_octree_max_count(cs, O):
    keys = _sorted_uniform_keys(O, 50000, 64, 8)
    rt, rc, rit = O.compute_octree(keys, 64, 64, max_count=100)
    t, c, _, it = cs.compute_octree(_tkeys(keys, 64), 64, max_count=100)
    torch.cuda.synchronize()
    assert np.array_equal(keys_u(t), rt) and np.array_equal(u32(c), rc) and it == rit


def test_compute_octree_capacity_retry(cs, O):
    keys = _sorted_uniform_keys(O, 40000, 64, 2)
    rt, rc, _ = O.compute_octree(keys, 8, 64)
    t, c, _, _ = cs.compute_octree(_tkeys(keys, 64), 8, capacity=16)  # forces CS_ERR_CAPACITY and a retry
    torch.cuda.synchronize()
    assert np.array_equal(keys_u(t), rt) and np.array_equal(u32(c), rc)


@pytest.mark.parametrize("bits", [32, 64])
def test_node_counts_and_decision(cs, O, bits):
    keys = gaussian_keys(40000, bits, 12)
    tree, counts, _ = O.compute_octree(keys, 16, bits)
    keys2 = gaussian_keys(40000, bits, 13)  # other keys: counts change, decisions become non-trivial
    rc = O.node_counts(tree, keys2, bits)
    c = cs.node_counts(_tkeys(tree, bits), _tkeys(keys2, bits))
    torch.cuda.synchronize()
    assert np.array_equal(u32(c), rc)
    for bucket in (4, 16, 100):
        rops, rconv = O.rebalance_decision(tree, rc, bucket, bits)
        ops, conv = cs.rebalance_decision(_tkeys(tree, bits), c, bucket)
        torch.cuda.synchronize()
        assert np.array_equal(ops.cpu().numpy(), rops) and conv == rconv


@pytest.mark.parametrize("n", [0, 1, 2047, 2048, 2049, 100000, 3000001])
def test_exclusive_scan(cs, n):
    """exclusiveScan (primitives/primitives_gpu.h:158-160) on int32, out of place and in place, with an init value"""
    rng = np.random.default_rng(n)
    v = rng.integers(-50, 1000, n).astype(np.int32)
    ref = (np.concatenate([[0], np.cumsum(v.astype(np.int64))[:-1]]) + 7).astype(np.int32) if n else v
    t = torch.from_numpy(v).to(dev())
    out = cs.exclusive_scan(t, 7)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), ref)
    cs.exclusive_scan(t, 7, t)
    torch.cuda.synchronize()
    assert np.array_equal(t.cpu().numpy(), ref)


@pytest.mark.parametrize("bits", [32, 64])
def test_node_ops_and_rebalance_tree(cs, O, bits):
    """computeNodeOpsGpu + rebalanceTreeGpu (tree/csarray_gpu.cu:172-231): scanned ops, the new leaf count, the
    converged flag and the emitted leaves equal the oracle's rebalance step"""
    keys = gaussian_keys(40000, bits, 12)
    tree, _, _ = O.compute_octree(keys, 16, bits)
    keys2 = gaussian_keys(60000, bits, 14)
    counts = O.node_counts(tree, keys2, bits)
    for bucket in (4, 16, 100, 1 << 20):
        rops, rconv = O.rebalance_decision(tree, counts, bucket, bits)
        rnew = O.rebalance_tree(tree, rops, bits)
        tt = _tkeys(tree, bits)
        ops, L2, conv = cs.node_ops(tt, torch.from_numpy(counts.view(np.int32)).to(dev()), bucket)
        new_tree = cs.rebalance_tree(tt, ops)
        torch.cuda.synchronize()
        assert L2 == rnew.size - 1 and conv == rconv, bucket
        assert np.array_equal(ops.cpu().numpy()[:-1], np.concatenate([[0], np.cumsum(rops)[:-1]]).astype(np.int32))
        assert np.array_equal(keys_u(new_tree), rnew), bucket


@pytest.mark.parametrize("bits", [32, 64])
def test_update_octree_steps(cs, O, bits):
    n = 50000
    rng = np.random.default_rng(21)
    x, y, z = uniform(O, 5, n, 0.0, 1.0)
    box = O.make_box(0.0, 1.0)
    keys = np.sort(O.sfc_keys(x, y, z, box, 0, bits))
    tree, counts, _ = O.compute_octree(keys, 32, bits)
    ttree, tcounts = _tkeys(tree, bits), torch.from_numpy(counts.view(np.int32)).to(dev())
    for step in range(4):
        d = 0.1 * n ** (-1.0 / 3)
        x = np.mod(x + rng.normal(0, d, n), 1.0)
        y = np.mod(y + rng.normal(0, d, n), 1.0)
        z = np.mod(z + rng.normal(0, d, n), 1.0)
        keys = np.sort(O.sfc_keys(x, y, z, box, 0, bits))
        tree, counts, conv = O.update_octree(keys, 32, tree, counts, bits)
        ttree, tcounts, tconv = cs.update_octree(_tkeys(keys, bits), 32, ttree, tcounts)
        torch.cuda.synchronize()
        assert np.array_equal(keys_u(ttree), tree), step
        assert np.array_equal(u32(tcounts), counts), step
        assert tconv == conv, step


@pytest.mark.parametrize("bits", [32, 64])
@pytest.mark.parametrize("bucket", [1, 16, 64])
def test_build_octree_link(cs, O, bits, bucket):
    keys = _plummer_keys(O, 80000, bits, 9)
    leaves, _, _ = O.compute_octree(keys, bucket, bits)
    ref = O.build_octree(leaves, bits)
    o = cs.build_octree(_tkeys(leaves, bits))
    torch.cuda.synchronize()
    assert np.array_equal(keys_u(o.prefixes), ref.prefixes)
    assert np.array_equal(o.child_offsets[: o.num_nodes].cpu().numpy(), ref.child_offsets)
    assert np.array_equal(o.parents.cpu().numpy(), ref.parents)
    assert np.array_equal(o.level_range.cpu().numpy(), ref.level_range)
    assert np.array_equal(o.internal_to_leaf.cpu().numpy(), ref.internal_to_leaf)
    assert np.array_equal(o.leaf_to_internal.cpu().numpy(), ref.leaf_to_internal)


def test_build_octree_single_leaf(cs, O):
    leaves = np.array([0, 1 << 63], np.uint64)
    ref = O.build_octree(leaves, 64)
    o = cs.build_octree(_tkeys(leaves, 64))
    torch.cuda.synchronize()
    assert np.array_equal(keys_u(o.prefixes), ref.prefixes)
    assert np.array_equal(o.level_range.cpu().numpy(), ref.level_range)


@pytest.mark.parametrize("bits", [32, 64])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("kind", [0, 1])
def test_geo_centers(cs, O, bits, dtype, kind):
    keys = _plummer_keys(O, 30000, bits, 4)
    leaves, _, _ = O.compute_octree(keys, 8, bits)
    ref = O.build_octree(leaves, bits)
    lo, hi = (-3.25, -1.0, 0.5), (7.0, 2.0, 0.75)
    npdt = np.float32 if dtype == torch.float32 else np.float64
    rc, rs = O.node_fp_centers(ref.prefixes, O.make_box(lo, hi), npdt, kind, bits)
    c, s = cs.geo_centers(_tkeys(ref.prefixes, bits), cs.make_box(lo, hi), dtype, kind)
    torch.cuda.synchronize()
    assert np.array_equal(c.cpu().numpy(), rc)
    assert np.array_equal(s.cpu().numpy(), rs)
