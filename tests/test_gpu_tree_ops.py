"""GPU parity of the functions around the path: upsweeps of counts and source centres (one launch and level by
level), spanning trees and SFC gap filling, focus-tree rebalance helpers, node layout and target groups, against
golden fixtures made by the reference's own CPU code and against the oracle on larger trees. Integer results are
compared bit for bit; the source centres are floating point evaluated in the reference's CPU order, also bit for bit.
"""
import os

import numpy as np
import pytest
import torch

from gpu_util import keys_u, to_dev, u32

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def g():
    return np.load(os.path.join(GOLDEN, "tree_ops.npz"))


def _dev_keys(a, bits=64):
    a = np.ascontiguousarray(a, np.uint64)
    return torch.from_numpy(a.view(np.int64) if bits == 64 else a.astype(np.uint32).view(np.int32)).cuda()


def _i32(a):
    return torch.from_numpy(np.ascontiguousarray(a).astype(np.int64).astype(np.int32)).cuda()


def _leaf_l2i(g):
    L = g["leaves"].size - 1
    return g["leaf_to_internal"][g["prefixes"].size - L:]


@pytest.mark.parametrize("linked", [True, False])
def test_upsweep_counts_golden(cs, g, linked):
    nc = np.zeros(g["prefixes"].size, np.uint32)
    nc[_leaf_l2i(g)] = g["leaf_counts"]
    d = _i32(nc.view(np.int32))
    co = _i32(g["child_offsets"])
    if linked:
        cs.upsweep_sum(co, d, parents=_i32(g["parents"]))
    else:
        cs.upsweep_sum(co, d, level_range=g["level_range"])
    assert np.array_equal(u32(d), g["node_counts"])


@pytest.mark.parametrize("dt", ["f64", "f32"])
@pytest.mark.parametrize("linked", [True, False])
def test_source_centers_golden(cs, g, dt, linked):
    t = np.float64 if dt == "f64" else np.float32
    x, y, z, m = to_dev(*(g[c].astype(t) for c in "xyzm"))
    N = g["prefixes"].size
    cen = torch.zeros((N, 4), dtype=x.dtype, device=x.device)
    layout = _i32(np.concatenate([[0], np.cumsum(g["leaf_counts"])]))
    cs.leaf_source_centers(x, y, z, m, _i32(_leaf_l2i(g)), layout, cen)
    co = _i32(g["child_offsets"])
    if linked:
        cs.upsweep_source_centers(co, cen, parents=_i32(g["parents"]))
    else:
        cs.upsweep_source_centers(co, cen, level_range=g["level_range"])
    assert np.array_equal(cen.cpu().numpy(), g[f"centers_{dt}"])


def test_source_centers_f32_masses_match_oracle(cs, O, g):
    x, y, z = (g[c] for c in "xyz")
    m = g["m"].astype(np.float32)
    l2i = _leaf_l2i(g)
    layout = np.concatenate([[0], np.cumsum(g["leaf_counts"])]).astype(np.uint32)
    N = g["prefixes"].size
    ref = O.leaf_mass_centers(x, y, z, m, l2i, layout, N)
    tx, ty, tz = to_dev(x, y, z)
    cen = torch.zeros((N, 4), dtype=torch.float64, device="cuda")
    cs.leaf_source_centers(tx, ty, tz, torch.from_numpy(m).cuda(), _i32(l2i), _i32(layout), cen)
    assert np.array_equal(cen.cpu().numpy(), ref)


@pytest.mark.parametrize("bits", [64, 32])
def test_spanning_tree_and_gaps_golden(cs, g, bits):
    k = g[f"span_keys_{bits}"]
    ref = g[f"span_tree_{bits}"]
    out = cs.spanning_tree(_dev_keys(k, bits))
    assert np.array_equal(keys_u(out), ref)
    dk = _dev_keys(k, bits)
    ops = cs.count_sfc_gaps(dk)
    scan = torch.zeros(ops.numel() + 1, dtype=torch.int32, device="cuda")
    scan[1:] = torch.cumsum(ops, 0)
    filled = cs.fill_sfc_gaps(dk, scan)
    assert np.array_equal(keys_u(filled), ref)


def test_focus_rebalance_golden(cs, g):
    pre = _dev_keys(g["prefixes"])
    co, par = _i32(g["child_offsets"]), _i32(g["parents"])
    counts = _i32(g["node_counts"].view(np.int32))
    macs = torch.from_numpy(g["macs"]).cuda()
    focus = tuple(int(v) for v in g["focus"])
    ops = cs.rebalance_decision_essential(pre, co, par, counts, macs, focus, 16)
    assert np.array_equal(ops.cpu().numpy(), g["ops_essential"])
    cops = cs.rebalance_decision_essential(_dev_keys(g["coarse_prefixes"]), _i32(g["coarse_child_offsets"]),
                                           _i32(g["coarse_parents"]), _i32(g["coarse_counts"].view(np.int32)),
                                           torch.from_numpy(g["coarse_macs"]).cuda(),
                                           tuple(int(v) for v in g["coarse_focus"]), 1)
    assert np.array_equal(cops.cpu().numpy(), g["coarse_ops"])
    conv = cs.protect_ancestors(pre, par, ops)
    assert np.array_equal(ops.cpu().numpy(), g["ops_protected"]) and conv == bool(g["protect_converged"])
    st = cs.enforce_keys(_dev_keys(g["forced_keys"]), pre, co, par, ops)
    assert np.array_equal(ops.cpu().numpy(), g["ops_enforced"]) and st == int(g["enforce_status"])
    f0, f1 = (int(v) for v in g["focus_leaf_range"])
    l2i = _i32(_leaf_l2i(g))
    mr = cs.mac_refine_decision(pre, macs, l2i, f0, f1)
    assert np.array_equal(mr.cpu().numpy(), g["mac_refine"])
    idx = g["range_idx"]
    rc = cs.range_count(_dev_keys(g["global_leaves"]), _i32(g["global_counts"].view(np.int32)),
                        _dev_keys(g["leaves"]), _i32(idx))
    assert np.array_equal(u32(rc)[idx], g["range_counts"][idx])
    lay = cs.node_layout(_i32(g["leaf_counts"].view(np.int32)), torch.from_numpy(g["layout_flags"]).cuda(), l2i, f0,
                         f1)
    assert np.array_equal(u32(lay), g["node_layout"])


def _plummer_tree(cs, O, n, bucket, dtype=np.float64, seed=3):
    x, y, z = (a.astype(dtype) for a in O.plummer(seed, n))
    lo, hi = (float(x.min()), float(y.min()), float(z.min())), (float(x.max()), float(y.max()), float(z.max()))
    pipe = cs.Pipeline(64 if dtype == np.float64 else 32, 64, cs.HILBERT, bucket, 0, 1.0, 1.0, False, False)
    tx, ty, tz = to_dev(x, y, z)
    pipe.run(tx, ty, tz, torch.zeros_like(tx), cs.make_box(lo, hi))
    out = {k: v.clone() for k, v in pipe.outputs().items()}
    torch.cuda.synchronize()
    return out, lo, hi


def test_upsweeps_large_tree_against_oracle(cs, O):
    out, lo, hi = _plummer_tree(cs, O, 1 << 20, 16)
    N = out["prefixes"].numel()
    L = out["leaves"].numel() - 1
    l2i = out["leaf_to_internal"][N - L:]
    nc = torch.zeros(N, dtype=torch.int32, device="cuda")
    nc[l2i.long()] = out["counts"]
    lr = out["level_range"].cpu().numpy()
    ref = O.upsweep_sum(lr, out["child_offsets"].cpu().numpy(), u32(nc))
    a = cs.upsweep_sum(out["child_offsets"], nc.clone(), parents=out["parents"])
    b = cs.upsweep_sum(out["child_offsets"], nc.clone(), level_range=lr)
    assert np.array_equal(u32(a), ref) and np.array_equal(u32(b), ref)
    m = torch.rand(out["x"].numel(), dtype=torch.float64, device="cuda") + 0.5
    cen = torch.zeros((N, 4), dtype=torch.float64, device="cuda")
    cs.leaf_source_centers(out["x"], out["y"], out["z"], m, l2i, out["layout"], cen)
    cs.upsweep_source_centers(out["child_offsets"], cen, parents=out["parents"])
    rc = O.leaf_mass_centers(*(out[c].cpu().numpy() for c in "xyz"), m.cpu().numpy(), l2i.cpu().numpy(),
                             u32(out["layout"]), N)
    rc = O.upsweep_centers(lr, out["child_offsets"].cpu().numpy(), rc)
    assert np.array_equal(cen.cpu().numpy(), rc)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("group_size", [32, 64])
def test_group_splits_against_oracle(cs, O, dtype, group_size):
    out, lo, hi = _plummer_tree(cs, O, 200_000, 32, dtype)
    n = out["x"].numel()
    h = torch.full((n,), 0.01, dtype=out["x"].dtype, device="cuda")
    h[::7] = 0.5
    first, last = 17, n - 5
    box = cs.make_box(lo, hi)
    for tol, hh in ((8.0, h), (2.0, None)):
        grp = cs.group_splits(first, last, out["x"], out["y"], out["z"], hh, out["leaves"], out["layout"], box,
                              group_size, tol)
        ref = O.group_splits(first, last, *(out[c].cpu().numpy() for c in "xyz"),
                             hh.cpu().numpy() if hh is not None else None, keys_u(out["leaves"]), u32(out["layout"]),
                             lo, hi, group_size, tol)
        assert np.array_equal(u32(grp), ref), (tol, hh is None)
