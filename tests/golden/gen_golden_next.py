"""Generate tests/golden/tree_ops.npz with the reference's OWN CPU code: upsweeps of counts and source centres,
spanning trees, and the focus-tree rebalance helpers (rebalanceDecisionEssential, macRefineOp, protectAncestors,
enforceKeys, rangeCount, computeNodeLayout) on a seeded Plummer tree.

Runs only where the reference sources are present (oracle/Makefile, target `ref`).

    python tests/golden/gen_golden_next.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402


def plummer_np(rng, n):
    u0, u1, u2 = rng.random(3 * n).reshape(3, n)
    r = 1.0 / np.sqrt(u0 ** (-2.0 / 3.0) - 1.0)
    keep = r < 100.0
    r, u1, u2 = r[keep], u1[keep], u2[keep]
    z = (1.0 - 2.0 * u1) * r
    phi = 2.0 * np.pi * u2
    rho = np.sqrt(r * r - z * z)
    return rho * np.cos(phi), rho * np.sin(phi), z


def tree_case(rng, n, bucket):
    x, y, z = plummer_np(rng, n)
    lo, hi = (x.min(), y.min(), z.min()), (x.max(), y.max(), z.max())
    box = O.make_box(lo, hi)
    keys = O.ref_sfc_keys(x, y, z, box)
    sk, perm = O.ref_sort_by_key(keys)
    leaves, counts, _ = O.ref_compute_octree(sk, bucket)
    tr = O.ref_build_octree(leaves)
    return x[perm], y[perm], z[perm], sk, leaves, counts, tr, lo, hi


def main():
    assert O.ref() is not None, "the reference sources are needed to generate golden fixtures"
    rng = np.random.default_rng(20241204)
    g = {}
    xs, ys, zs, sk, leaves, counts, tr, lo, hi = tree_case(rng, 8000, 16)
    N, L = tr.num_nodes, tr.num_leaves
    l2i = tr.leaf_to_internal[tr.num_internal:]
    g.update(x=xs, y=ys, z=zs, lo=np.array(lo), hi=np.array(hi), leaves=leaves, leaf_counts=counts)
    for f in ("prefixes", "child_offsets", "parents", "level_range", "internal_to_leaf", "leaf_to_internal"):
        g[f] = getattr(tr, f)

    # upsweep of counts
    nc = np.zeros(N, np.uint32)
    nc[l2i] = counts
    g["node_counts"] = O.upsweep_sum(tr.level_range, tr.child_offsets, nc, use_ref=True)

    # source centres: signed masses, f64 and f32
    m = rng.uniform(-1.0, 2.0, xs.size)
    layout = O.layout_from_counts(counts)
    g["m"] = m
    c64 = O.leaf_mass_centers(xs, ys, zs, m, l2i, layout, N, use_ref=True)
    g["centers_f64"] = O.upsweep_centers(tr.level_range, tr.child_offsets, c64, use_ref=True)
    c32 = O.leaf_mass_centers(xs.astype(np.float32), ys.astype(np.float32), zs.astype(np.float32),
                              m.astype(np.float32), l2i, layout, N, use_ref=True)
    g["centers_f32"] = O.upsweep_centers(tr.level_range, tr.child_offsets, c32, use_ref=True)

    # spanning trees of random sorted keys, 64 and 32 bits
    for bits in (64, 32):
        top = 1 << (63 if bits == 64 else 30)
        k = np.unique(rng.integers(1, top, 300, dtype=np.uint64))
        k = np.concatenate([[0], k, [top]]).astype(np.uint64)
        g[f"span_keys_{bits}"] = k
        g[f"span_tree_{bits}"] = O.ref_spanning_tree(k, bits)

    # focus rebalance on the tree above
    macs = (rng.random(N) < 0.3).astype(np.uint8)
    focus = (int(leaves[L // 3]), int(leaves[2 * L // 3]))
    g["macs"] = macs
    g["focus"] = np.array(focus, np.uint64)
    ops = O.rebalance_decision_essential(tr.prefixes, tr.child_offsets, tr.parents, g["node_counts"], macs, focus, 16,
                                         use_ref=True)
    g["ops_essential"] = ops
    pops, conv = O.protect_ancestors(tr.prefixes, tr.parents, ops, use_ref=True)
    g["ops_protected"], g["protect_converged"] = pops, np.array(conv)
    forced = np.sort(rng.choice(leaves[1:-1], 40, replace=False)).astype(np.uint64)
    forced = np.concatenate([forced, (forced[:10] + (np.uint64(1) << np.uint64(30))).astype(np.uint64)])
    eops, status = O.enforce_keys(forced, tr.prefixes, tr.child_offsets, tr.parents, pops, use_ref=True)
    g["forced_keys"], g["ops_enforced"], g["enforce_status"] = forced, eops, np.array(status)
    # a coarse tree (bucket 2000) decided with bucket 1: leaf counts far above the bucket give the 8/64/512 splits
    cleaves, ccounts, _ = O.ref_compute_octree(sk, 2000)
    ctr = O.ref_build_octree(cleaves)
    cnc = np.zeros(ctr.num_nodes, np.uint32)
    cnc[ctr.leaf_to_internal[ctr.num_internal:]] = ccounts
    cnc = O.upsweep_sum(ctr.level_range, ctr.child_offsets, cnc, use_ref=True)
    cmacs = (rng.random(ctr.num_nodes) < 0.5).astype(np.uint8)
    for f in ("prefixes", "child_offsets", "parents", "level_range"):
        g["coarse_" + f] = getattr(ctr, f)
    g["coarse_counts"], g["coarse_macs"] = cnc, cmacs
    cfocus = (0, int(cleaves[ctr.num_leaves // 2]))
    g["coarse_focus"] = np.array(cfocus, np.uint64)
    g["coarse_ops"] = O.rebalance_decision_essential(ctr.prefixes, ctr.child_offsets, ctr.parents, cnc, cmacs, cfocus,
                                                     1, use_ref=True)
    ffirst, flast = L // 3, 2 * L // 3
    g["mac_refine"] = np.array([O.ref().csr_mac_refine_op(O.C.c_uint64(int(tr.prefixes[l2i[i]])),
                                                          int(macs[l2i[i]]), 64)
                                if (i < ffirst or i >= flast) else 1 for i in range(L)], np.int32)
    g["focus_leaf_range"] = np.array([ffirst, flast], np.int32)

    # rangeCount: a fine global tree (bucket 4) against this tree, for focus leaves whose boundaries exist in it
    gleaves, gcounts, _ = O.ref_compute_octree(sk, 4)
    inside = np.isin(leaves[:-1], gleaves) & np.isin(leaves[1:], gleaves)
    idx = np.nonzero(inside)[0].astype(np.int32)
    g["global_leaves"], g["global_counts"], g["range_idx"] = gleaves, gcounts, idx
    g["range_counts"] = O.range_count(gleaves, gcounts, leaves, idx, use_ref=True)

    # computeNodeLayout: flags on nodes, the assigned range above
    flags = (rng.random(N) < 0.2).astype(np.uint8)
    g["layout_flags"] = flags
    g["node_layout"] = O.node_layout(counts, flags, l2i, ffirst, flast, use_ref=True)

    path = os.path.join(HERE, "tree_ops.npz")
    np.savez_compressed(path, **g)
    print(f"tree_ops.npz  {os.path.getsize(path) / 1024:.1f} KiB, {N} nodes, {L} leaves")


if __name__ == "__main__":
    main()
