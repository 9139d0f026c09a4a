"""Generate the golden fixtures of this directory with the reference's OWN CPU code.

Runs only where the reference sources are present: it builds oracle/_ref/libcsref.so from the reference headers in
place (oracle/Makefile, target `ref`) and stores seeded inputs together with the reference's outputs as compressed
.npz files. The CPU tests check the oracle against these files, the GPU tests check the CUDA path against them.

    python tests/golden/gen_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402


def save(name, **arrays):
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **arrays)
    print(f"{name}.npz  {os.path.getsize(path) / 1024:.1f} KiB")


def plummer_np(rng, n):
    u0, u1, u2 = rng.random(3 * n).reshape(3, n)
    r = 1.0 / np.sqrt(u0 ** (-2.0 / 3.0) - 1.0)
    keep = r < 100.0
    r, u1, u2 = r[keep], u1[keep], u2[keep]
    z = (1.0 - 2.0 * u1) * r
    phi = 2.0 * np.pi * u2
    rho = np.sqrt(r * r - z * z)
    x, y = rho * np.cos(phi), rho * np.sin(phi)
    return x - x.mean(), y - y.mean(), z - z.mean()


def main():
    assert O.ref() is not None, "the reference sources are needed to generate golden fixtures"
    rng = np.random.default_rng(20240601)

    # ---- keys: both curves, both widths, f32/f64, open and periodic anisotropic boxes ----
    keys = {}
    for dt, dname in ((np.float64, "f64"), (np.float32, "f32")):
        for bi, (lo, hi, bnd) in enumerate((((-1.0,) * 3, (1.0,) * 3, 0), ((-1.2, -0.213, -5.1), (0.23, 3.213, 1.23), 1))):
            box = O.make_box(lo, hi, bnd)
            xyz = [rng.uniform(lo[k], hi[k], 1000).astype(dt) for k in range(3)]
            for k in range(3):
                xyz[k][:2] = [dt(lo[k]), dt(hi[k])]
            keys[f"x_{dname}_{bi}"], keys[f"y_{dname}_{bi}"], keys[f"z_{dname}_{bi}"] = xyz
            keys[f"lo_{bi}"], keys[f"hi_{bi}"], keys[f"bnd_{bi}"] = np.array(lo), np.array(hi), np.array(bnd)
            for kind in (0, 1):
                for bits in (32, 64):
                    keys[f"keys_{dname}_{bi}_{kind}_{bits}"] = O.ref_sfc_keys(*xyz, box, kind, bits)
    save("keys", **keys)

    # ---- stable sort with many duplicates ----
    k = rng.integers(0, 1 << 63, size=6000, dtype=np.uint64)
    k[rng.integers(0, 6000, 2000)] = k[rng.integers(0, 6000, 2000)]
    sk, perm = O.ref_sort_by_key(k)
    save("sort", keys=k, sorted_keys=sk, perm=perm)

    # ---- tree: Plummer keys, builds at two bucket sizes, link, geometry, halos, neighbours ----
    x, y, z = plummer_np(rng, 9000)
    lo = (x.min(), y.min(), z.min())
    hi = (x.max(), y.max(), z.max())
    box = O.make_box(lo, hi)
    keys64 = O.ref_sfc_keys(x, y, z, box, 1, 64)
    sk, perm = O.ref_sort_by_key(keys64)
    xs, ys, zs = x[perm], y[perm], z[perm]
    out = dict(x=x, y=y, z=z, lo=np.array(lo), hi=np.array(hi), sorted_keys=sk, perm=perm)
    for bucket in (8, 64):
        t, c, it = O.ref_compute_octree(sk, bucket, 64)
        out[f"leaves_b{bucket}"], out[f"counts_b{bucket}"], out[f"iterations_b{bucket}"] = t, c, np.array(it)
    leaves = out["leaves_b8"]
    tr = O.ref_build_octree(leaves, 64)
    out.update(prefixes=tr.prefixes, child_offsets=tr.child_offsets, parents=tr.parents, level_range=tr.level_range,
               internal_to_leaf=tr.internal_to_leaf, leaf_to_internal=tr.leaf_to_internal)
    cen, siz = O.ref_node_fp_centers(tr.prefixes, box, np.float64, 64)
    out.update(centers=cen, sizes=siz)
    layout = O.layout_from_counts(out["counts_b8"])
    # h: distance to the 20th next particle in SFC order (as estimateH in the reference test fixtures), + 2% noise
    j = np.minimum(np.arange(xs.size) + 20, xs.size - 1)
    hs = 0.5001 * np.sqrt((xs - xs[j]) ** 2 + (ys - ys[j]) ** 2 + (zs - zs[j]) ** 2) * rng.uniform(1, 1.02, xs.size)
    hs[hs == 0] = hs[hs > 0].min()
    out["h_sorted"] = hs
    first, last = 0, int(np.searchsorted(leaves, np.uint64(1) << np.uint64(61)))
    l2i = tr.leaf_to_internal[tr.num_internal:]
    sc, ss = O.ref_search_boxes(xs, ys, zs, hs, layout, first, last, 2.0, l2i, cen)
    flags = O.ref_find_halos(tr, cen, siz, sc, ss, box, first, last, 64)
    out.update(focus=np.array([first, last]), search_centers=sc[first:last], search_sizes=ss[first:last],
               halo_flags=flags)
    ngmax = 48
    nb, nc = O.ref_find_neighbors(xs, ys, zs, hs, 0, xs.size, box, tr, layout, cen, siz, ngmax)
    mask = np.arange(ngmax)[None, :] < np.minimum(nc, ngmax)[:, None]
    out.update(ngmax=np.array(ngmax), nc=nc, nb_flat=nb[mask])
    save("plummer_tree", **out)

    # ---- f32, 32-bit Hilbert keys, periodic box: tree + neighbours ----
    n = 4000
    x, y, z = (rng.uniform(0.0, 1.0, n).astype(np.float32) for _ in range(3))
    box = O.make_box(0.0, 1.0, 1)
    keys32 = O.ref_sfc_keys(x, y, z, box, 1, 32)
    sk, perm = O.ref_sort_by_key(keys32)
    xs, ys, zs = x[perm], y[perm], z[perm]
    t, c, it = O.ref_compute_octree(sk, 16, 32)
    tr = O.ref_build_octree(t, 32)
    cen, siz = O.ref_node_fp_centers(tr.prefixes, box, np.float32, 32)
    hs = np.full(n, 0.06, np.float32)
    ngmax = 64
    nb, nc = O.ref_find_neighbors(xs, ys, zs, hs, 0, n, box, tr, O.layout_from_counts(c), cen, siz, ngmax)
    mask = np.arange(ngmax)[None, :] < np.minimum(nc, ngmax)[:, None]
    save("periodic_f32", x=x, y=y, z=z, sorted_keys=sk, perm=perm, leaves=t, counts=c, iterations=np.array(it),
         prefixes=tr.prefixes, child_offsets=tr.child_offsets, centers=cen, sizes=siz, h_sorted=hs,
         ngmax=np.array(ngmax), nc=nc, nb_flat=nb[mask])


if __name__ == "__main__":
    main()
