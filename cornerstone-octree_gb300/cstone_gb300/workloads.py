"""Seeded synthetic inputs for the benchmark configurations (no dataset is involved).

- uniform(n, lo, hi, seed): i.i.d. uniform coordinates in a box.
- plummer(n, seed): Plummer sphere with scale radius 1 truncated at r = 100 (R = (u^(-2/3) - 1)^(-1/2),
  z = (1 - 2u) R, phi = 2 pi u), shifted to its centre of mass.
- h_for_k_neighbors(...): per-particle smoothing length such that exactly k other particles lie within 2h
  (the k-th nearest-neighbour distance, up to the gap to the (k+1)-th), found by per-particle bisection on
  neighbour counts computed with this library's own GPU search. This is input preparation, not part of the path.
"""
import types

import numpy as np
import torch

from . import HILBERT, Pipeline, find_neighbors


def uniform(n, lo, hi, seed, dtype=np.float64):
    rng = np.random.default_rng(seed)
    return [rng.uniform(lo, hi, n).astype(dtype) for _ in range(3)]


def plummer(n, seed, rmax=100.0):
    rng = np.random.default_rng(seed)
    xs, ys, zs = [], [], []
    need = n
    while need > 0:
        m = int(need * 1.01) + 64
        u0 = rng.random(m)
        u1 = rng.random(m)
        u2 = rng.random(m)
        ok = u0 > 0
        r = np.full(m, np.inf)
        r[ok] = 1.0 / np.sqrt(u0[ok] ** (-2.0 / 3.0) - 1.0)
        keep = r < rmax
        r, u1, u2 = r[keep][:need], u1[keep][:need], u2[keep][:need]
        zz = (1.0 - 2.0 * u1) * r
        phi = 2.0 * np.pi * u2
        rho = np.sqrt(r * r - zz * zz)
        xs.append(rho * np.cos(phi))
        ys.append(rho * np.sin(phi))
        zs.append(zz)
        need -= r.size
    x, y, z = (np.concatenate(a) for a in (xs, ys, zs))
    return x - x.mean(), y - y.mean(), z - z.mean()


def tight_box(x, y, z):
    return (float(x.min()), float(y.min()), float(z.min())), (float(x.max()), float(y.max()), float(z.max()))


def h_for_k_neighbors(x, y, z, box, k=100, bucket=64, key_bits=64, kind=HILBERT, max_iter=64):
    """x, y, z: device tensors (input order). Returns h (input order) and the final neighbour counts."""
    n = x.numel()
    coord_bits = 64 if x.dtype == torch.float64 else 32
    pipe = Pipeline(coord_bits, key_bits, kind, bucket, ngmax=0, do_halos=False, do_neighbors=False)
    pipe.run(x, y, z, torch.zeros_like(x), box)
    out = {key: v.clone() for key, v in pipe.outputs().items()}
    r = pipe.result
    tree = types.SimpleNamespace(num_leaves=r.num_leaves, num_nodes=r.num_nodes,
                                 child_offsets=out["child_offsets"], parents=out["parents"],
                                 internal_to_leaf=out["internal_to_leaf"])
    xs, ys, zs = out["x"], out["y"], out["z"]
    idx = torch.arange(n, device=x.device)
    j = torch.where(idx + k < n, idx + k, (idx - k).clamp(min=0))
    h = 0.5 * torch.sqrt((xs - xs[j]) ** 2 + (ys - ys[j]) ** 2 + (zs - zs[j]) ** 2)
    h = torch.where(h > 0, h, torch.full_like(h, float(h[h > 0].min()) if bool((h > 0).any()) else 1e-3))
    lo = torch.zeros_like(h)
    hi = torch.full_like(h, float("inf"))
    dummy = torch.empty((1, 1), dtype=torch.int32, device=x.device)
    nc = torch.empty(n, dtype=torch.int32, device=x.device)
    for _ in range(max_iter):
        find_neighbors(xs, ys, zs, h, 0, n, box, tree, out["layout"], out["centers"], out["sizes"], 0,
                       out=(dummy, nc))
        low = nc < k
        high = nc > k
        if not bool((low | high).any()):
            break
        lo = torch.where(low, h, lo)
        hi = torch.where(high, h, hi)
        ratio = (k / nc.clamp(min=1).to(h.dtype)) ** (1.0 / 3.0)
        bracketed = (lo > 0) & torch.isfinite(hi)
        grow = h * ratio.clamp(1.02, 4.0)
        shrink = h * ratio.clamp(0.25, 0.98)
        h_new = torch.where(bracketed, 0.5 * (lo + hi), torch.where(low, grow, shrink))
        h = torch.where(low | high, h_new, h)
    h_in = torch.empty_like(h)
    h_in[out["order"].long()] = h
    nc_in = torch.empty_like(nc)
    nc_in[out["order"].long()] = nc
    return h_in, nc_in
