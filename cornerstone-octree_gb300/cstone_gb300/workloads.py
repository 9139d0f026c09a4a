"""Seeded synthetic inputs for the benchmark configurations (no dataset is involved).

- uniform, plummer, tight_box: the numpy generators of cstone_synth (re-exported).
- batched_sets(...): the batched workload's sets, generated on the device.
- h_for_k_neighbors(...): per-particle smoothing length such that exactly k other particles lie within 2h
  (the k-th nearest-neighbour distance, up to the gap to the (k+1)-th), found by per-particle bisection on
  neighbour counts computed with this library's own GPU search. This is input preparation, not part of the path.
"""
import os
import sys
import types

import numpy as np
import torch

from . import HILBERT, Pipeline, find_neighbors

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from cstone_synth import plummer, tight_box, uniform  # noqa: E402  (numpy-only generators, shared with the CPU arm)


def batched_sets(num_sets, seed, device, lo_exp=10, hi_exp=20, k=60):
    """The batched workload: num_sets independent FP32 sets, sizes n_s = floor(2^(lo_exp + (hi_exp - lo_exp) u))
    (log-uniform), uniform in the unit cube or Plummer with a tight box (alternating 50/50), bucket sizes drawn from
    {16, 32, 64}, per-set constant h: for a uniform set 0.5 * (3 k / (4 pi n / V))^(1/3) (about k neighbours within
    2h), for a Plummer set the same formula on the volume of the sphere holding half the particles (about k
    neighbours at the half-mass radius). Generated on the device with a seeded torch generator.
    Returns (list of dicts with n, x, y, z, h device tensors, lo, hi, bucket)."""
    g = torch.Generator(device=device).manual_seed(seed)
    rng = np.random.default_rng(seed)
    sets = []
    for s in range(num_sets):
        n = int(2 ** (lo_exp + (hi_exp - lo_exp) * rng.random()))
        bucket = int(rng.choice([16, 32, 64]))
        if s % 2 == 0:
            x, y, z = (torch.rand(n, generator=g, device=device, dtype=torch.float32) for _ in range(3))
            lo, hi = (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)
            hval = 0.5 * (3 * k / (4 * np.pi * n)) ** (1 / 3)
        else:
            u = torch.rand(3, int(n * 1.01) + 64, generator=g, device=device, dtype=torch.float64)
            r = 1.0 / torch.sqrt(u[0].clamp_min(1e-300) ** (-2.0 / 3.0) - 1.0)
            keep = r < 100.0
            r, u1, u2 = r[keep][:n], u[1][keep][:n], u[2][keep][:n]
            while r.numel() < n:  # rare: top up the rejected ones
                v = torch.rand(3, n, generator=g, device=device, dtype=torch.float64)
                rr = 1.0 / torch.sqrt(v[0].clamp_min(1e-300) ** (-2.0 / 3.0) - 1.0)
                kk = rr < 100.0
                m = n - r.numel()
                r = torch.cat([r, rr[kk][:m]])
                u1 = torch.cat([u1, v[1][kk][:m]])
                u2 = torch.cat([u2, v[2][kk][:m]])
            zz = (1.0 - 2.0 * u1) * r
            phi = 2.0 * np.pi * u2
            rho = torch.sqrt(r * r - zz * zz)
            x, y, z = (a.float() for a in (rho * torch.cos(phi), rho * torch.sin(phi), zz))
            lo = (float(x.min()), float(y.min()), float(z.min()))
            hi = (float(x.max()), float(y.max()), float(z.max()))
            rhalf = 1.0 / np.sqrt(0.5 ** (-2.0 / 3.0) - 1.0)  # half-mass radius of a Plummer sphere of scale 1
            hval = 0.5 * (3 * k / (4 * np.pi * (n / 2) / (4 / 3 * np.pi * rhalf ** 3))) ** (1 / 3)
        h = torch.full((n,), hval, device=device, dtype=torch.float32)
        sets.append(dict(n=n, x=x, y=y, z=z, h=h, lo=lo, hi=hi, bucket=bucket))
    return sets


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


def chunk_sets(sets, chunk_cap=64 * 1024 * 1024):
    """groups consecutive sets of batched_sets(...) into chunks of at most chunk_cap particles (a larger set forms a
    chunk of its own); per chunk: (set indices, offsets[len + 1], concatenated x, y, z, h device tensors)"""
    chunks, cur, acc = [], [], 0
    for s, st in enumerate(sets):
        if cur and acc + st["n"] > chunk_cap:
            chunks.append(cur)
            cur, acc = [], 0
        cur.append(s)
        acc += st["n"]
    if cur:
        chunks.append(cur)
    packed = []
    for ch in chunks:
        offs = np.concatenate([[0], np.cumsum([sets[s]["n"] for s in ch])])
        xyzh = [torch.cat([sets[s][c] for s in ch]) for c in "xyzh"]
        packed.append((ch, offs, xyzh))
    return packed
