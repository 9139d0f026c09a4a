"""Seeded synthetic inputs of the benchmark configurations, in plain numpy (no dataset is involved).

This module imports neither torch nor the CUDA library, so that the CPU reference arm of the benchmark and the tests'
oracle runs can build exactly the same inputs as the GPU arm without loading libcstone_gb300.so.

- uniform(n, lo, hi, seed): i.i.d. uniform coordinates in a box.
- plummer(n, seed): Plummer sphere with scale radius 1 truncated at r = 100 (R = (u^(-2/3) - 1)^(-1/2),
  z = (1 - 2u) R, phi = 2 pi u), shifted to its centre of mass.
- tight_box(x, y, z): per-axis min/max.
"""
import numpy as np


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
