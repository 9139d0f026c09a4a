"""Helpers shared by the GPU parity tests: seeded inputs and device/host conversions."""
import numpy as np
import torch


def dev():
    return torch.device("cuda:0")


def to_dev(*arrays):
    return [torch.from_numpy(np.ascontiguousarray(a)).to(dev()) for a in arrays]


def u64(t):
    return t.detach().cpu().numpy().view(np.uint64)


def u32(t):
    return t.detach().cpu().numpy().view(np.uint32)


def keys_u(t):
    a = t.detach().cpu().numpy()
    return a.view(np.uint64) if a.dtype == np.int64 else a.view(np.uint32).astype(np.uint64)


def uniform(O, seed, n, lo, hi, dtype=np.float64):
    return [O.philox_uniform(seed, s, n, lo, hi).astype(dtype) for s in range(3)]


def gaussian_keys(n, bits, seed):
    """sorted keys ~ N(mid, range/5), clipped to the key range (as makeRandomGaussianKeys in the reference tests)"""
    rng = np.random.default_rng(seed)
    top = float((1 << (30 if bits == 32 else 63)) - 1)
    v = rng.normal(top / 2, top / 5, size=3 * n)
    v = v[(v >= 0) & (v <= top)][:n]
    return np.sort(v.astype(np.uint64))


def neighbor_lists_equal(nb_gpu, nc_gpu, nb_ref, nc_ref, ngmax):
    assert np.array_equal(nc_gpu, nc_ref), f"counts differ at {np.nonzero(nc_gpu != nc_ref)[0][:10]}"
    mask = np.arange(ngmax)[None, :] < np.minimum(nc_ref, ngmax)[:, None]
    a = np.where(mask, nb_gpu, 0)
    b = np.where(mask, nb_ref, 0)
    bad = np.nonzero((a != b).any(axis=1))[0]
    assert bad.size == 0, f"neighbour lists differ for particles {bad[:10]}"
