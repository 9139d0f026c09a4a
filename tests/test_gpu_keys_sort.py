"""GPU parity: SFC keys, stable radix sort and gathers through the C ABI, bit-exact against the oracle."""
import numpy as np
import pytest
import torch

from gpu_util import dev, keys_u, to_dev, u32, uniform

pytestmark = pytest.mark.gpu

BOXES = [((-1.0, 1.0), 0), ((0.0, 1.0), 1), ((-0.7, 1.3), 0), (((-2.5, 0.1, 3.0), (4.0, 0.2, 3.5)), 0)]


def _box_args(spec):
    (lo, hi), bnd = spec
    return lo, hi, bnd


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("bits", [32, 64])
@pytest.mark.parametrize("boxspec", BOXES)
def test_keys(cs, O, dtype, kind, bits, boxspec):
    lo, hi, bnd = _box_args(boxspec)
    n = 100003
    los = np.broadcast_to(np.asarray(lo, float), 3)
    his = np.broadcast_to(np.asarray(hi, float), 3)
    xyz = [O.philox_uniform(11, s, n, los[s], his[s]).astype(dtype) for s in range(3)]
    # include the box corners, which quantise to the largest integer coordinate
    for a, l, h in zip(xyz, los, his):
        a[:2] = [dtype(l), dtype(h)]
    ref = O.sfc_keys(*xyz, O.make_box(lo, hi, bnd), kind, bits)
    tx, ty, tz = to_dev(*xyz)
    k = cs.sfc_keys(tx, ty, tz, cs.make_box(lo, hi, bnd), kind, bits)
    torch.cuda.synchronize()
    assert np.array_equal(keys_u(k), ref)


@pytest.mark.parametrize("bits", [32, 64])
@pytest.mark.parametrize("lo,width", [(1000.25, 0.5), (-3.5, 7.0), (123456.789, 1e-3), (-1e-4, 3e-4), (7.0, 1.0),
                                      (0.1, 2.0 / 3.0)])
def test_keys_fp64_offsets_and_cell_boundaries(cs, O, bits, lo, width):
    """FP64 quantisation int(floor(x * m) - xmin * m) with boxes whose xmin * m has integer, near-integer and
    arbitrary fractions and large or negative offsets; points on the cell boundaries (x = (floor(xmin m) + j) / m),
    just beside them, and outside the box, against the oracle"""
    rng = np.random.default_rng(int(abs(lo) * 1000) % 1000 + bits)
    L = 10 if bits == 32 else 21
    m = float(1 << L) * (1.0 / width)
    o = lo * m
    j = rng.integers(-3, (1 << L) + 4, 30000)
    on = (np.floor(o) + j) / m
    pts = np.concatenate([on, np.nextafter(on, np.inf), np.nextafter(on, -np.inf),
                          lo + width * rng.random(30000), lo + width * (3 * rng.random(3000) - 1)])
    x = pts
    y = rng.permutation(pts)
    z = rng.permutation(pts)
    box = ((lo, lo, lo), (lo + width, lo + width, lo + width))
    for kind in (0, 1):
        ref = O.sfc_keys(x, y, z, O.make_box(*box), kind, bits)
        tx, ty, tz = to_dev(x, y, z)
        k = cs.sfc_keys(tx, ty, tz, cs.make_box(*box), kind, bits)
        torch.cuda.synchronize()
        assert np.array_equal(keys_u(k), ref), kind


@pytest.mark.parametrize("bits", [32, 64])
def test_keys_respect_remove_key(cs, O, bits):
    n = 5000
    x, y, z = uniform(O, 3, n, -1.0, 1.0)
    rm = 1 << (30 if bits == 32 else 63)
    init = np.zeros(n, np.uint64)
    init[::7] = rm
    ref = O.sfc_keys(x, y, z, O.make_box(-1, 1), 1, bits, keys=init, respect_remove_key=True)
    keys = torch.from_numpy(init.astype(np.int64 if bits == 64 else np.uint32).view(
        np.int64 if bits == 64 else np.int32)).to(dev())
    tx, ty, tz = to_dev(x, y, z)
    cs.sfc_keys(tx, ty, tz, cs.make_box(-1, 1), 1, bits, keys=keys, respect_remove_key=True)
    torch.cuda.synchronize()
    assert np.array_equal(keys_u(keys), ref)


@pytest.mark.parametrize("bits", [32, 64])
@pytest.mark.parametrize("n", [0, 1, 2, 31, 4095, 4096, 4097, 65536 + 17, 1000003])
def test_sort_random(cs, O, bits, n):
    rng = np.random.default_rng(n + bits)
    top = 1 << (30 if bits == 32 else 63)
    keys = rng.integers(0, top, size=n, dtype=np.uint64)
    if n > 10:
        keys[rng.integers(0, n, size=n // 3)] = keys[rng.integers(0, n, size=n // 3)]  # many duplicates
    rk, rp = O.sort_by_key(keys)
    tk = torch.from_numpy(keys.astype(np.int64) if bits == 64 else keys.astype(np.int32)).to(dev())
    sk, perm = cs.sort_pairs(tk)
    torch.cuda.synchronize()
    assert np.array_equal(keys_u(sk), rk)
    assert np.array_equal(u32(perm), rp)


@pytest.mark.parametrize("case", ["all_equal", "sorted", "reversed", "two_values", "low_entropy"])
def test_sort_patterns(cs, O, case):
    n = 300001
    rng = np.random.default_rng(5)
    if case == "all_equal":
        keys = np.full(n, 12345, np.uint64)
    elif case == "sorted":
        keys = np.sort(rng.integers(0, 1 << 63, size=n, dtype=np.uint64))
    elif case == "reversed":
        keys = np.sort(rng.integers(0, 1 << 63, size=n, dtype=np.uint64))[::-1].copy()
    elif case == "two_values":
        keys = np.where(rng.random(n) < 0.5, np.uint64(7), np.uint64(1 << 62))
    else:
        keys = (rng.integers(0, 4, size=n, dtype=np.uint64) << np.uint64(40)) | np.uint64(3)
    rk, rp = O.sort_by_key(keys)
    sk, perm = cs.sort_pairs(torch.from_numpy(keys.view(np.int64)).to(dev()))
    torch.cuda.synchronize()
    assert np.array_equal(keys_u(sk), rk)
    assert np.array_equal(u32(perm), rp)


def test_sort_bit_range_and_values(cs, O):
    n = 200000
    rng = np.random.default_rng(9)
    keys = rng.integers(0, 1 << 63, size=n, dtype=np.uint64)
    vals = rng.integers(0, 1 << 32, size=n, dtype=np.uint64).astype(np.uint32)
    # only bits [8, 40) take part: the reference of that is a stable sort on the masked key
    masked = (keys >> np.uint64(8)) & np.uint64((1 << 32) - 1)
    order = np.argsort(masked, kind="stable")
    tk = torch.from_numpy(keys.view(np.int64)).to(dev())
    tv = torch.from_numpy(vals.view(np.int32)).to(dev())
    sk, sv = cs.sort_pairs(tk, tv, begin_bit=8, end_bit=40, iota=False)
    torch.cuda.synchronize()
    assert np.array_equal(keys_u(sk), keys[order])
    assert np.array_equal(u32(sv), vals[order])


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_gather(cs, dtype):
    n = 123457
    rng = np.random.default_rng(2)
    perm = rng.permutation(n).astype(np.uint32)
    arrs = [rng.random(n).astype(dtype) for _ in range(4)]
    tp = torch.from_numpy(perm.view(np.int32)).to(dev())
    ta = to_dev(*arrs)
    outs = cs.gather4(tp, *ta)
    one = cs.gather(tp, ta[0])
    torch.cuda.synchronize()
    for o, a in zip(outs, arrs):
        assert np.array_equal(o.cpu().numpy(), a[perm])
    assert np.array_equal(one.cpu().numpy(), arrs[0][perm])
