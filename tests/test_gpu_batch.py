"""GPU parity of the batched path (cs_batch_*): many independent sets of uneven size, uniform and Plummer, mixed
bucket sizes, in one run; every set's permutation, leaves, counts and neighbour lists equal the oracle's single-set
pipeline (and the GPU single-set pipeline) on the same set."""
import numpy as np
import pytest
import torch

from gpu_util import neighbor_lists_equal, to_dev, u32

pytestmark = pytest.mark.gpu


def make_sets(O, S, seed, lo_exp=10, hi_exp=14, dtype=np.float32, k=60):
    """S sets, sizes log-uniform in [2^lo_exp, 2^hi_exp], uniform-in-cube or Plummer (50/50), per-set constant h for
    about k neighbours, bucket sizes from {16, 32, 64}"""
    rng = np.random.default_rng(seed)
    sets = []
    for s in range(S):
        n = int(2 ** (lo_exp + (hi_exp - lo_exp) * rng.random()))
        if s % 2 == 0:
            x, y, z = (O.philox_uniform(seed * 1000 + s, a, n, 0.0, 1.0) for a in range(3))
            lo, hi = (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)
        else:
            x, y, z = (a.astype(dtype) for a in O.plummer(seed * 1000 + s, n))
            lo, hi = (float(x.min()), float(y.min()), float(z.min())), (float(x.max()), float(y.max()), float(z.max()))
        x, y, z = (a.astype(dtype) for a in (x, y, z))
        vol = float(np.prod(np.array(hi) - np.array(lo)))
        h = np.full(n, 0.5 * (3 * k / (4 * np.pi * n / vol)) ** (1 / 3), dtype)
        if s % 2:
            h[:] = 0.5 * np.median(np.sqrt(x.astype(np.float64) ** 2 + y ** 2 + z ** 2)) * (k / n) ** (1 / 3)
        sets.append(dict(x=x, y=y, z=z, h=h, lo=lo, hi=hi, bucket=int(rng.choice([16, 32, 64]))))
    return sets


def run_batch(cs, sets, coord_bits, kind, ngmax):
    offsets = np.concatenate([[0], np.cumsum([s["x"].size for s in sets])])
    x, y, z, h = (np.concatenate([s[c] for s in sets]) for c in "xyzh")
    tx, ty, tz, th = to_dev(x, y, z, h)
    b = cs.Batch(coord_bits, kind, ngmax)
    b.run(tx, ty, tz, th, offsets, [cs.make_box(s["lo"], s["hi"]) for s in sets], [s["bucket"] for s in sets])
    out = b.outputs()
    torch.cuda.synchronize()
    return b, out, offsets


def check_set(O, out, offsets, j, st, kind, ngmax):
    obox = O.make_box(st["lo"], st["hi"])
    ref = O.pipeline(st["x"], st["y"], st["z"], st["h"], obox, st["bucket"], ngmax, kind, 32)
    a, e = int(offsets[j]), int(offsets[j + 1])
    assert np.array_equal(u32(out["order"][a:e]) - a, ref["perm"]), j
    lb = out["set_leaf_begin"].cpu().numpy()
    leaves = out["leaves"][lb[j]: lb[j + 1] + 1].cpu().numpy().view(np.uint64) - (np.uint64(j) << np.uint64(30))
    assert np.array_equal(leaves, ref["leaves"]), j
    assert np.array_equal(u32(out["counts"][lb[j]: lb[j + 1]]), ref["counts"]), j
    nc = u32(out["neighbor_counts"][a:e])
    nb = u32(out["neighbors"][a:e]).astype(np.int64) - a
    neighbor_lists_equal(nb.astype(np.uint32), nc, ref["nb"], ref["nc"], ngmax)


@pytest.mark.parametrize("coord_bits,kind", [(32, 0), (64, 1)])
def test_batch_equals_single_sets(cs, O, coord_bits, kind):
    S, ngmax = 24, 100
    sets = make_sets(O, S, 7 + coord_bits, dtype=np.float32 if coord_bits == 32 else np.float64)
    b, out, offsets = run_batch(cs, sets, coord_bits, kind, ngmax)
    assert b.result.num_sets == S and b.result.num_particles == offsets[-1]
    for j, st in enumerate(sets):
        check_set(O, out, offsets, j, st, kind, ngmax)


def test_batch_equals_gpu_pipeline_and_handles_tiny_and_empty_sets(cs, O):
    """sets of 0, 1, 7 and a few thousand particles, and the same sets through the single-set GPU pipeline"""
    rng = np.random.default_rng(3)
    sets = []
    for n in (0, 1, 7, 3000, 0, 5000, 64, 65):
        x, y, z = (rng.random(n).astype(np.float32) for _ in range(3))
        sets.append(dict(x=x, y=y, z=z, h=np.full(n, 0.05, np.float32), lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0),
                         bucket=16))
    ngmax = 64
    b, out, offsets = run_batch(cs, sets, 32, cs.MORTON, ngmax)
    for j, st in enumerate(sets):
        n = st["x"].size
        if n == 0:
            continue
        check_set(O, out, offsets, j, st, 0, ngmax)
        pipe = cs.Pipeline(32, 32, cs.MORTON, 16, ngmax, 1.0, 1.0, False, True)
        tx, ty, tz, th = to_dev(st["x"], st["y"], st["z"], st["h"])
        pipe.run(tx, ty, tz, th, cs.make_box(st["lo"], st["hi"]))
        po = pipe.outputs()
        torch.cuda.synchronize()
        a = int(offsets[j])
        assert torch.equal(po["neighbor_counts"].cpu(), out["neighbor_counts"][a:a + n].cpu()), j
