"""GPU: the tunings change the speed, never the results. Every candidate of the autotuner (targets per warp 32 / 16 /
8, by-target switch cost 0 / 5 / 7 / 10, sort tiles of 16 or 12 keys per thread) gives sorted keys, neighbour counts
and lists identical to the default, which equal the oracle's; the autotuner keeps one of its candidates; invalid
tunings are refused; the batched path with another tuning gives the same results."""
import numpy as np
import pytest
import torch

from gpu_util import keys_u, neighbor_lists_equal, to_dev, u32

pytestmark = pytest.mark.gpu

CANDIDATES = [(32, 7), (32, 0), (32, 5), (32, 10), (16, 7), (8, 7)]
SORT_ITEMS = [16, 12]


def _inputs(O, case):
    if case == "plummer64":
        n = 40000
        x, y, z = O.plummer(29, n)
        lo, hi = (x.min(), y.min(), z.min()), (x.max(), y.max(), z.max())
        h = 0.5 * (60.0 / n) ** (1 / 3) * np.sqrt(1.0 + x * x + y * y + z * z)
        return (x, y, z, h), lo, hi, 64, 1, 64, 32
    n = 50000
    x, y, z = (O.philox_uniform(31, a, n, 0.0, 1.0).astype(np.float32) for a in range(3))
    h = np.full(n, 0.5 * (3 * 60 / (4 * np.pi * n)) ** (1 / 3), np.float32)
    return (x, y, z, h), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), 32, 0, 32, 16


def _run(cs, pipe, t, box):
    pipe.run(*t, box)
    out = pipe.outputs()
    torch.cuda.synchronize()
    return u32(out["neighbor_counts"]).copy(), u32(out["neighbors"]).copy()


@pytest.mark.parametrize("case", ["plummer64", "uniform32"])
def test_every_tuning_gives_the_same_neighbours(cs, O, case):
    (x, y, z, h), lo, hi, cbits, kind, kbits, bucket = _inputs(O, case)
    ngmax = 120
    box = cs.make_box(lo, hi)
    t = to_dev(x, y, z, h)
    pipe = cs.Pipeline(cbits, kbits, kind, bucket, ngmax, 1.0, 1.0, False, True)
    nc0, nb0 = _run(cs, pipe, t, box)
    ref = O.pipeline(x, y, z, h, O.make_box(lo, hi), bucket, ngmax, kind, kbits)
    neighbor_lists_equal(nb0.reshape(-1, ngmax), nc0, ref["nb"], ref["nc"], ngmax)
    for g, c in CANDIDATES:
        pipe.set_tuning(g, c)
        assert pipe.get_tuning() == {"nb_group": g, "nb_by_target_cost": c, "sort_items": 16}
        nc, nb = _run(cs, pipe, t, box)
        assert np.array_equal(nc, nc0), (g, c)
        neighbor_lists_equal(nb.reshape(-1, ngmax), nc, nb0.reshape(-1, ngmax), nc0, ngmax)
    pipe.set_tuning(32, 7, 12)
    nc, nb = _run(cs, pipe, t, box)
    out = pipe.outputs()
    assert np.array_equal(keys_u(out["sorted_keys"]), np.asarray(ref["sorted_keys"], np.uint64))
    assert np.array_equal(u32(out["order"]), ref["perm"])
    assert np.array_equal(nc, nc0)
    neighbor_lists_equal(nb.reshape(-1, ngmax), nc, nb0.reshape(-1, ngmax), nc0, ngmax)


def test_autotune_keeps_a_candidate_and_the_results(cs, O):
    (x, y, z, h), lo, hi, cbits, kind, kbits, bucket = _inputs(O, "plummer64")
    ngmax = 120
    box = cs.make_box(lo, hi)
    t = to_dev(x, y, z, h)
    pipe = cs.Pipeline(cbits, kbits, kind, bucket, ngmax, 1.0, 1.0, False, True)
    nc0, nb0 = _run(cs, pipe, t, box)
    r = pipe.autotune(2)
    tried = [(c["nb_group"], c["nb_by_target_cost"]) for c, _ in r["tried"]]
    nbt = len(CANDIDATES)
    # the traversal candidates with the default sort shape, then the sort shapes with the fastest traversal
    assert tried[:nbt] == CANDIDATES and all(ms > 0 for _, ms in r["tried"])
    assert [c["sort_items"] for c, _ in r["tried"][:nbt]] == [16] * nbt
    assert [c["sort_items"] for c, _ in r["tried"][nbt:]] == SORT_ITEMS
    assert r["best"] in [c for c, _ in r["tried"]] and pipe.get_tuning() == r["best"]
    fastest_nb = min(r["tried"][:nbt], key=lambda cm: cm[1])[0]
    assert (r["best"]["nb_group"], r["best"]["nb_by_target_cost"]) == (fastest_nb["nb_group"],
                                                                      fastest_nb["nb_by_target_cost"])
    assert r["best"]["sort_items"] == min(r["tried"][nbt:], key=lambda cm: cm[1])[0]["sort_items"]
    out = pipe.outputs()
    torch.cuda.synchronize()
    assert np.array_equal(u32(out["neighbor_counts"]), nc0)
    nc, nb = _run(cs, pipe, t, box)
    assert np.array_equal(nc, nc0)
    neighbor_lists_equal(nb.reshape(-1, ngmax), nc, nb0.reshape(-1, ngmax), nc0, ngmax)


def test_invalid_tunings_are_refused(cs):
    pipe = cs.Pipeline(64, 64, cs.HILBERT, 64, 100, 1.0, 1.0, False, True)
    for g, c, s in [(4, 7, 16), (64, 7, 16), (32, -1, 16), (32, 65, 16), (32, 7, 8), (32, 7, 24)]:
        with pytest.raises(cs.CsError):
            pipe.set_tuning(g, c, s)
    assert pipe.get_tuning() == {"nb_group": 32, "nb_by_target_cost": 7, "sort_items": 16}
    with pytest.raises(cs.CsError):
        pipe.autotune(1)  # no previous run


def test_batch_with_another_tuning_gives_the_same_results(cs, O):
    rng = np.random.default_rng(41)
    sets = [rng.random((3, n)).astype(np.float32) for n in (3000, 700, 5000, 64)]
    offsets = np.concatenate([[0], np.cumsum([s.shape[1] for s in sets])])
    x, y, z = (np.concatenate([s[k] for s in sets]) for k in range(3))
    h = np.full(x.size, 0.04, np.float32)
    tx, ty, tz, th = to_dev(x, y, z, h)
    boxes = [cs.make_box(0.0, 1.0) for _ in sets]
    outs = []
    for tuning in [(32, 7, 16), (16, 7, 16), (32, 0, 12)]:
        b = cs.Batch(32, cs.MORTON, 64)
        b.set_tuning(*tuning)
        b.run(tx, ty, tz, th, offsets, boxes, [16] * len(sets))
        o = b.outputs()
        torch.cuda.synchronize()
        outs.append((u32(o["neighbor_counts"]).copy(), u32(o["neighbors"]).copy()))
    for nc, nb in outs[1:]:
        assert np.array_equal(nc, outs[0][0])
        neighbor_lists_equal(nb.reshape(-1, 64), nc, outs[0][1].reshape(-1, 64), outs[0][0], 64)
