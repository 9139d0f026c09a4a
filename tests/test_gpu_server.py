"""GPU tests of the request server (cs_server_*): every request's result (leaf count, neighbour counts, checksum of
the neighbour lists) is the same alone and in a mix of concurrent requests, builds agree with the single-set
pipeline, resident trees take incremental updates, and admission follows the memory budget."""
import numpy as np
import pytest
import torch

from gpu_util import to_dev

pytestmark = pytest.mark.gpu

GB = 1 << 30


def make_requests(O, count, seed):
    """one-off builds of uniform and Plummer sets (2^12 .. 2^16 particles), and a resident tree 7 built, updated
    twice (small displacements) and rebuilt"""
    rng = np.random.default_rng(seed)
    reqs = []
    for j in range(count):
        n = int(2 ** (12 + 4 * rng.random()))
        if j % 2:
            x, y, z = (O.philox_uniform(seed * 100 + j, a, n, -1.0, 1.0) for a in range(3))
            lo, hi = (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0)
            h = np.full(n, 0.5 * (3 * 100 / (4 * np.pi * n / 8.0)) ** (1 / 3))
        else:
            x, y, z = O.plummer(seed * 100 + j, n)
            lo, hi = (x.min(), y.min(), z.min()), (x.max(), y.max(), z.max())
            h = np.full(n, 0.5 * (100 / n) ** (1 / 3))
        reqs.append(dict(x=x, y=y, z=z, h=h, lo=lo, hi=hi, kind=0, tree=-1))
    n = 20000
    x, y, z = (O.philox_uniform(seed + 5, a, n, 0.0, 1.0) for a in range(3))
    h = np.full(n, 0.6 * n ** (-1 / 3))
    sp = n ** (-1 / 3)
    for step in range(4):
        kind = 0 if step in (0, 3) else 1
        if step:
            x, y, z = (np.clip(a + rng.normal(0, 0.05 * sp, n), 0.0, 1.0 - 1e-12) for a in (x, y, z))
        reqs.insert(2 * step + 1, dict(x=x, y=y, z=z, h=h, lo=(0.0,) * 3, hi=(1.0,) * 3, kind=kind, tree=7))
    return reqs


def submit_all(cs, srv, reqs, serial):
    out = []
    ids = []
    for r in reqs:
        rid = srv.submit(r["x"], r["y"], r["z"], r["h"], cs.make_box(r["lo"], r["hi"]), r["kind"], r["tree"])
        if serial:
            out.append(srv.wait(rid))
        else:
            ids.append(rid)
    for rid in ids:
        out.append(srv.wait(rid))
    return out


def test_results_same_alone_and_in_a_mix(cs, O):
    reqs = make_requests(O, 12, 3)
    alone = cs.Server(1, 64 * GB)
    solo = submit_all(cs, alone, reqs, serial=True)
    alone.close()
    mixed = cs.Server(4, 64 * GB)
    mix = submit_all(cs, mixed, reqs, serial=False)
    st = mixed.stats()
    mixed.close()
    assert st.completed == len(reqs) and st.failed == 0 and st.p99_ms >= st.p50_ms > 0
    for j, ((ra, ca), (rb, cb)) in enumerate(zip(solo, mix)):
        assert ra.status == 0 and rb.status == 0, j
        assert ra.num_leaves == rb.num_leaves and ra.neighbor_checksum == rb.neighbor_checksum, j
        assert np.array_equal(ca, cb), j


def test_builds_agree_with_the_pipeline_and_updates_with_steps(cs, O):
    reqs = make_requests(O, 4, 9)
    srv = cs.Server(2, 64 * GB)
    res = submit_all(cs, srv, reqs, serial=False)
    srv.close()
    tree_pipe = cs.Pipeline(64, 64, cs.HILBERT, 64, 200, 1.0, 1.0, False, True)
    for r, (rr, nc) in zip(reqs, res):
        box = cs.make_box(r["lo"], r["hi"])
        tx, ty, tz, th = to_dev(r["x"], r["y"], r["z"], r["h"])
        if r["tree"] < 0:
            pipe = cs.Pipeline(64, 64, cs.HILBERT, 64, 200, 1.0, 1.0, False, True)
            pipe.run(tx, ty, tz, th, box)
            out = pipe.outputs()
        else:
            if r["kind"] == 0:
                tree_pipe.reset_steps()
            tree_pipe.step(tx, ty, tz, th, box, False)
            out = tree_pipe.outputs()
        torch.cuda.synchronize()
        assert np.array_equal(out["neighbor_counts"].cpu().numpy().view(np.uint32), nc)


def test_admission_budget_and_invalid_updates(cs, O):
    n = 1 << 15
    x, y, z = (O.philox_uniform(21, a, n, 0.0, 1.0) for a in range(3))
    h = np.full(n, 0.04)
    box = cs.make_box(0.0, 1.0)
    tiny = cs.Server(2, 1 << 20)  # 1 MiB: no request fits
    rid = tiny.submit(x, y, z, h, box)
    with pytest.raises(cs.CsError) as e:
        tiny.wait(rid)
    assert e.value.code == 2
    rid = tiny.submit(x, y, z, h, box, cs.REQ_UPDATE, 3)  # no resident tree 3
    with pytest.raises(cs.CsError) as e:
        tiny.wait(rid)
    assert e.value.code == 1
    tiny.close()
    # 30 resident trees of about 30 MB each do not fit in 512 MiB: the least recently used idle trees are released
    srv = cs.Server(1, GB // 2)
    for t in range(30):
        srv.wait(srv.submit(x, y, z, h, box, cs.REQ_BUILD, t))
    st = srv.stats()
    assert 0 < st.resident_trees < 30 and st.failed == 0 and st.device_bytes <= GB // 2
    r, nc = srv.wait(srv.submit(x, y, z, h, box, cs.REQ_UPDATE, 29))  # the most recent tree is still there
    assert r.status == 0
    srv.close()
