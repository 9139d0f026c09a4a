"""Benchmark: keys -> neighbours throughput (Mparticles/s) of the whole octree path on N Plummer particles.

Workload (default): 16M FP64 particles from a Plummer sphere (scale radius 1, truncated at r = 100, seeded, centre of
mass at the origin), tight bounding box, 64-bit Hilbert keys, bucketSize 64, findHalos for the leaves in the first
quarter of the key space [0, 2^61), findNeighbors with ngmax 200, per-particle h such that exactly 100 neighbours lie
within 2h (set once before timing by bisection on neighbour counts). One step = one full pass of the path over the
particles: keys, stable sort, gather of x/y/z/h, computeOctree from the root, internal-tree link, node geometry,
search boxes + halo flags, neighbour search.

Reports (one JSON line on rank 0):
  value     device throughput, inputs resident in HBM (particles of all ranks / max-over-ranks step time)
  e2e       the same through the host-buffer C-ABI call (pipelined: step k + 1's copies overlap step k; the
            synchronous call's time beside it): pinned host inputs copied in, neighbour counts and halo
            flags copied back every step
  roofline  for the dominant kernel (neighbour search): algorithmic bytes per launch / its event-timed duration
  cpu_baseline  the CPU oracle of the same path on the host cores, on a bounded sample of the workload

--impl reference times the reference's CPU implementation of the path (the oracle port; the reference's own build
cannot run on the GPU host) on the same workload family, one bounded sample per step.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "cornerstone-octree_gb300"))

METRIC = "Mparticles/s keys->neighbors (16M Plummer)"
UNIT = "Mparticles/s"
NGMAX = 200
BUCKET = 64
K_NEIGHBORS = 100
FOCUS = (0, 1 << 61)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=30)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--n", "--particles", dest="n", type=int, default=None,
                   help="particles (default 16M plummer, 64M incremental)")
    p.add_argument("--sets", type=int, default=4096, help="sets of the batched workload")
    p.add_argument("--requests", type=int, default=600, help="requests of the served workload")
    p.add_argument("--rate", type=float, default=2000.0, help="Poisson arrival rate (requests/s), served workload")
    p.add_argument("--workload", default="plummer",
                   choices=["plummer", "incremental", "batched", "served", "sort", "ijloop"],
                   help="plummer: the 16M keys->neighbours pass (default); incremental: 64M FP32 time steps with one "
                        "updateOctree step each, replayed from CUDA graphs; batched: 4096 uneven FP32 sets in "
                        "one batched run per chunk against a per-set loop of the single-set pipeline; served: a "
                        "Poisson stream of build and update requests through the request server; sort: the stable "
                        "key sort of the 16M Plummer workload's Hilbert keys alone, with its HBM fraction; ijloop: "
                        "the neighbour-list consumers on the 16M Plummer particles (cluster-pair lists built and an "
                        "SPH density summed over them, and the same sum over the stored neighbour lists)")
    p.add_argument("--seed", type=int, default=2024)
    p.add_argument("--ijloop-dist", default="plummer", choices=["plummer", "uniform"],
                   help="particles of the ijloop workload: the Plummer sphere (the benchmark), or uniform in the unit "
                        "cube (small profiling cases: the Plummer sphere's sparse outskirts need long cluster lists "
                        "at small n)")
    p.add_argument("--cpu-sample", type=int, default=1 << 20, help="particles of the CPU baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-autotune", action="store_true",
                   help="keep the default traversal tuning instead of autotuning it during the warm-up")
    return p.parse_args()


def dist_setup():
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while the timed region runs"""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_hbm_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profile_figures(n):
    """per-launch DRAM bytes and warp instructions of the neighbour search, from the committed ncu summary of a
    smaller capture of the same workload, scaled to n particles by particle count (None where absent)"""
    path = os.path.join(ROOT, "profiles", "neighbors_plummer.md")
    fig = {}
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_particle:"):
                    fig["traffic"] = float(line.split(":")[1]) * n
                elif line.startswith("warp_instructions_per_particle:"):
                    fig["warp_instructions"] = float(line.split(":")[1]) * n
                elif line.startswith("capture_particles:"):
                    fig["source"] = (f"ncu capture of the {int(line.split(':')[1])}-particle case "
                                     f"(profiles/neighbors_plummer.md), scaled by particle count")
    except OSError:
        pass
    return fig


def density_profile_figures():
    """the cluster density loop's FP64 pipe activity from its committed ncu summary (None where absent)"""
    path = os.path.join(ROOT, "profiles", "ijloop_density_uniform4m.md")
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("fp64_pipe_active_fraction:"):
                    return {"fp64_pipe_active": float(line.split(":")[1]),
                            "source": "ncu capture of the 4194304-particle uniform case "
                                      "(profiles/ijloop_density_uniform4m.md)"}
    except OSError:
        pass
    return None


# ---------------------------------------------------------------------------------------------------------------
# CPU side (oracle): bounded sample of the workload
# ---------------------------------------------------------------------------------------------------------------

def cpu_sample(n_sample, seed, tol=0.1):
    """the workload's inputs for the CPU oracle: the same numpy generator as the GPU arm (cstone_synth, which loads no
    CUDA library), h by per-particle bisection with the oracle's own neighbour counts to within tol of k"""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    import cstone_synth as S

    x, y, z = S.plummer(n_sample, seed)
    lo, hi = S.tight_box(x, y, z)
    box = O.make_box(lo, hi)
    h = O.h_for_k_neighbors_cpu(x, y, z, box, K_NEIGHBORS, tol=tol)
    return O, x, y, z, h, box


def host_cpu():
    """model and logical CPU count of the host (lscpu), for the CPU baseline's record"""
    info = {"model": None, "cpus": os.cpu_count()}
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            k, _, v = line.partition(":")
            if k.strip() == "Model name" and info["model"] is None:
                info["model"] = v.strip()
            elif k.strip() == "CPU(s)":
                info["cpus"] = int(v.strip())
    except (OSError, ValueError, subprocess.SubprocessError):
        pass
    return info


def cpu_time(O, x, y, z, h, box):
    t, _ = O.timed_pipeline(x, y, z, h, box, BUCKET, NGMAX, FOCUS)
    return t


def run_reference(args, world, rank):
    """The reference's CPU path (the oracle port, OpenMP on all host cores, serial stable sort as std::stable_sort)
    on the GPU arm's workload: the same 16M Plummer particles (same generator and seed), tight box, Hilbert64, bucket
    64, focus [0, 2^61), ngmax 200; h such that each particle has 100 +- 2 neighbours within 2h, prepared once with
    the oracle (not timed). Loads only oracle/ libraries, never the CUDA library."""
    if rank != 0:
        return
    n = args.n or 16 * 1024 * 1024
    t0 = time.perf_counter()
    O, x, y, z, h, box = cpu_sample(n, args.seed, tol=0.02)
    prep_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        cpu_time(O, x, y, z, h, box)
    t0 = time.perf_counter()
    stages = []
    for _ in range(args.steps):
        stages.append(cpu_time(O, x, y, z, h, box))
    dt = (time.perf_counter() - t0) / args.steps
    value = n / dt / 1e6
    cores = O.num_threads()
    sample = (f"the whole workload every step: {n} particles of the Plummer sphere (seed {args.seed}), h for "
              f"{K_NEIGHBORS} +- 2 neighbours prepared by the oracle in {prep_s:.0f} s")
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "plummer-keys-to-neighbors", "n_particles_per_gpu": n, "ngmax": NGMAX,
                       "bucket_size": BUCKET, "keys": "hilbert64", "focus": "[0, 2^61)",
                       "neighbours_target": K_NEIGHBORS, "l2": "inputs (512 MB) larger than L2",
                       "parallelism": "replicas x1"},
            "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": sample, "host_cpu": host_cpu()},
            "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "stage_seconds": {k: round(statistics.mean(s[k] for s in stages), 4) for k in stages[0]}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------------------------------------------

def run_incremental(args, world, rank, local):
    """64M FP32 particles uniform in [0,1]^3, periodic; every step displaces each particle by N(0, 0.1 * spacing)
    (periodic wrap) and runs one incremental pipeline step: Morton64 keys, sort, one updateOctree step from the
    previous tree (bucket 32), link, geometry, neighbours (h = 1.2 * spacing, ngmax 150). The first step builds from
    the root; the warm-up steps capture the two graphs of the leaf ping-pong."""
    import torch

    import cstone_gb300 as cs

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n = args.n or 64 * 1024 * 1024
    spacing = n ** (-1.0 / 3)
    g = torch.Generator(device=dev).manual_seed(args.seed + rank)
    x, y, z = (torch.rand(n, generator=g, device=dev, dtype=torch.float32) for _ in range(3))
    h = torch.full((n,), 1.2 * spacing, device=dev, dtype=torch.float32)
    box = cs.make_box(0.0, 1.0, cs.PERIODIC)

    def displace():
        for a in (x, y, z):
            a.add_(torch.randn(n, generator=g, device=dev, dtype=torch.float32), alpha=0.1 * spacing)
            a.sub_(torch.floor(a))  # periodic wrap into [0, 1)

    def timed(pipe, use_graph, steps):
        wall, dev_ms, stage_acc = 0.0, 0.0, None
        for _ in range(steps):
            displace()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            pipe.step(x, y, z, h, box, use_graph)
            wall += time.perf_counter() - t0
            st = pipe.stage_times()
            dev_ms += sum(st.values())
            stage_acc = st if stage_acc is None else {k: stage_acc[k] + st[k] for k in st}
        return wall * 1e3 / steps, dev_ms / steps, {k: round(v / steps, 4) for k, v in stage_acc.items()}

    pipe = cs.Pipeline(32, 64, cs.MORTON, 32, 150, 1.0, 1.0, False, True)
    pipe.step(x, y, z, h, box, True)  # root build
    for _ in range(max(3, args.warmup)):
        displace()
        pipe.step(x, y, z, h, box, True)
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        barrier(world)
        g_wall, g_dev, g_st = timed(pipe, True, args.steps)
        barrier(world)
    replays = pipe.graph_replays()
    res = pipe.result
    nc = pipe.outputs()["neighbor_counts"]
    mean_nc = float(nc.double().mean())
    del nc, pipe  # release the first pipeline's buffers (about 45 GB at 64M) before the second one
    torch.cuda.synchronize()
    # the same steps without graphs, for comparison
    plain = cs.Pipeline(32, 64, cs.MORTON, 32, 150, 1.0, 1.0, False, True)
    plain.step(x, y, z, h, box, False)
    for _ in range(max(3, args.warmup)):
        displace()
        plain.step(x, y, z, h, box, False)
    p_wall, p_dev, _ = timed(plain, False, args.steps)
    ms = max_over_ranks(g_wall, world)
    if rank == 0:
        line = {"metric": "Mparticles/s incremental step (64M FP32 uniform periodic, Morton64, CUDA graph)",
                "value": round(world * n / (ms * 1e-3) / 1e6, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": max(3, args.warmup), "ms_per_step": round(ms, 3), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": "incremental-steps", "n_particles_per_gpu": n, "bucket_size": 32,
                           "ngmax": 150, "keys": "morton64", "box": "periodic [0,1]^3", "sigma": "0.1 spacing",
                           "h": "1.2 spacing", "l2": f"inputs ({12 * n >> 20} MB) larger than L2",
                           "parallelism": f"replicas x{world}"},
                "device_ms_per_step": round(g_dev, 3), "graph_replays": replays,
                "ungraphed": {"ms_per_step": round(p_wall, 3), "device_ms_per_step": round(p_dev, 3)},
                "stages_ms": g_st, "clocks": clocks.summary(),
                "tree": {"leaves": res.num_leaves, "nodes": res.num_nodes, "max_depth": res.max_depth},
                "mean_neighbors": round(mean_nc, 2)}
        print(json.dumps(line), flush=True)


def run_batched(args, world, rank, local):
    """4096 independent FP32 sets, sizes log-uniform in [2^10, 2^20], uniform or Plummer (50/50), Morton32 keys,
    bucket sizes from {16, 32, 64}, per-set constant h for about 60 neighbours, ngmax 100: the batched path (one run
    per chunk of at most 64M particles, bounded by the neighbour lists' memory) against a per-set loop of the
    single-set pipeline on the same device-resident sets. Reports sets/s of both and whether every set's neighbour
    counts agree."""
    import numpy as np
    import torch

    import cstone_gb300 as cs
    from cstone_gb300 import workloads as W

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    ngmax = 100
    sets = W.batched_sets(args.sets, args.seed + rank, dev)
    total = sum(st["n"] for st in sets)
    chunk_cap = 64 * 1024 * 1024
    packed = [(offs, xyzh, [cs.make_box(sets[s]["lo"], sets[s]["hi"]) for s in ch], [sets[s]["bucket"] for s in ch])
              for ch, offs, xyzh in W.chunk_sets(sets, chunk_cap)]
    chunks = packed
    del sets
    torch.cuda.synchronize()

    batch = cs.Batch(32, cs.MORTON, ngmax)

    def batched_pass():
        for offs, (x, y, z, h), boxes, buckets in packed:
            batch.run(x, y, z, h, offs, boxes, buckets)

    pipes = {b: cs.Pipeline(32, 32, cs.MORTON, b, ngmax, 1.0, 1.0, False, True) for b in (16, 32, 64)}

    def per_set_pass(check=False):
        """the per-set loop; with check, every set's neighbour counts and stored lists against the batched run's
        (batched lists hold chunk-global indices: shifted by the set's offset)"""
        bad = 0
        for ci, (offs, (x, y, z, h), boxes, buckets) in enumerate(packed):
            if check:
                batch.run(x, y, z, h, offs, boxes, buckets)
                bo = batch.outputs()
                bnc, bnb = bo["neighbor_counts"], bo["neighbors"]
            for j in range(len(buckets)):
                a, e = int(offs[j]), int(offs[j + 1])
                if e == a:
                    continue
                pipe = pipes[buckets[j]]
                pipe.run(x[a:e], y[a:e], z[a:e], h[a:e], boxes[j])
                if check:
                    po = pipe.outputs()
                    pnc, pnb = po["neighbor_counts"], po["neighbors"]
                    stored = torch.arange(ngmax, device=dev)[None, :] < pnc.clamp(max=ngmax)[:, None]
                    same = torch.equal(pnc, bnc[a:e]) and torch.equal(torch.where(stored, pnb, 0),
                                                                       torch.where(stored, bnb[a:e] - a, 0))
                    bad += int(not same)
        return bad

    steps = max(1, min(args.steps, 3))
    batched_pass()  # warm-up: buffers sized by the largest chunk
    per_set_pass()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(steps):
            batched_pass()
        torch.cuda.synchronize()
        tb = (time.perf_counter() - t0) / steps
        t0 = time.perf_counter()
        for _ in range(steps):
            per_set_pass()
        torch.cuda.synchronize()
        tp = (time.perf_counter() - t0) / steps
        barrier(world)
    mismatched = per_set_pass(check=True)
    tb = max_over_ranks(tb, world)
    if rank == 0:
        line = {"metric": "sets/s batched (4096 uneven FP32 sets, Morton32, build + neighbours)",
                "value": round(world * args.sets / tb, 3), "unit": "sets/s", "n_gpus": world, "steps": steps,
                "warmup": 1, "ms_per_step": round(tb * 1e3, 3), "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": "batched-sets", "sets": args.sets, "particles": total,
                           "sizes": "log-uniform [2^10, 2^20]", "mix": "uniform / Plummer 50/50",
                           "keys": "morton32", "buckets": "{16, 32, 64}", "ngmax": ngmax, "neighbours": "about 60",
                           "chunks": len(chunks), "chunk_particles_max": chunk_cap,
                           "parallelism": f"replicas x{world}"},
                "particles_per_s": round(total / tb / 1e6, 3),
                "per_set_loop": {"sets_per_s": round(args.sets / tp, 3), "ms_per_pass": round(tp * 1e3, 3),
                                 "particles_per_s_M": round(total / tp / 1e6, 3)},
                "identical_neighbor_lists": mismatched == 0, "mismatched_sets": mismatched,
                "check": "every set's neighbour counts and stored lists, batched run against the per-set loop",
                "clocks": clocks.summary()}
        print(json.dumps(line), flush=True)


def run_sort(args, world, rank, local):
    """The stable (key, index) sort of the 16M Plummer workload's 64-bit Hilbert keys (63 significant bits: a
    histogram pass and 8 onesweep passes of 8 bits), inputs resident; each timed sort starts from the unsorted keys
    (restored by a copy outside the timed events). Algorithmic bytes per sort: the histogram pass reads the keys (8 B
    per key) and every onesweep pass reads and writes key and index (24 B per key; the first pass reads no index)."""
    import torch

    import cstone_gb300 as cs
    from cstone_gb300 import workloads as W

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n = args.n or 16 * 1024 * 1024
    x, y, z = W.plummer(n, args.seed + rank)
    lo, hi = W.tight_box(x, y, z)
    box = cs.make_box(lo, hi)
    tx, ty, tz = (torch.from_numpy(a).to(dev) for a in (x, y, z))
    k0 = cs.sfc_keys(tx, ty, tz, box, cs.HILBERT, 64)
    keys = torch.empty_like(k0)
    ws = torch.empty(cs.lib.cs_sort_pairs_workspace_bytes(n, 64), dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()
    acc = 0.0
    with ClockSampler(local) as clocks:
        for it in range(args.warmup + args.steps):
            keys.copy_(k0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            kk, _ = cs.sort_pairs(keys, end_bit=63, workspace=ws)
            e1.record(stream)
            torch.cuda.synchronize()
            if it >= args.warmup:
                acc += e0.elapsed_time(e1)
    ms = max_over_ranks(acc / args.steps, world)
    ok = bool((kk[1:] >= kk[:-1]).all())
    sorted_ref = kk.clone()
    passes = 8
    algo = n * (8 + 20 + (passes - 1) * 24)
    peak, peak_kind = measured_hbm_peak()
    achieved = algo / (ms * 1e-3) / 1e9
    cub = cub_sort_leg(args, k0, sorted_ref, stream, dev, peak, world)
    if rank == 0:
        line = {"metric": "Mkeys/s stable sort (16M Hilbert64 keys of the Plummer workload)",
                "value": round(world * n / (ms * 1e-3) / 1e6, 3), "unit": "Mkeys/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
                "config": {"workload": "sort-hilbert64-keys", "n_keys": n, "bits": 63, "passes": passes,
                           "values": "indices (first pass: generated)", "parallelism": f"replicas x{world}"},
                "sorted": ok,
                "roofline": {"kernel": "histogram + onesweep passes", "bound": "hbm", "achieved": round(achieved, 1),
                             "peak": peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
                             "algorithmic_bytes": algo},
                "cub": cub,
                "clocks": clocks.summary()}
        print(json.dumps(line), flush=True)


def cub_sort_leg(args, k0, sorted_ref, stream, dev, peak, world):
    """CUB's DeviceRadixSort::SortPairs (the sort behind the reference's sortByKey) on the same keys with iota values,
    over bits [0, 63) like the library's sort and over [0, 64) as the reference calls it; event-timed like the
    library's sort, results checked equal to it"""
    import ctypes as C

    import torch

    path = os.path.join(ROOT, "cornerstone-octree_gb300", "baseline", "libcub_sort.so")
    if not os.path.exists(path):
        return {"unavailable": "baseline/libcub_sort.so not built"}
    cub = C.CDLL(path)
    cub.cub_sort_pairs_u64_temp_bytes.restype = C.c_size_t
    n = k0.numel()
    kin = torch.empty_like(k0)
    kout = torch.empty_like(k0)
    vin = torch.arange(n, dtype=torch.int32, device=dev)
    vout = torch.empty_like(vin)
    out = {"api": "cub::DeviceRadixSort::SortPairs (CUDA toolkit CUB), keys u64, values u32 iota"}
    for end_bit in (63, 64):
        tb = cub.cub_sort_pairs_u64_temp_bytes(C.c_size_t(n), 0, end_bit)
        tmp = torch.empty(tb, dtype=torch.uint8, device=dev)
        acc = 0.0
        for it in range(args.warmup + args.steps):
            kin.copy_(k0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            rc = cub.cub_sort_pairs_u64(C.c_void_p(stream.cuda_stream), C.c_void_p(kin.data_ptr()),
                                        C.c_void_p(kout.data_ptr()), C.c_void_p(vin.data_ptr()),
                                        C.c_void_p(vout.data_ptr()), C.c_size_t(n), 0, end_bit,
                                        C.c_void_p(tmp.data_ptr()), C.c_size_t(tb))
            e1.record(stream)
            torch.cuda.synchronize()
            if rc:
                return {"unavailable": f"CUB SortPairs returned {rc}"}
            if it >= args.warmup:
                acc += e0.elapsed_time(e1)
        ms = max_over_ranks(acc / args.steps, world)
        passes = (end_bit + 7) // 8
        algo = n * (8 + 20 + (passes - 1) * 24)
        out[f"bits_0_{end_bit}"] = {"ms": round(ms, 4), "Mkeys_per_s": round(n / (ms * 1e-3) / 1e6, 3),
                                    "hbm_frac": round(algo / (ms * 1e-3) / 1e9 / peak, 4),
                                    "same_result": bool(torch.equal(kout, sorted_ref))}
    return out


def run_ijloop(args, world, rank, local):
    """Neighbour-list consumers on the 16M FP64 Plummer workload (same particles, h for 100 neighbours, Hilbert64,
    bucket 64): per step the cluster-pair lists are built (8-particle clusters, octree walk) and an SPH density is
    summed over them (FP64, ascending j); beside it, the same density over the stored neighbour lists of the pipeline
    (ngmax 200). Algorithmic bytes of the cluster loop: x, y, z, h, m read and rho written per particle (48 B), plus
    the list entries read (4 B per listed j-cluster per i-cluster)."""
    import numpy as np
    import torch
    import types

    import cstone_gb300 as cs
    from cstone_gb300 import workloads as W

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n = args.n or 16 * 1024 * 1024
    if args.ijloop_dist == "plummer":
        x, y, z = W.plummer(n, args.seed + rank)
    else:
        x, y, z = W.uniform(n, 0.0, 1.0, args.seed + rank)
    lo, hi = W.tight_box(x, y, z)
    box = cs.make_box(lo, hi)
    tx, ty, tz = (torch.from_numpy(a).to(dev) for a in (x, y, z))
    th, _ = W.h_for_k_neighbors(tx, ty, tz, box, K_NEIGHBORS, BUCKET)
    pipe = cs.Pipeline(64, 64, cs.HILBERT, BUCKET, NGMAX, 1.0, 1.0, False, True)
    r = pipe.run(tx, ty, tz, th, box)
    out = pipe.outputs()
    tree = types.SimpleNamespace(num_leaves=r.num_leaves, num_nodes=r.num_nodes, child_offsets=out["child_offsets"],
                                 parents=out["parents"], internal_to_leaf=out["internal_to_leaf"])
    m = torch.rand(n, dtype=torch.float64, device=dev, generator=torch.Generator(device=dev).manual_seed(5)) + 0.5
    xs, ys, zs, hs = out["x"], out["y"], out["z"], out["h"]
    cen, siz = out["centers"].reshape(-1), out["sizes"].reshape(-1)
    stream = torch.cuda.current_stream()
    lists, counts = cs.cluster_nblist(xs, ys, zs, hs, box, tree, out["layout"], cen, siz, 64, 512)
    ncmax = lists.shape[1]

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    with ClockSampler(local) as clocks:
        build_ms = timed(lambda: cs.cluster_nblist(xs, ys, zs, hs, box, tree, out["layout"], cen, siz, 64, ncmax))
        loop_ms = timed(lambda: cs.ijloop_density_clusters(xs, ys, zs, hs, m, lists, counts))
        list_ms = timed(lambda: cs.ijloop_density_list(xs, ys, zs, hs, m, box, out["neighbors"],
                                                        out["neighbor_counts"]))
    rho_c = cs.ijloop_density_clusters(xs, ys, zs, hs, m, lists, counts)
    rho_l = cs.ijloop_density_list(xs, ys, zs, hs, m, box, out["neighbors"], out["neighbor_counts"])
    nc = out["neighbor_counts"]
    complete = bool((nc <= NGMAX).all())
    # both sums add every neighbour of every particle in ascending j when no list was truncated
    agree = float((rho_c == rho_l).double().mean())
    listed = float(counts.clamp(max=ncmax).double().sum())
    step_ms = max_over_ranks(build_ms + loop_ms, world)
    peak, peak_kind = measured_hbm_peak()
    algo = n * 48 + 4 * listed
    achieved = algo / (loop_ms * 1e-3) / 1e9
    if rank == 0:
        dist = "Plummer" if args.ijloop_dist == "plummer" else "uniform"
        line = {"metric": f"Mparticles/s neighbour-list consumers: cluster-pair lists + SPH density "
                          f"({n / 2 ** 20:g}M {dist}, FP64)",
                "value": round(world * n / (step_ms * 1e-3) / 1e6, 3), "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step_ms, 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic",
                "config": {"workload": "ijloop-density", "particles": args.ijloop_dist, "n_particles_per_gpu": n,
                           "neighbours_target": K_NEIGHBORS,
                           "cluster": 8, "ncmax": ncmax, "keys": "hilbert64", "bucket_size": BUCKET,
                           "l2": f"inputs ({n * 40 / 1e6:.0f} MB) "
                                 f"{'larger' if n * 40 > 129e6 else 'smaller'} than L2",
                           "parallelism": f"replicas x{world}"},
                "stages_ms": {"cluster_lists": round(build_ms, 4), "density_over_clusters": round(loop_ms, 4),
                              "density_over_stored_lists": round(list_ms, 4)},
                "pair_tests_per_neighbour": round(8 * listed * 8 / max(1.0, float(nc.double().sum())), 3),
                "roofline": {"kernel": "densityClusterKernel<double>", "bound": "fp64",
                             "achieved": round(achieved, 1), "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                             "frac": round(achieved / peak, 4), "algorithmic_bytes": algo,
                             "note": "the hbm fraction above is small by construction: the loop's exact tests and "
                                     "interaction terms run on the FP64 pipe, whose activity is below",
                             "fp64_pipe": density_profile_figures()},
                "stored_lists_complete": complete, "rho_identical_frac": agree,
                "rho_identical_note": "the cluster loop sums over every j within 2 h_i (checked against a brute-force "
                                      "sum); the stored lists follow findNeighbors, which looks only into leaves "
                                      "that pass its cell test, and a j just inside 2 h_i can sit in a leaf that "
                                      "fails it at the edge, so a few particles (19 of 16M) differ by one pair",
                "clocks": clocks.summary()}
        print(json.dumps(line), flush=True)


def run_served(args, world, rank, local):
    """A Poisson stream of requests (rate 2000/s) through the request server: sizes log-uniform in [2^12, 2^22], FP64
    uniform or Plummer (50/50), Hilbert64, bucket 64, per-request constant h for about 100 neighbours, 30 % of the
    requests incremental updates (displacement 0.05 spacing) of resident trees, 150 GB admission budget, 4 slots.
    Inputs come from a pool of pre-generated sets (the generation is not timed). Reports latency percentiles and the
    particles/s of the completed requests."""
    import numpy as np
    import torch

    import cstone_gb300 as cs
    from cstone_gb300 import workloads as W

    torch.cuda.set_device(local)
    rng = np.random.default_rng(args.seed + rank)
    pool = []
    for j in range(24):
        n = int(2 ** (12 + 10 * rng.random()))
        if j % 2:
            x, y, z = W.uniform(n, 0.0, 1.0, args.seed * 100 + j)
            lo, hi = (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)
            h = 0.5 * (3 * 100 / (4 * np.pi * n)) ** (1 / 3)
        else:
            x, y, z = W.plummer(n, args.seed * 100 + j)
            lo, hi = W.tight_box(x, y, z)
            rhalf = 1.0 / np.sqrt(0.5 ** (-2.0 / 3.0) - 1.0)
            h = 0.5 * (3 * 100 / (4 * np.pi * (n / 2) / (4 / 3 * np.pi * rhalf ** 3))) ** (1 / 3)
        hh = np.full(n, h)
        sp = (np.prod(np.array(hi) - np.array(lo)) / n) ** (1 / 3)
        moved = [np.clip(a + rng.normal(0, 0.05 * sp, n), l, u) for a, l, u in zip((x, y, z), lo, hi)]
        pool.append(dict(n=n, xyz=(x, y, z), moved=moved, h=hh, box=cs.make_box(lo, hi)))
    trees = list(range(8))
    srv = cs.Server(4, 150 * (1 << 30), 64, 64, cs.HILBERT, 64, 200, 1.0)
    # resident trees for the update requests (not timed)
    for t in trees:
        p = pool[t]
        srv.wait(srv.submit(*p["xyz"], p["h"], p["box"], cs.REQ_BUILD, t), counts=False)
    flip = {t: 0 for t in trees}

    def serve(rate, nreq, clocks=None):
        """Poisson arrivals at `rate` of nreq requests (30 % updates of resident trees); returns sorted latencies
        (ms), particles, seconds from the first arrival to the last result, the last arrival time"""
        arrivals = np.cumsum(rng.exponential(1.0 / rate, nreq))
        plan = []
        for k in range(nreq):
            if rng.random() < 0.3:
                t = int(rng.choice(trees))
                flip[t] ^= 1
                p = pool[t]
                plan.append((t, p["moved"] if flip[t] else p["xyz"], p, cs.REQ_UPDATE))
            else:
                p = pool[int(rng.integers(len(pool)))]
                plan.append((-1, p["xyz"], p, cs.REQ_BUILD))
        ids = []
        t0 = time.perf_counter()
        for k, (t, xyz, p, kind) in enumerate(plan):
            wait = t0 + arrivals[k] - time.perf_counter()
            if wait > 0:
                time.sleep(wait)
            ids.append((srv.submit(*xyz, p["h"], p["box"], kind, t), p["n"]))
        lat, parts = [], 0
        for rid, n in ids:
            r, _ = srv.wait(rid, counts=False)
            lat.append(r.latency_ms)
            parts += n
        return np.sort(np.array(lat)), parts, time.perf_counter() - t0, arrivals[-1]

    with ClockSampler(local) as clocks:
        lat, parts, elapsed, last_arrival = serve(args.rate, args.requests)
        # a rate the server sustains: 70 % of the completion rate it reached under the offered load
        sustain_rate = 0.7 * args.requests / elapsed
        nsus = max(60, args.requests // 3)
        slat, sparts, selapsed, slast = serve(sustain_rate, nsus)
    st = srv.stats()
    srv.close()
    arrivals = [last_arrival]
    if rank == 0:
        line = {"metric": "served requests: p50/p99 latency and Mparticles/s (Poisson 2000/s, 2^12..2^22 FP64)",
                "value": round(parts / elapsed / 1e6, 3), "unit": "Mparticles/s", "n_gpus": world,
                "steps": args.requests, "warmup": len(trees), "ms_per_step": round(elapsed * 1e3 / args.requests, 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic",
                "config": {"workload": "served-requests", "requests": args.requests, "rate_per_s": args.rate,
                           "sizes": "log-uniform [2^12, 2^22]", "mix": "uniform / Plummer 50/50",
                           "updates": "30 % of requests, one updateOctree step of a resident tree",
                           "keys": "hilbert64", "bucket_size": 64, "ngmax": 200, "neighbours": "about 100",
                           "slots": 4, "hbm_budget_gb": 150, "pool_sets": len(pool),
                           "parallelism": f"replicas x{world}"},
                "p50_ms": round(float(np.percentile(lat, 50)), 3), "p99_ms": round(float(np.percentile(lat, 99)), 3),
                "completed": int(st.completed) - len(trees) - nsus, "failed": int(st.failed), "particles": parts,
                "offered_Mparticles_per_s": round(parts / arrivals[-1] / 1e6, 3),
                "elapsed_s": round(elapsed, 3),
                "sustainable_rate": {"rate_per_s": round(sustain_rate, 2), "requests": nsus,
                                     "p50_ms": round(float(np.percentile(slat, 50)), 3),
                                     "p99_ms": round(float(np.percentile(slat, 99)), 3),
                                     "Mparticles_per_s": round(sparts / selapsed / 1e6, 3),
                                     "offered_Mparticles_per_s": round(sparts / slast / 1e6, 3),
                                     "note": "70 % of the completion rate reached at the configured rate"},
                "clocks": clocks.summary()}
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if args.workload == "incremental":
        run_incremental(args, world, rank, local)
        return
    if args.workload == "batched":
        run_batched(args, world, rank, local)
        return
    if args.workload == "served":
        run_served(args, world, rank, local)
        return
    if args.workload == "sort":
        run_sort(args, world, rank, local)
        return
    if args.workload == "ijloop":
        run_ijloop(args, world, rank, local)
        return

    import numpy as np
    import torch

    import cstone_gb300 as cs
    from cstone_gb300 import workloads as W

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n = args.n or 16 * 1024 * 1024
    x, y, z = W.plummer(n, args.seed + rank)
    lo, hi = W.tight_box(x, y, z)
    box = cs.make_box(lo, hi)
    tx, ty, tz = (torch.from_numpy(a).to(dev) for a in (x, y, z))
    th, hnc = W.h_for_k_neighbors(tx, ty, tz, box, K_NEIGHBORS, BUCKET)
    torch.cuda.synchronize()

    pipe = cs.Pipeline(64, 64, cs.HILBERT, BUCKET, NGMAX, 1.0, 1.0, True, True)
    for _ in range(args.warmup):
        pipe.run(tx, ty, tz, th, box, FOCUS)
    # the autotuner (part of the warm-up): each traversal tuning on the warm-up's inputs (scored by the neighbour
    # stage), then each sort tile shape (scored by the sort stage), the fastest kept
    autotune = None
    if not args.no_autotune:
        pipe.run(tx, ty, tz, th, box, FOCUS)
        r = pipe.autotune(2)
        # the last two candidates vary the sort's tile shape under the fastest traversal (scored by the sort stage)
        tried = r["tried"]
        autotune = {"neighbors_stage": {cs.tuning_label(c): round(ms, 3) for c, ms in tried[:-2]},
                    "sort_stage": {cs.tuning_label(c): round(ms, 3) for c, ms in tried[-2:]}}
    torch.cuda.synchronize()

    # ---- device-resident timed region ----
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stage_acc = {k: 0.0 for k in cs.STAGES}
    with ClockSampler(local) as clocks:
        barrier(world)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            torch.cuda.nvtx.range_push("step")
            pipe.run(tx, ty, tz, th, box, FOCUS)
            torch.cuda.nvtx.range_pop()
            st = pipe.stage_times()
            for k in st:
                stage_acc[k] += st[k]
        e1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
    ms = e0.elapsed_time(e1) / args.steps
    ms = max_over_ranks(ms, world)
    value = world * n / (ms * 1e-3) / 1e6
    stages = {k: v / args.steps for k, v in stage_acc.items()}
    res = pipe.result
    nc = pipe.outputs()["neighbor_counts"]
    mean_nc = float(nc.double().mean())
    stored = float(nc.clamp(max=NGMAX).double().sum())

    # ---- end to end through the host-buffer calls ----
    # headline e2e: pinned host inputs in, neighbour counts, halo flags and the stored neighbour lists (CSR, written
    # straight into pinned host memory) out, every step; the same without the lists beside it
    e2e = None
    if not args.no_e2e:
        hx, hy, hz, hh = (t.cpu().pin_memory() for t in (tx, ty, tz, th))
        nc_host = torch.empty(n, dtype=torch.int32).pin_memory()
        flags_host = torch.empty(res.num_nodes * 2 + 1024, dtype=torch.uint8).pin_memory()
        total = int(stored)
        off_host = torch.empty(n + 1, dtype=torch.int64).pin_memory()
        list_host = torch.empty(total + total // 8 + 1024, dtype=torch.int32).pin_memory()
        del nc
        torch.cuda.empty_cache()

        def timed_e2e(call, sync_each):
            for _ in range(max(1, args.warmup)):
                call()
                if sync_each:
                    pipe.wait()
            pipe.wait()
            barrier(world)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            e0.record(stream)
            for _ in range(args.steps):
                call()
                if sync_each:
                    pipe.wait()
            pipe.wait()
            e1.record(stream)
            torch.cuda.synchronize()
            wall = (time.perf_counter() - t0) * 1e3 / args.steps
            barrier(world)
            return max_over_ranks(e0.elapsed_time(e1) / args.steps, world), wall

        lists_ms, lists_wall = timed_e2e(
            lambda: pipe.run_host_csr(hx, hy, hz, hh, box, FOCUS, off_host, list_host, nc_out=nc_host,
                                      flags_out=flags_host, asynchronous=True), False)
        lists_ok = int(off_host[-1]) == total
        # the last pipelined step's device times: its stages and its copy-back (compaction, list copy)
        last_stages = {k: round(v, 3) for k, v in pipe.stage_times().items()}
        last_copy = {k: round(v, 3) for k, v in pipe.copy_times().items()}
        lists_sync_ms, _ = timed_e2e(
            lambda: pipe.run_host_csr(hx, hy, hz, hh, box, FOCUS, off_host, list_host, nc_out=nc_host,
                                      flags_out=flags_host), False)
        dev_ms, dev_wall = timed_e2e(
            lambda: pipe.run_host_async(hx, hy, hz, hh, box, FOCUS, nc_host, flags_host), False)
        d2h_small = n * 4 + res.num_nodes
        e2e = {"value": round(world * n / (lists_ms * 1e-3) / 1e6, 3), "unit": UNIT,
               "h2d_bytes_per_step": 4 * n * 8,
               "d2h_bytes_per_step": d2h_small + 8 * (n + 1) + 4 * total,
               "ms_per_step": round(lists_ms, 3), "wall_ms_per_step": round(lists_wall, 3),
               "returns": "neighbour counts, halo flags and the stored neighbour lists (CSR: u64 offsets + u32 "
                          "indices, the first min(nc, ngmax) per particle)",
               "lists_total": total, "lists_complete": lists_ok,
               "last_step_ms": {"stages": last_stages, "copy_back": last_copy},
               "api": "cs_pipeline_run_host_csr_async per step, cs_pipeline_wait at the end",
               "synchronous_calls": {"value": round(world * n / (lists_sync_ms * 1e-3) / 1e6, 3),
                                     "ms_per_step": round(lists_sync_ms, 3), "api": "cs_pipeline_run_host_csr"},
               "lists_on_device": {"value": round(world * n / (dev_ms * 1e-3) / 1e6, 3),
                                   "ms_per_step": round(dev_ms, 3), "wall_ms_per_step": round(dev_wall, 3),
                                   "d2h_bytes_per_step": d2h_small,
                                   "returns": "neighbour counts and halo flags; lists stay in device memory",
                                   "api": "cs_pipeline_run_host_async per step, cs_pipeline_wait at the end"}}

    # ---- roofline of the dominant kernel (neighbour search): HBM bytes and issued instructions ----
    peak, peak_kind = measured_hbm_peak()
    nb_bytes = n * (4 * 8 + 4) + 4.0 * stored  # x,y,z,h read + count written + stored neighbour indices
    nb_ms = stages["neighbors"]
    achieved = nb_bytes / (nb_ms * 1e-3) / 1e9
    prof = profile_figures(n)
    sm_mhz = clocks.summary().get("sm_mhz") or 2070.0
    roofline = {"kernel": "findNeighborsGroupKernel<double>", "bound": "issue", "achieved": round(achieved, 1),
                "peak": peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
                "traffic": prof.get("traffic"), "algorithmic_bytes": nb_bytes, "ms": round(nb_ms, 4),
                "traffic_source": prof.get("source"),
                "note": "the hbm fraction above is algorithmic bytes / event time / measured copy bandwidth; the "
                        "kernel is bound by instruction issue, whose fraction is below"}
    if prof.get("warp_instructions"):
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        issue_peak = sms * 4 * sm_mhz * 1e6 / 1e9  # warp instructions per ns = G/s
        issue_ach = prof["warp_instructions"] / (nb_ms * 1e-3) / 1e9
        roofline["issue"] = {"achieved": round(issue_ach, 1), "peak": round(issue_peak, 1),
                             "unit": "G warp-instructions/s", "frac": round(issue_ach / issue_peak, 4),
                             "warp_instructions": prof["warp_instructions"],
                             "peak_basis": f"{sms} SMs x 4 issue slots/clk x {sm_mhz:.0f} MHz (sampled)",
                             "source": prof.get("source")}

    # ---- CPU baseline on a bounded sample ----
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        O, sx, sy, sz, sh, sbox = cpu_sample(args.cpu_sample, args.seed)
        t = cpu_time(O, sx, sy, sz, sh, sbox)
        cpu = {"value": round(args.cpu_sample / t["total"] / 1e6, 3), "unit": UNIT, "cores": O.num_threads(),
               "kind": "port",
               "sample": f"{args.cpu_sample} particles of the same Plummer workload, one full pass",
               "stage_seconds": {k: round(v, 4) for k, v in t.items()}}

    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": "plummer-keys-to-neighbors", "n_particles_per_gpu": n, "ngmax": NGMAX,
                           "bucket_size": BUCKET, "keys": "hilbert64", "focus": "[0, 2^61)",
                           "neighbours_target": K_NEIGHBORS, "l2": "inputs (512 MB) larger than L2",
                           "parallelism": f"replicas x{world}"},
                "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks.summary(),
                "gpu_launches": None,
                "stages_ms": {k: round(v, 4) for k, v in stages.items()},
                "tuning": pipe.get_tuning(), "autotune_stage_ms": autotune,
                "tree": {"leaves": res.num_leaves, "nodes": res.num_nodes, "iterations": res.iterations,
                         "max_depth": res.max_depth, "focus_leaves": res.focus_last - res.focus_first},
                "mean_neighbors": round(mean_nc, 2), "h_converged_frac": float((hnc == K_NEIGHBORS).double().mean())}
        line["gpu_launches"] = gpu_launches_per_step(res) * args.steps
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def gpu_launches_per_step(res):
    """kernels this library launches in one pipeline step (memsets and copies not counted): keys 1, sort 1 histogram
    + 1 scan + one pass per 8 key bits, gather 1, build 1 cooperative + 1 one-warp read of its result, link 1 layout +
    prefix sort + invert + levelRange + link, geometry 1, halos 3 (search boxes, containment list, traversals),
    neighbour node prep 1 + outside-leaf marks 1, neighbours 1 (no periodic axis here)"""
    key_passes = (63 + 7) // 8
    prefix_passes = (3 * res.max_depth + 1 + 7) // 8
    return 1 + (2 + key_passes) + 1 + (1 + 1) + (1 + 2 + prefix_passes + 3) + 1 + 3 + 2 + 1


if __name__ == "__main__":
    main()
