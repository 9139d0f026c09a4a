"""numpy front-end for the CPU oracle (cs_oracle.c) and, where it was built, for the reference's own CPU code
(oracle/_ref/libcsref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by the CPU-baseline leg of bench.py.
The product path never imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcsoracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libcsref.so")

MORTON, HILBERT = 0, 1
OPEN, PERIODIC = 0, 1


class CsoBox(C.Structure):
    _fields_ = [("lo", C.c_double * 3), ("hi", C.c_double * 3), ("boundary", C.c_int * 3)]


def make_box(lo, hi, boundary=(0, 0, 0)):
    lo = [float(v) for v in (lo if np.ndim(lo) else [lo] * 3)]
    hi = [float(v) for v in (hi if np.ndim(hi) else [hi] * 3)]
    b = list(boundary) if np.ndim(boundary) else [int(boundary)] * 3
    return CsoBox((C.c_double * 3)(*lo), (C.c_double * 3)(*hi), (C.c_int * 3)(*b))


def build(force=False):
    """Compile the restatement with the committed Makefile (gcc, OpenMP)."""
    if force or not os.path.exists(LIB_PATH) or _stale(LIB_PATH, ["cs_oracle.c", "cs_oracle_real.inc",
                                                                  "cs_oracle_next.inc", "cs_oracle.h"]):
        subprocess.check_call(["make", "-s", "-C", HERE, "libcsoracle.so"])


def build_ref(reference_root="/root/reference"):
    """Compile the reference's CPU code in place (only where its sources exist). Returns True if available."""
    if not os.path.isdir(os.path.join(reference_root, "include", "cstone")):
        return os.path.exists(REF_PATH)
    if not os.path.exists(REF_PATH) or _stale(REF_PATH, ["ref_driver.cpp"]):
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", f"REFERENCE={reference_root}"])
    return True


def _stale(target, sources):
    t = os.path.getmtime(target)
    return any(os.path.getmtime(os.path.join(HERE, s)) > t for s in sources)


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB_PATH)
        _lib.cso_imorton.restype = C.c_uint64
        _lib.cso_ihilbert.restype = C.c_uint64
        _lib.cso_rebalance_decision.restype = C.c_int
        _lib.cso_rebalance_tree.restype = C.c_int32
        _lib.cso_update_octree.restype = C.c_int
        _lib.cso_compute_octree.restype = C.c_int32
        _lib.cso_binary_key_weight.restype = C.c_int32
        _lib.cso_num_threads.restype = C.c_int
        for name in ("cso_span_sfc_range", "cso_fill_sfc_gaps", "cso_group_splits_f64", "cso_group_splits_f32"):
            getattr(_lib, name).restype = C.c_int32
        _lib.cso_protect_ancestors.restype = C.c_int
        _lib.cso_enforce_keys.restype = C.c_int
    return _lib


def ref():
    """The reference's own CPU implementation, or None where it cannot be built."""
    global _ref
    if _ref is None:
        if not build_ref():
            return None
        _ref = C.CDLL(REF_PATH)
        _ref.csr_imorton.restype = C.c_uint64
        _ref.csr_ihilbert.restype = C.c_uint64
        _ref.csr_rebalance_decision.restype = C.c_int
        _ref.csr_compute_octree.restype = C.c_int32
        _ref.csr_update_octree.restype = C.c_int
        _ref.csr_binary_key_weight.restype = C.c_int32
        _ref.csr_spanning_tree.restype = C.c_int32
        _ref.csr_mac_refine_op.restype = C.c_int
        _ref.csr_protect_ancestors.restype = C.c_int
        _ref.csr_enforce_keys.restype = C.c_int
    return _ref


def num_threads():
    return lib().cso_num_threads()


# ---------------------------------------------------------------------------------------------------------------
# restatement API (numpy in / numpy out)
# ---------------------------------------------------------------------------------------------------------------

def imorton(ix, iy, iz, key_bits):
    return lib().cso_imorton(C.c_uint(ix), C.c_uint(iy), C.c_uint(iz), key_bits)


def ihilbert(ix, iy, iz, key_bits):
    return lib().cso_ihilbert(C.c_uint(ix), C.c_uint(iy), C.c_uint(iz), key_bits)


def decode_hilbert(key, key_bits):
    out = (C.c_uint * 3)()
    lib().cso_decode_hilbert(C.c_uint64(key), key_bits, out)
    return tuple(out)


def decode_morton(key, key_bits):
    out = (C.c_uint * 3)()
    lib().cso_decode_morton(C.c_uint64(key), key_bits, out)
    return tuple(out)


def sfc_keys(x, y, z, box, kind=HILBERT, key_bits=64, keys=None, respect_remove_key=False):
    x, y, z = (np.ascontiguousarray(a) for a in (x, y, z))
    n = x.size
    keys = np.zeros(n, np.uint64) if keys is None else np.ascontiguousarray(keys, dtype=np.uint64).copy()
    fn = lib().cso_sfc_keys_f64 if x.dtype == np.float64 else lib().cso_sfc_keys_f32
    fn(_p(x), _p(y), _p(z), _p(keys), C.c_size_t(n), C.byref(box), kind, key_bits, int(respect_remove_key))
    return keys


def sort_by_key(keys, values=None):
    k = np.ascontiguousarray(keys, dtype=np.uint64).copy()
    v = np.arange(k.size, dtype=np.uint32) if values is None else np.ascontiguousarray(values, np.uint32).copy()
    lib().cso_sort_by_key(_p(k), _p(v), C.c_size_t(k.size))
    return k, v


def find_search_bounds(guess, target, codes, key_bits=64):
    codes = np.ascontiguousarray(codes, np.uint64)
    lo, hi = C.c_int64(), C.c_int64()
    lib().cso_find_search_bounds(C.c_int64(guess), C.c_uint64(target), _p(codes), C.c_int64(codes.size), key_bits,
                                 C.byref(lo), C.byref(hi))
    return lo.value, hi.value


def node_counts(tree, keys, key_bits=64, max_count=0xFFFFFFFF, guess_counts=None):
    tree = np.ascontiguousarray(tree, np.uint64)
    keys = np.ascontiguousarray(keys, np.uint64)
    L = tree.size - 1
    counts = np.zeros(L, np.uint32) if guess_counts is None else np.ascontiguousarray(guess_counts, np.uint32).copy()
    lib().cso_node_counts(_p(tree), _p(counts), L, _p(keys), C.c_size_t(keys.size), C.c_uint32(max_count),
                          int(guess_counts is not None), key_bits)
    return counts


def rebalance_decision(tree, counts, bucket, key_bits=64):
    tree = np.ascontiguousarray(tree, np.uint64)
    counts = np.ascontiguousarray(counts, np.uint32)
    L = tree.size - 1
    ops = np.zeros(L + 1, np.int32)
    conv = lib().cso_rebalance_decision(_p(tree), _p(counts), L, bucket, _p(ops), key_bits)
    return ops[:L], bool(conv)


def rebalance_tree(tree, ops, key_bits=64):
    tree = np.ascontiguousarray(tree, np.uint64)
    L = tree.size - 1
    o = np.zeros(L + 1, np.int32)
    o[:L] = ops[:L]
    cap = int(np.sum(o, dtype=np.int64))
    nt = np.zeros(cap + 1, np.uint64)
    nn = lib().cso_rebalance_tree(_p(tree), L, _p(o), _p(nt), cap, key_bits)
    return nt[: nn + 1]


def compute_octree(keys, bucket, key_bits=64, max_count=0xFFFFFFFF):
    keys = np.ascontiguousarray(keys, np.uint64)
    cap = max(64, 8 * (keys.size // max(bucket, 1) + 1) * 8)
    while True:
        tree = np.zeros(cap + 1, np.uint64)
        counts = np.zeros(cap, np.uint32)
        it = C.c_int()
        L = lib().cso_compute_octree(_p(keys), C.c_size_t(keys.size), bucket, C.c_uint32(max_count), _p(tree),
                                     _p(counts), cap, key_bits, C.byref(it))
        if L > 0:
            return tree[: L + 1].copy(), counts[:L].copy(), it.value
        cap = 2 * max(cap, -L)


def update_octree(keys, bucket, tree, counts, key_bits=64, max_count=0xFFFFFFFF):
    keys = np.ascontiguousarray(keys, np.uint64)
    L0 = np.asarray(tree).size - 1
    cap = max(64, 4096 * L0 + 8)
    t = np.zeros(cap + 1, np.uint64)
    c = np.zeros(cap, np.uint32)
    t[: L0 + 1] = tree
    c[:L0] = counts
    L = C.c_int32(L0)
    conv = lib().cso_update_octree(_p(keys), C.c_size_t(keys.size), bucket, C.c_uint32(max_count), _p(t), _p(c),
                                   C.byref(L), cap, key_bits)
    assert conv >= 0
    return t[: L.value + 1].copy(), c[: L.value].copy(), bool(conv)


def binary_key_weight(key, level, key_bits=64):
    return lib().cso_binary_key_weight(C.c_uint64(key), level, key_bits)


class Octree:
    """Linked octree arrays (OctreeData, tree/octree.hpp:285-360)."""

    def __init__(self, **kw):
        self.__dict__.update(kw)


def octree_sizes(L):
    I = (L - 1) // 7
    N = L + I
    return I, N, max(1, (N - 1) // 8)


def build_octree(leaves, key_bits=64):
    leaves = np.ascontiguousarray(leaves, np.uint64)
    L = leaves.size - 1
    I, N, P = octree_sizes(L)
    prefixes = np.zeros(N, np.uint64)
    child = np.zeros(N + 1, np.int32)
    parents = np.zeros(P, np.int32)
    lr = np.zeros((10 if key_bits == 32 else 21) + 2, np.int32)
    i2l = np.zeros(N, np.int32)
    l2i = np.zeros(N, np.int32)
    lib().cso_build_octree(_p(leaves), L, key_bits, _p(prefixes), _p(child), _p(parents), _p(lr), _p(i2l), _p(l2i))
    return Octree(num_leaves=L, num_internal=I, num_nodes=N, prefixes=prefixes, child_offsets=child[:N],
                  parents=parents, level_range=lr, internal_to_leaf=i2l, leaf_to_internal=l2i, leaves=leaves)


def node_fp_centers(prefixes, box, dtype=np.float64, kind=HILBERT, key_bits=64):
    prefixes = np.ascontiguousarray(prefixes, np.uint64)
    N = prefixes.size
    c = np.zeros((N, 3), dtype)
    s = np.zeros((N, 3), dtype)
    fn = lib().cso_node_fp_centers_f64 if dtype == np.float64 else lib().cso_node_fp_centers_f32
    fn(_p(prefixes), N, kind, key_bits, C.byref(box), _p(c), _p(s))
    return c, s


def search_boxes(x, y, z, h, layout, first, last, scale, leaf_to_internal_leaves, node_centers, use_ref=False):
    """computeBoundingBox per leaf; h may be float32 with double coordinates (Th = float)"""
    dt = x.dtype
    if dt == np.float64 and h.dtype == np.float32:
        L = layout.size - 1
        sc = np.zeros((L, 3), dt)
        ss = np.zeros((L, 3), dt)
        fn = ref().csr_search_boxes_f64_hf32 if use_ref else lib().cso_search_boxes_f64_hf32
        fn(_p(x), _p(y), _p(z), _p(h), _p(np.ascontiguousarray(layout, np.uint32)), first, last, C.c_float(scale),
           _p(np.ascontiguousarray(leaf_to_internal_leaves, np.int32)), _p(np.ascontiguousarray(node_centers, dt)),
           _p(sc), _p(ss))
        return sc, ss
    L = layout.size - 1
    sc = np.zeros((L, 3), dt)
    ss = np.zeros((L, 3), dt)
    fn = lib().cso_search_boxes_f64 if dt == np.float64 else lib().cso_search_boxes_f32
    cs = C.c_double(scale) if dt == np.float64 else C.c_float(scale)
    l2i = np.ascontiguousarray(leaf_to_internal_leaves, np.int32)
    fn(_p(x), _p(y), _p(z), _p(h), _p(np.ascontiguousarray(layout, np.uint32)), first, last, cs, _p(l2i),
       _p(np.ascontiguousarray(node_centers, dt)), _p(sc), _p(ss))
    return sc, ss


def find_halos(tree, node_centers, node_sizes, search_centers, search_sizes, box, first, last, key_bits=64):
    dt = node_centers.dtype
    flags = np.zeros(tree.num_nodes, np.uint8)
    fn = lib().cso_find_halos_f64 if dt == np.float64 else lib().cso_find_halos_f32
    fn(_p(tree.prefixes), _p(tree.child_offsets), _p(tree.parents), _p(node_centers), _p(node_sizes),
       _p(tree.leaves), _p(np.ascontiguousarray(search_centers, dt)), _p(np.ascontiguousarray(search_sizes, dt)),
       C.byref(box), first, last, key_bits, _p(flags))
    return flags


def find_neighbors(x, y, z, h, first, last, box, tree, layout, centers, sizes, ngmax, search_ext=1.0):
    """findNeighbors over [first, last); h may be float32 with double coordinates (Th = float)"""
    dt = x.dtype
    n = last - first
    nb = np.zeros(n * ngmax, np.uint32)
    nc = np.zeros(n, np.uint32)
    fn = lib().cso_find_neighbors_f64 if dt == np.float64 else lib().cso_find_neighbors_f32
    if dt == np.float64 and h.dtype == np.float32:
        fn = lib().cso_find_neighbors_f64_hf32
    fn(_p(x), _p(y), _p(z), _p(h), C.c_uint32(first), C.c_uint32(last), C.byref(box), _p(tree.child_offsets),
       _p(tree.parents), _p(tree.internal_to_leaf), _p(np.ascontiguousarray(layout, np.uint32)), _p(centers),
       _p(sizes), C.c_float(search_ext), C.c_uint(ngmax), _p(nb), _p(nc))
    return nb.reshape(n, ngmax), nc


def philox_uniform(seed, stream, n, lo, hi):
    out = np.empty(n, np.float64)
    lib().cso_philox_uniform_f64(C.c_uint64(seed), C.c_uint64(stream), _p(out), C.c_size_t(n), C.c_double(lo),
                                 C.c_double(hi))
    return out


def plummer(seed, n, rmax=100.0):
    x, y, z = (np.empty(n, np.float64) for _ in range(3))
    lib().cso_plummer_f64(C.c_uint64(seed), _p(x), _p(y), _p(z), C.c_size_t(n), C.c_double(rmax))
    return x, y, z


def layout_from_counts(counts):
    layout = np.zeros(counts.size + 1, np.uint32)
    np.cumsum(counts, out=layout[1:])
    return layout


def pipeline(x, y, z, h, box, bucket, ngmax, kind=HILBERT, key_bits=64, search_ext=1.0, with_neighbors=True):
    """keys -> stable sort -> gather -> computeOctree -> link -> node geometry -> findNeighbors (all CPU)."""
    keys = sfc_keys(x, y, z, box, kind, key_bits)
    skeys, perm = sort_by_key(keys)
    xs, ys, zs, hs = (a[perm] for a in (x, y, z, h))
    leaves, counts, iters = compute_octree(skeys, bucket, key_bits)
    tree = build_octree(leaves, key_bits)
    centers, sizes = node_fp_centers(tree.prefixes, box, x.dtype, kind, key_bits)
    layout = layout_from_counts(counts)
    out = dict(keys=keys, sorted_keys=skeys, perm=perm, x=xs, y=ys, z=zs, h=hs, leaves=leaves, counts=counts,
               iterations=iters, tree=tree, centers=centers, sizes=sizes, layout=layout)
    if with_neighbors:
        nb, nc = find_neighbors(xs, ys, zs, hs, 0, x.size, box, tree, layout, centers, sizes, ngmax, search_ext)
        out.update(nb=nb, nc=nc)
    return out


# ---------------------------------------------------------------------------------------------------------------
# the reference's own CPU code (oracle/_ref), same call shapes as above; used to pin the restatement
# ---------------------------------------------------------------------------------------------------------------

def _box_arrays(box):
    lo = np.array(box.lo[:], np.float64)
    hi = np.array(box.hi[:], np.float64)
    b = np.array(box.boundary[:], np.int32)
    return lo, hi, b


def ref_sfc_keys(x, y, z, box, kind=HILBERT, key_bits=64, keys=None):
    r = ref()
    n = x.size
    keys = np.zeros(n, np.uint64) if keys is None else np.ascontiguousarray(keys, np.uint64).copy()
    lo, hi, b = _box_arrays(box)
    fn = r.csr_sfc_keys_f64 if x.dtype == np.float64 else r.csr_sfc_keys_f32
    fn(_p(x), _p(y), _p(z), _p(keys), C.c_size_t(n), _p(lo), _p(hi), _p(b), kind, key_bits)
    return keys


def ref_sort_by_key(keys, values=None):
    k = np.ascontiguousarray(keys, np.uint64).copy()
    v = np.arange(k.size, dtype=np.uint32) if values is None else np.ascontiguousarray(values, np.uint32).copy()
    ref().csr_sort_by_key(_p(k), _p(v), C.c_size_t(k.size))
    return k, v


def ref_find_search_bounds(guess, target, codes):
    codes = np.ascontiguousarray(codes, np.uint64)
    lo, hi = C.c_int64(), C.c_int64()
    ref().csr_find_search_bounds(C.c_int64(guess), C.c_uint64(target), _p(codes), C.c_int64(codes.size),
                                 C.byref(lo), C.byref(hi))
    return lo.value, hi.value


def ref_node_counts(tree, keys, key_bits=64, max_count=0xFFFFFFFF, guess_counts=None):
    tree = np.ascontiguousarray(tree, np.uint64)
    keys = np.ascontiguousarray(keys, np.uint64)
    L = tree.size - 1
    counts = np.zeros(L, np.uint32) if guess_counts is None else np.ascontiguousarray(guess_counts, np.uint32).copy()
    ref().csr_node_counts(_p(tree), _p(counts), L, _p(keys), C.c_size_t(keys.size), C.c_uint32(max_count),
                          int(guess_counts is not None), key_bits)
    return counts


def ref_rebalance_decision(tree, counts, bucket, key_bits=64):
    tree = np.ascontiguousarray(tree, np.uint64)
    counts = np.ascontiguousarray(counts, np.uint32)
    L = tree.size - 1
    ops = np.zeros(L + 1, np.int32)
    conv = ref().csr_rebalance_decision(_p(tree), _p(counts), L, bucket, _p(ops), key_bits)
    return ops[:L], bool(conv)


def ref_compute_octree(keys, bucket, key_bits=64, max_count=0xFFFFFFFF):
    keys = np.ascontiguousarray(keys, np.uint64)
    cap = max(64, 64 * (keys.size // max(bucket, 1) + 1))
    while True:
        tree = np.zeros(cap + 1, np.uint64)
        counts = np.zeros(cap, np.uint32)
        it = C.c_int()
        L = ref().csr_compute_octree(_p(keys), C.c_size_t(keys.size), bucket, C.c_uint32(max_count), _p(tree),
                                     _p(counts), cap, key_bits, C.byref(it))
        if L > 0:
            return tree[: L + 1].copy(), counts[:L].copy(), it.value
        cap = 2 * max(cap, -L)


def ref_update_octree(keys, bucket, tree, counts, key_bits=64, max_count=0xFFFFFFFF):
    keys = np.ascontiguousarray(keys, np.uint64)
    L0 = np.asarray(tree).size - 1
    cap = max(64, 4096 * L0 + 8)
    t = np.zeros(cap + 1, np.uint64)
    c = np.zeros(cap, np.uint32)
    t[: L0 + 1] = tree
    c[:L0] = counts
    L = C.c_int32(L0)
    conv = ref().csr_update_octree(_p(keys), C.c_size_t(keys.size), bucket, C.c_uint32(max_count), _p(t), _p(c),
                                   C.byref(L), cap, key_bits)
    return t[: L.value + 1].copy(), c[: L.value].copy(), bool(conv)


def ref_build_octree(leaves, key_bits=64):
    leaves = np.ascontiguousarray(leaves, np.uint64)
    L = leaves.size - 1
    I, N, P = octree_sizes(L)
    prefixes = np.zeros(N, np.uint64)
    child = np.zeros(N + 1, np.int32)
    parents = np.zeros(P, np.int32)
    lr = np.zeros((10 if key_bits == 32 else 21) + 2, np.int32)
    i2l = np.zeros(N, np.int32)
    l2i = np.zeros(N, np.int32)
    ref().csr_build_octree(_p(leaves), L, key_bits, _p(prefixes), _p(child), _p(parents), _p(lr), _p(i2l), _p(l2i))
    return Octree(num_leaves=L, num_internal=I, num_nodes=N, prefixes=prefixes, child_offsets=child[:N],
                  parents=parents, level_range=lr, internal_to_leaf=i2l, leaf_to_internal=l2i, leaves=leaves)


def ref_node_fp_centers(prefixes, box, dtype=np.float64, key_bits=64):
    prefixes = np.ascontiguousarray(prefixes, np.uint64)
    N = prefixes.size
    c = np.zeros((N, 3), dtype)
    s = np.zeros((N, 3), dtype)
    lo, hi, b = _box_arrays(box)
    fn = ref().csr_node_fp_centers_f64 if dtype == np.float64 else ref().csr_node_fp_centers_f32
    fn(_p(prefixes), N, key_bits, _p(lo), _p(hi), _p(b), _p(c), _p(s))
    return c, s


def ref_search_boxes(x, y, z, h, layout, first, last, scale, leaf_to_internal_leaves, node_centers):
    dt = x.dtype
    L = layout.size - 1
    sc = np.zeros((L, 3), dt)
    ss = np.zeros((L, 3), dt)
    fn = ref().csr_search_boxes_f64 if dt == np.float64 else ref().csr_search_boxes_f32
    cs = C.c_double(scale) if dt == np.float64 else C.c_float(scale)
    l2i = np.ascontiguousarray(leaf_to_internal_leaves, np.int32)
    fn(_p(x), _p(y), _p(z), _p(h), _p(np.ascontiguousarray(layout, np.uint32)), first, last, cs, _p(l2i),
       _p(np.ascontiguousarray(node_centers, dt)), _p(sc), _p(ss))
    return sc, ss


def ref_find_halos(tree, node_centers, node_sizes, search_centers, search_sizes, box, first, last, key_bits=64):
    dt = node_centers.dtype
    flags = np.zeros(tree.num_nodes, np.uint8)
    lo, hi, b = _box_arrays(box)
    fn = ref().csr_find_halos_f64 if dt == np.float64 else ref().csr_find_halos_f32
    fn(_p(tree.prefixes), _p(tree.child_offsets), _p(tree.parents), _p(node_centers), _p(node_sizes),
       _p(tree.leaves), tree.num_nodes, tree.num_leaves, _p(np.ascontiguousarray(search_centers, dt)),
       _p(np.ascontiguousarray(search_sizes, dt)), _p(lo), _p(hi), _p(b), first, last, key_bits, _p(flags))
    return flags


def ref_find_neighbors(x, y, z, h, first, last, box, tree, layout, centers, sizes, ngmax, search_ext=1.0):
    dt = x.dtype
    n = last - first
    nb = np.zeros(n * ngmax, np.uint32)
    nc = np.zeros(n, np.uint32)
    lo, hi, b = _box_arrays(box)
    fn = ref().csr_find_neighbors_f64 if dt == np.float64 else ref().csr_find_neighbors_f32
    if dt == np.float64 and h.dtype == np.float32:
        fn = ref().csr_find_neighbors_f64_hf32
    fn(_p(x), _p(y), _p(z), _p(h), C.c_uint32(first), C.c_uint32(last), _p(lo), _p(hi), _p(b), tree.num_leaves,
       tree.num_nodes, _p(tree.child_offsets), _p(tree.parents), _p(tree.internal_to_leaf),
       _p(np.ascontiguousarray(layout, np.uint32)), _p(centers), _p(sizes), C.c_float(search_ext), C.c_uint(ngmax),
       _p(nb), _p(nc))
    return nb.reshape(n, ngmax), nc


# ---------------------------------------------------------------------------------------------------------------
# CPU baseline: the whole path on the host cores, stage by stage
# ---------------------------------------------------------------------------------------------------------------

def h_for_k_neighbors_cpu(x, y, z, box, k=100, tol=0.1, bucket=64, max_iter=40):
    """h (input order) with |count(2h) - k| <= tol*k, by per-particle bisection with the oracle's counts."""
    n = x.size
    keys = sfc_keys(x, y, z, box)
    skeys, perm = sort_by_key(keys)
    xs, ys, zs = x[perm], y[perm], z[perm]
    leaves, counts, _ = compute_octree(skeys, bucket)
    tree = build_octree(leaves)
    centers, sizes = node_fp_centers(tree.prefixes, box, x.dtype)
    layout = layout_from_counts(counts)
    idx = np.arange(n)
    j = np.where(idx + k < n, idx + k, np.maximum(idx - k, 0))
    h = 0.5 * np.sqrt((xs - xs[j]) ** 2 + (ys - ys[j]) ** 2 + (zs - zs[j]) ** 2)
    h[h <= 0] = h[h > 0].min()
    lo = np.zeros(n)
    hi = np.full(n, np.inf)
    for _ in range(max_iter):
        _, nc = find_neighbors(xs, ys, zs, h, 0, n, box, tree, layout, centers, sizes, 0)
        low = nc < k * (1 - tol)
        high = nc > k * (1 + tol)
        if not (low | high).any():
            break
        lo = np.where(low, h, lo)
        hi = np.where(high, h, hi)
        ratio = (k / np.maximum(nc, 1)) ** (1.0 / 3.0)
        br = (lo > 0) & np.isfinite(hi)
        hn = np.where(br, 0.5 * (lo + hi), np.where(low, h * np.clip(ratio, 1.02, 4), h * np.clip(ratio, 0.25, 0.98)))
        h = np.where(low | high, hn, h)
    out = np.empty(n)
    out[perm] = h
    return out


def timed_pipeline(x, y, z, h, box, bucket, ngmax, focus=(0, 0), kind=HILBERT, key_bits=64, halo_ext=1.0):
    """keys -> stable sort -> gather -> computeOctree -> link -> geometry -> search boxes + findHalos ->
    findNeighbors on the CPU; returns (stage seconds dict, outputs dict)."""
    import time

    t = {}
    n = x.size
    c0 = time.perf_counter()
    keys = sfc_keys(x, y, z, box, kind, key_bits)
    c1 = time.perf_counter()
    skeys, perm = sort_by_key(keys)
    c2 = time.perf_counter()
    outs = []
    for a in (x, y, z, h):
        o = np.empty_like(a)
        fn = lib().cso_gather_f64 if a.dtype == np.float64 else lib().cso_gather_f32
        fn(_p(perm), _p(a), _p(o), C.c_size_t(n))
        outs.append(o)
    xs, ys, zs, hs = outs
    c3 = time.perf_counter()
    leaves, counts, iters = compute_octree(skeys, bucket, key_bits)
    c4 = time.perf_counter()
    tree = build_octree(leaves, key_bits)
    c5 = time.perf_counter()
    centers, sizes = node_fp_centers(tree.prefixes, box, x.dtype, kind, key_bits)
    layout = layout_from_counts(counts)
    c6 = time.perf_counter()
    flags = sboxes = None
    if focus[1] > focus[0]:
        first = int(np.searchsorted(leaves, np.uint64(focus[0])))
        last = int(np.searchsorted(leaves, np.uint64(focus[1])))
        l2i = tree.leaf_to_internal[tree.num_internal:]
        sc, ss = search_boxes(xs, ys, zs, hs, layout, first, last, 2.0 * halo_ext, l2i, centers)
        flags = find_halos(tree, centers, sizes, sc, ss, box, first, last, key_bits)
        sboxes = (first, last, sc, ss)
    c7 = time.perf_counter()
    nb, nc = find_neighbors(xs, ys, zs, hs, 0, n, box, tree, layout, centers, sizes, ngmax)
    c8 = time.perf_counter()
    t = dict(keys=c1 - c0, sort=c2 - c1, gather=c3 - c2, build=c4 - c3, link=c5 - c4, geometry=c6 - c5,
             halos=c7 - c6, neighbors=c8 - c7, total=c8 - c0)
    return t, dict(sorted_keys=skeys, perm=perm, leaves=leaves, counts=counts, iterations=iters, tree=tree,
                   centers=centers, sizes=sizes, flags=flags, search_boxes=sboxes, nb=nb, nc=nc)


# ---------------------------------------------------------------------------------------------------------------
# around the path: upsweeps, source centres, groups, SFC gaps, focus rebalance (cs_oracle_next.inc) and the
# reference's own versions (csr_*) where it has CPU code
# ---------------------------------------------------------------------------------------------------------------

def span_sfc_range(a, b, key_bits=64):
    n = lib().cso_span_sfc_range(C.c_uint64(a), C.c_uint64(b), None, key_bits)
    out = np.zeros(max(n, 1), np.uint64)
    lib().cso_span_sfc_range(C.c_uint64(a), C.c_uint64(b), _p(out), key_bits)
    return out[:n]


def fill_sfc_gaps(keys, key_bits=64):
    keys = np.ascontiguousarray(keys, np.uint64)
    cap = 64
    while True:
        out = np.zeros(cap, np.uint64)
        r = lib().cso_fill_sfc_gaps(_p(keys), keys.size - 1, _p(out), cap, key_bits)
        if r > 0:
            return out[:r]
        cap = -r


def ref_spanning_tree(keys, key_bits=64):
    keys = np.ascontiguousarray(keys, np.uint64)
    cap = 64
    while True:
        out = np.zeros(cap, np.uint64)
        r = ref().csr_spanning_tree(_p(keys), keys.size, _p(out), cap, key_bits)
        if r > 0:
            return out[:r]
        cap = -r


def upsweep_sum(level_range, child_offsets, counts, use_ref=False):
    lr = np.ascontiguousarray(level_range, np.int32)
    c = np.ascontiguousarray(counts, np.uint32).copy()
    fn = ref().csr_upsweep_sum if use_ref else lib().cso_upsweep_sum
    fn(_p(lr), lr.size - 1, _p(np.ascontiguousarray(child_offsets, np.int32)), _p(c))
    return c


def leaf_mass_centers(x, y, z, m, leaf_to_internal, layout, num_nodes, use_ref=False):
    dt = np.float64 if x.dtype == np.float64 else np.float32
    cen = np.zeros((num_nodes, 4), dt)
    l2i = np.ascontiguousarray(leaf_to_internal, np.int32)
    lay = np.ascontiguousarray(layout, np.uint32)
    if use_ref:
        fn = ref().csr_leaf_mass_centers_f64 if dt == np.float64 else ref().csr_leaf_mass_centers_f32
        fn(_p(x), _p(y), _p(z), _p(m), _p(l2i), l2i.size, _p(lay), _p(cen), C.c_size_t(x.size))
    else:
        if dt == np.float64:
            fn = lib().cso_leaf_mass_centers_f64 if m.dtype == np.float64 else lib().cso_leaf_mass_centers_f64m32
        else:
            fn = lib().cso_leaf_mass_centers_f32
        fn(_p(x), _p(y), _p(z), _p(m), _p(l2i), l2i.size, _p(lay), _p(cen))
    return cen


def upsweep_centers(level_range, child_offsets, centers, use_ref=False):
    lr = np.ascontiguousarray(level_range, np.int32)
    c = np.ascontiguousarray(centers).copy()
    if use_ref:
        fn = ref().csr_upsweep_centers_f64 if c.dtype == np.float64 else ref().csr_upsweep_centers_f32
    else:
        fn = lib().cso_upsweep_centers_f64 if c.dtype == np.float64 else lib().cso_upsweep_centers_f32
    fn(_p(lr), lr.size - 1, _p(np.ascontiguousarray(child_offsets, np.int32)), _p(c))
    return c


def group_splits(first, last, x, y, z, h, leaves, layout, lo, hi, group_size, tol, key_bits=64):
    dt = x.dtype
    fn = lib().cso_group_splits_f64 if dt == np.float64 else lib().cso_group_splits_f32
    lo = np.array(lo, np.float64)
    hi = np.array(hi, np.float64)
    leaves = np.ascontiguousarray(leaves, np.uint64)
    lay = np.ascontiguousarray(layout, np.uint32)
    cap = 2 * ((last - first) // max(1, group_size) + 2)
    while True:
        g = np.zeros(cap, np.uint32)
        r = fn(C.c_uint32(first), C.c_uint32(last), _p(x), _p(y), _p(z), _p(h), _p(leaves), leaves.size - 1, _p(lay),
               _p(lo), _p(hi), C.c_uint(group_size), C.c_float(tol), _p(g), cap, key_bits)
        if r >= 0:
            return g[: r + 1]
        cap = -r


def rebalance_decision_essential(prefixes, child_offsets, parents, counts, macs, focus, bucket, key_bits=64,
                                 use_ref=False):
    N = prefixes.size
    ops = np.zeros(N, np.int32)
    args = [_p(np.ascontiguousarray(prefixes, np.uint64)), _p(np.ascontiguousarray(child_offsets, np.int32)),
            _p(np.ascontiguousarray(parents, np.int32)), _p(np.ascontiguousarray(counts, np.uint32)),
            _p(np.ascontiguousarray(macs, np.uint8)), N, C.c_uint64(focus[0]), C.c_uint64(focus[1]),
            C.c_uint(bucket), _p(ops), key_bits]
    (ref().csr_rebalance_decision_essential if use_ref else lib().cso_rebalance_decision_essential)(*args)
    return ops


def mac_refine_decision(prefixes, macs, l2i, focus_first, focus_last, key_bits=64):
    L = l2i.size
    ops = np.zeros(L, np.int32)
    lib().cso_mac_refine_decision(_p(np.ascontiguousarray(prefixes, np.uint64)),
                                  _p(np.ascontiguousarray(macs, np.uint8)), _p(np.ascontiguousarray(l2i, np.int32)),
                                  L, focus_first, focus_last, _p(ops), key_bits)
    return ops


def protect_ancestors(prefixes, parents, ops, key_bits=64, use_ref=False):
    o = np.ascontiguousarray(ops, np.int32).copy()
    pre = np.ascontiguousarray(prefixes, np.uint64)
    par = np.ascontiguousarray(parents, np.int32)
    fn = ref().csr_protect_ancestors if use_ref else lib().cso_protect_ancestors
    conv = fn(_p(pre), _p(par), _p(o), pre.size, key_bits)
    return o, bool(conv)


def enforce_keys(keys, prefixes, child_offsets, parents, ops, key_bits=64, use_ref=False):
    o = np.ascontiguousarray(ops, np.int32).copy()
    k = np.ascontiguousarray(keys, np.uint64)
    pre = np.ascontiguousarray(prefixes, np.uint64)
    co = np.ascontiguousarray(child_offsets, np.int32)
    par = np.ascontiguousarray(parents, np.int32)
    if use_ref:
        st = ref().csr_enforce_keys(_p(k), k.size, _p(pre), pre.size, _p(co), _p(par), _p(o), key_bits)
    else:
        st = lib().cso_enforce_keys(_p(k), k.size, _p(pre), _p(co), _p(par), _p(o), key_bits)
    return o, int(st)


def range_count(leaves, counts, leaves_focus, focus_idx, key_bits=64, use_ref=False):
    lv = np.ascontiguousarray(leaves, np.uint64)
    lf = np.ascontiguousarray(leaves_focus, np.uint64)
    idx = np.ascontiguousarray(focus_idx, np.int32)
    out = np.zeros(lf.size - 1, np.uint32)
    cnt = np.ascontiguousarray(counts, np.uint32)
    if use_ref:
        ref().csr_range_count(_p(lv), lv.size, _p(cnt), _p(lf), lf.size, _p(idx), idx.size, _p(out), key_bits)
    else:
        lib().cso_range_count(_p(lv), lv.size, _p(cnt), _p(lf), _p(idx), idx.size, _p(out))
    return out


def node_layout(focus_leaf_counts, flags, l2i, first, last, use_ref=False):
    c = np.ascontiguousarray(focus_leaf_counts, np.uint32)
    f = np.ascontiguousarray(flags, np.uint8)
    l2 = np.ascontiguousarray(l2i, np.int32)
    out = np.zeros(c.size + 1, np.uint32)
    if use_ref:
        ref().csr_node_layout(_p(c), c.size, _p(f), f.size, _p(l2), first, last, _p(out))
    else:
        lib().cso_node_layout(_p(c), c.size, _p(f), _p(l2), first, last, _p(out))
    return out


def ijloop_density_list(x, y, z, h, m, first, last, box, nb, nc, ngmax):
    """the SPH density of the tests' ijLoop interaction over the CPU full neighbour lists (ngmax-strided rows)"""
    dt = x.dtype
    rho = np.zeros(last - first, dt)
    fn = lib().cso_ijloop_density_list_f64 if dt == np.float64 else lib().cso_ijloop_density_list_f32
    fn(_p(x), _p(y), _p(z), _p(h), _p(m), C.c_uint32(first), C.c_uint32(last), C.byref(box),
       _p(np.ascontiguousarray(nb, np.uint32)), _p(np.ascontiguousarray(nc, np.uint32)), C.c_uint(ngmax), _p(rho))
    return rho


def ijloop_density_all(x, y, z, h, m, box):
    """the same density over every pair within 2 h_i, ascending j (brute force: small n only)"""
    dt = x.dtype
    rho = np.zeros(x.size, dt)
    fn = lib().cso_ijloop_density_all_f64 if dt == np.float64 else lib().cso_ijloop_density_all_f32
    fn(_p(x), _p(y), _p(z), _p(h), _p(m), C.c_uint32(x.size), C.byref(box), _p(rho))
    return rho
