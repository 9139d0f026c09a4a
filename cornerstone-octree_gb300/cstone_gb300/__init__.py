"""Python binding of libcstone_gb300.so (the C ABI in include/cstone_gb300.h) over torch CUDA tensors.

The binding is deliberately thin: every function passes device pointers, sizes and the current torch stream
straight to one C-ABI entry point and raises CsError on a non-zero status. There is no CPU path: if the shared
library is missing or fails to load, import raises.
"""
import ctypes as C
import os

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcstone_gb300.so")

MORTON, HILBERT = 0, 1
OPEN, PERIODIC, FIXED, CUBIC_OPEN = 0, 1, 2, 3
CS_OK, CS_ERR_INVALID, CS_ERR_CAPACITY, CS_ERR_CUDA, CS_ERR_TIMEOUT, CS_ERR_DEVICE = range(6)


class CsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"cstone_gb300 status {code}: {msg}")
        self.code = code


class Box(C.Structure):
    _fields_ = [("lo", C.c_double * 3), ("hi", C.c_double * 3), ("boundary", C.c_int * 3)]


def make_box(lo, hi, boundary=OPEN):
    lo = [float(v) for v in (lo if np.ndim(lo) else [lo] * 3)]
    hi = [float(v) for v in (hi if np.ndim(hi) else [hi] * 3)]
    b = list(boundary) if np.ndim(boundary) else [int(boundary)] * 3
    return Box((C.c_double * 3)(*lo), (C.c_double * 3)(*hi), (C.c_int * 3)(*b))


class OctreeView(C.Structure):
    _fields_ = [("num_leaf_nodes", C.c_int32), ("num_internal_nodes", C.c_int32), ("num_nodes", C.c_int32),
                ("prefixes", C.c_void_p), ("child_offsets", C.c_void_p), ("parents", C.c_void_p),
                ("level_range", C.c_void_p), ("internal_to_leaf", C.c_void_p), ("leaf_to_internal", C.c_void_p)]


class NsView(C.Structure):
    _fields_ = [("num_leaf_nodes", C.c_int32), ("num_nodes", C.c_int32), ("child_offsets", C.c_void_p),
                ("parents", C.c_void_p), ("internal_to_leaf", C.c_void_p), ("layout", C.c_void_p),
                ("centers", C.c_void_p), ("sizes", C.c_void_p), ("search_ext_factor", C.c_float)]


if not os.path.exists(LIB_PATH):
    raise ImportError(f"{LIB_PATH} is missing: run __graft_entry__.build() (or cornerstone-octree_gb300/build.py)")
lib = C.CDLL(LIB_PATH)
lib.cs_last_error.restype = C.c_char_p
for _name in ("cs_sort_pairs_workspace_bytes", "cs_node_counts_workspace_bytes", "cs_compute_octree_workspace_bytes",
              "cs_update_octree_workspace_bytes", "cs_build_octree_workspace_bytes"):
    getattr(lib, _name).restype = C.c_size_t
lib.cs_sort_pairs_workspace_bytes.argtypes = [C.c_size_t, C.c_int]
lib.cs_build_octree_workspace_bytes.argtypes = [C.c_int32, C.c_int]
lib.cs_compute_octree_workspace_bytes.argtypes = [C.c_int32]
lib.cs_update_octree_workspace_bytes.argtypes = [C.c_int32, C.c_int32]
lib.cs_node_counts_workspace_bytes.argtypes = [C.c_int32]


def _check(rc):
    if rc != 0:
        raise CsError(rc, lib.cs_last_error().decode())


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)


_KB = {torch.int32: 32, torch.uint32: 32, torch.int64: 64, torch.uint64: 64}
_TB = {torch.float32: "f32", torch.float64: "f64"}


def key_bits(t):
    return _KB[t.dtype]


def key_dtype(bits):
    return torch.int32 if bits == 32 else torch.int64


def max_level(bits):
    return 10 if bits == 32 else 21


# ---------------------------------------------------------------------------------------------------------------
# keys, sort, gather
# ---------------------------------------------------------------------------------------------------------------

def sfc_keys(x, y, z, box, kind=HILBERT, bits=64, keys=None, respect_remove_key=False):
    n = x.numel()
    if keys is None:
        keys = torch.empty(n, dtype=key_dtype(bits), device=x.device)
    fn = getattr(lib, f"cs_sfc_keys_{'hilbert' if kind == HILBERT else 'morton'}_u{bits}_{_TB[x.dtype]}")
    _check(fn(_stream(), _p(x), _p(y), _p(z), _p(keys), C.c_size_t(n), C.byref(box), int(respect_remove_key)))
    return keys


def sort_pairs(keys, values=None, begin_bit=0, end_bit=None, iota=True, workspace=None):
    """Stable sort in place of keys (int32/int64 tensors holding u32/u64 keys); returns (keys, values)."""
    n = keys.numel()
    bits = key_bits(keys)
    end_bit = bits if end_bit is None else end_bit
    if values is None:
        values = torch.empty(n, dtype=torch.int32, device=keys.device)
        iota = True
    kalt = torch.empty_like(keys)
    valt = torch.empty_like(values)
    ws_bytes = lib.cs_sort_pairs_workspace_bytes(n, bits)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=keys.device) if workspace is None else workspace
    fn = lib.cs_sort_pairs_u32 if bits == 32 else lib.cs_sort_pairs_u64
    _check(fn(_stream(), _p(keys), _p(values), C.c_size_t(n), _p(kalt), _p(valt), begin_bit, end_bit, int(iota),
              _p(ws), C.c_size_t(ws.numel())))
    return keys, values


def gather(perm, src):
    out = torch.empty_like(src)
    fn = lib.cs_gather_f32 if src.dtype == torch.float32 else lib.cs_gather_f64
    _check(fn(_stream(), _p(perm), _p(src), _p(out), C.c_size_t(src.numel())))
    return out


def gather4(perm, a, b, c, d):
    outs = [torch.empty_like(t) for t in (a, b, c, d)]
    fn = lib.cs_gather4_f32 if a.dtype == torch.float32 else lib.cs_gather4_f64
    _check(fn(_stream(), _p(perm), C.c_size_t(a.numel()), _p(a), _p(b), _p(c), _p(d), *[_p(o) for o in outs]))
    return outs


def neighbors_csr(nb, nc, ngmax, offsets=None, lst=None):
    """compacts ngmax-strided neighbour rows (nb: n x ngmax, nc: n) into (offsets[n + 1] int64, list int32)"""
    n = nc.numel()
    if offsets is None:
        offsets = torch.empty(n + 1, dtype=torch.int64, device=nc.device)
    if lst is None:
        total = int(nc.clamp(max=ngmax).sum()) if n else 0
        lst = torch.empty(max(total, 1), dtype=torch.int32, device=nc.device)
    lib.cs_neighbors_csr_workspace_bytes.restype = C.c_size_t
    _check(lib.cs_neighbors_csr(_stream(), _p(nb), _p(nc), C.c_size_t(n), C.c_uint(ngmax), _p(offsets), _p(lst),
                                C.c_size_t(lst.numel()), None, C.c_size_t(0)))
    return offsets, lst


# ---------------------------------------------------------------------------------------------------------------
# cornerstone leaf array
# ---------------------------------------------------------------------------------------------------------------

def node_counts(tree, keys, max_count=0xFFFFFFFF):
    L = tree.numel() - 1
    counts = torch.empty(L, dtype=torch.int32, device=tree.device)
    bits = key_bits(tree)
    fn = lib.cs_node_counts_u32 if bits == 32 else lib.cs_node_counts_u64
    _check(fn(_stream(), _p(tree), _p(counts), L, _p(keys), C.c_size_t(keys.numel()), C.c_uint32(max_count), 0,
              None, C.c_size_t(0)))
    return counts


def rebalance_decision(tree, counts, bucket):
    L = tree.numel() - 1
    ops = torch.empty(L + 1, dtype=torch.int32, device=tree.device)
    conv = torch.empty(1, dtype=torch.int32, device=tree.device)
    fn = lib.cs_rebalance_decision_u32 if key_bits(tree) == 32 else lib.cs_rebalance_decision_u64
    _check(fn(_stream(), _p(tree), _p(counts), L, C.c_uint(bucket), _p(ops), _p(conv)))
    return ops[:L], bool(conv.item())


def exclusive_scan(values, init=0, out=None):
    """exclusiveScan of int32 values (out may be values itself)"""
    out = torch.empty_like(values) if out is None else out
    _check(lib.cs_exclusive_scan_i32(_stream(), _p(values), _p(out), C.c_size_t(values.numel()), C.c_int32(init),
                                     None, C.c_size_t(0)))
    return out


def node_ops(tree, counts, bucket):
    """computeNodeOpsGpu: decision + exclusive scan; returns (scanned ops[L+1], new leaf count, converged)"""
    L = tree.numel() - 1
    ops, conv = rebalance_decision(tree, counts, bucket)
    full = torch.zeros(L + 1, dtype=torch.int32, device=tree.device)
    full[:L] = ops
    exclusive_scan(full, 0, full)
    return full, int(full[L].item()), conv


def rebalance_tree(tree, scanned_ops):
    """rebalanceTreeGpu's emission: the new leaf array (scanned_ops[L] + 1 keys)"""
    L = tree.numel() - 1
    new_tree = torch.empty(int(scanned_ops[L].item()) + 1, dtype=tree.dtype, device=tree.device)
    fn = lib.cs_rebalance_tree_u32 if key_bits(tree) == 32 else lib.cs_rebalance_tree_u64
    _check(fn(_stream(), _p(tree), L, _p(scanned_ops), _p(new_tree)))
    return new_tree


def compute_octree(keys, bucket, max_count=0xFFFFFFFF, capacity=None):
    """computeOctree: returns (tree[L+1], counts[L], layout[L+1], iterations)."""
    n = keys.numel()
    bits = key_bits(keys)
    cap = capacity or max(64, 16 * (n // max(bucket, 1)) + 4096)
    fn = lib.cs_compute_octree_u32 if bits == 32 else lib.cs_compute_octree_u64
    while True:
        tree = torch.empty(cap + 1, dtype=keys.dtype, device=keys.device)
        counts = torch.empty(cap, dtype=torch.int32, device=keys.device)
        layout = torch.empty(cap + 1, dtype=torch.int32, device=keys.device)
        L = C.c_int32()
        it = C.c_int()
        rc = fn(_stream(), _p(keys), C.c_size_t(n), C.c_uint(bucket), C.c_uint32(max_count), _p(tree), _p(counts),
                _p(layout), cap, C.byref(L), C.byref(it), None, C.c_size_t(0))
        if rc == CS_ERR_CAPACITY:
            cap = 2 * max(cap, L.value)
            continue
        _check(rc)
        return tree[: L.value + 1], counts[: L.value], layout[: L.value + 1], it.value


def update_octree(keys, bucket, tree, counts, max_count=0xFFFFFFFF, capacity=None):
    """one updateOctree step: returns (tree, counts, converged)."""
    bits = key_bits(keys)
    Lin = tree.numel() - 1
    cap = capacity or (8 * Lin + 4096)
    fn = lib.cs_update_octree_u32 if bits == 32 else lib.cs_update_octree_u64
    while True:
        tout = torch.empty(cap + 1, dtype=keys.dtype, device=keys.device)
        cout = torch.empty(cap, dtype=torch.int32, device=keys.device)
        L = C.c_int32()
        conv = C.c_int()
        rc = fn(_stream(), _p(keys), C.c_size_t(keys.numel()), C.c_uint(bucket), C.c_uint32(max_count), _p(tree),
                _p(counts), Lin, _p(tout), _p(cout), cap, C.byref(L), C.byref(conv), None, C.c_size_t(0))
        if rc == CS_ERR_CAPACITY:
            cap = 2 * max(cap, L.value)
            continue
        _check(rc)
        return tout[: L.value + 1], cout[: L.value], bool(conv.value)


class Octree:
    """Device arrays of a linked octree (cstone::OctreeData)."""

    def __init__(self, leaves):
        L = leaves.numel() - 1
        bits = key_bits(leaves)
        dev = leaves.device
        self.bits = bits
        self.leaves = leaves
        self.num_leaves = L
        self.num_internal = (L - 1) // 7
        self.num_nodes = L + self.num_internal
        N = self.num_nodes
        self.prefixes = torch.empty(N, dtype=leaves.dtype, device=dev)
        self.child_offsets = torch.empty(N + 1, dtype=torch.int32, device=dev)
        self.parents = torch.empty(max(1, (N - 1) // 8), dtype=torch.int32, device=dev)
        self.level_range = torch.empty(max_level(bits) + 2, dtype=torch.int32, device=dev)
        self.internal_to_leaf = torch.empty(N, dtype=torch.int32, device=dev)
        self.leaf_to_internal = torch.empty(N, dtype=torch.int32, device=dev)

    def view(self):
        return OctreeView(self.num_leaves, self.num_internal, self.num_nodes, self.prefixes.data_ptr(),
                          self.child_offsets.data_ptr(), self.parents.data_ptr(), self.level_range.data_ptr(),
                          self.internal_to_leaf.data_ptr(), self.leaf_to_internal.data_ptr())


def build_octree(leaves):
    o = Octree(leaves)
    fn = lib.cs_build_octree_u32 if o.bits == 32 else lib.cs_build_octree_u64
    v = o.view()
    _check(fn(_stream(), _p(leaves), o.num_leaves, C.byref(v), None, None, C.c_size_t(0)))
    return o


def geo_centers(prefixes, box, dtype=torch.float64, kind=HILBERT):
    N = prefixes.numel()
    c = torch.empty((N, 3), dtype=dtype, device=prefixes.device)
    s = torch.empty((N, 3), dtype=dtype, device=prefixes.device)
    fn = getattr(lib, f"cs_geo_centers_u{key_bits(prefixes)}_{_TB[dtype]}")
    _check(fn(_stream(), _p(prefixes), N, _p(c), _p(s), C.byref(box), kind))
    return c, s


def search_boxes(x, y, z, h, layout, first, last, scale, leaf_to_internal_leaves, node_centers, init=None):
    """computeBoundingBoxGpu for leaves [first, last). With leaf_to_internal_leaves None the boxes start from init
    (L x 3, the reference's in/out searchCenters) instead of the leaves' geometric centres."""
    L = layout.numel() - 1
    sc = torch.zeros((L, 3), dtype=x.dtype, device=x.device) if init is None else init.clone()
    ss = torch.zeros((L, 3), dtype=x.dtype, device=x.device)
    if x.dtype == torch.float32:
        _check(lib.cs_search_boxes_f32(_stream(), _p(x), _p(y), _p(z), _p(h), _p(layout), first, last,
                                       C.c_float(scale), _p(leaf_to_internal_leaves), _p(node_centers), _p(sc),
                                       _p(ss)))
    elif h.dtype == torch.float32:  # double coordinates, float h
        _check(lib.cs_search_boxes_f64_hf32(_stream(), _p(x), _p(y), _p(z), _p(h), _p(layout), first, last,
                                            C.c_float(scale), _p(leaf_to_internal_leaves), _p(node_centers), _p(sc),
                                            _p(ss)))
    else:
        _check(lib.cs_search_boxes_f64(_stream(), _p(x), _p(y), _p(z), _p(h), _p(layout), first, last,
                                       C.c_double(scale), _p(leaf_to_internal_leaves), _p(node_centers), _p(sc),
                                       _p(ss)))
    return sc, ss


def find_halos(o, node_centers, node_sizes, search_centers, search_sizes, box, first, last, flags=None):
    if flags is None:
        flags = torch.zeros(o.num_nodes, dtype=torch.uint8, device=o.prefixes.device)
    fn = getattr(lib, f"cs_find_halos_u{o.bits}_{_TB[node_centers.dtype]}")
    _check(fn(_stream(), _p(o.prefixes), _p(o.child_offsets), _p(o.parents), _p(node_centers), _p(node_sizes),
              _p(o.leaves), _p(search_centers), _p(search_sizes), C.byref(box), first, last, _p(flags)))
    return flags


def ns_view(o, layout, centers, sizes, search_ext=1.0):
    return NsView(o.num_leaves, o.num_nodes, o.child_offsets.data_ptr(), o.parents.data_ptr(),
                  o.internal_to_leaf.data_ptr(), layout.data_ptr(), centers.data_ptr(), sizes.data_ptr(),
                  float(search_ext))


def find_neighbors(x, y, z, h, first, last, box, o, layout, centers, sizes, ngmax, search_ext=1.0, out=None):
    n = last - first
    if out is None:
        nb = torch.empty((n, ngmax), dtype=torch.int32, device=x.device)
        nc = torch.empty(n, dtype=torch.int32, device=x.device)
    else:
        nb, nc = out
    v = ns_view(o, layout, centers, sizes, search_ext)
    fn = lib.cs_find_neighbors_f32 if x.dtype == torch.float32 else lib.cs_find_neighbors_f64
    if x.dtype == torch.float64 and h.dtype == torch.float32:  # double coordinates, float h
        fn = lib.cs_find_neighbors_f64_hf32
    _check(fn(_stream(), _p(x), _p(y), _p(z), _p(h), C.c_uint32(first), C.c_uint32(last), C.byref(box),
              C.byref(v), C.c_uint(ngmax), _p(nb), _p(nc)))
    return nb, nc


# ---------------------------------------------------------------------------------------------------------------
# whole path (cs_pipeline_*)
# ---------------------------------------------------------------------------------------------------------------

class PipelineConfig(C.Structure):
    _fields_ = [("sfc_kind", C.c_int), ("bucket_size", C.c_uint), ("max_count", C.c_uint32), ("ngmax", C.c_uint),
                ("search_ext", C.c_float), ("halo_search_ext", C.c_float), ("do_halos", C.c_int),
                ("do_neighbors", C.c_int)]


class PipelineResult(C.Structure):
    _fields_ = [("num_leaves", C.c_int32), ("num_nodes", C.c_int32), ("iterations", C.c_int32),
                ("focus_first", C.c_int32), ("focus_last", C.c_int32), ("max_depth", C.c_int32)]


class PipelineOutputs(C.Structure):
    _fields_ = [("sorted_keys", C.c_void_p), ("order", C.c_void_p), ("x", C.c_void_p), ("y", C.c_void_p),
                ("z", C.c_void_p), ("h", C.c_void_p), ("leaves", C.c_void_p), ("counts", C.c_void_p),
                ("layout", C.c_void_p), ("octree", OctreeView), ("centers", C.c_void_p), ("sizes", C.c_void_p),
                ("halo_flags", C.c_void_p), ("neighbors", C.c_void_p), ("neighbor_counts", C.c_void_p),
                ("search_centers", C.c_void_p), ("search_sizes", C.c_void_p)]


lib.cs_pipeline_device_bytes.restype = C.c_size_t
lib.cs_pipeline_device_bytes.argtypes = [C.c_void_p]


class Tuning(C.Structure):
    """speed knobs (results do not depend on them): targets per warp of the neighbour traversal (32, 16, 8), its
    by-target switch cost (0: never), and the key sort's keys per thread (16 or 12)"""
    _fields_ = [("nb_group", C.c_int), ("nb_by_target_cost", C.c_int), ("sort_items", C.c_int)]

    def as_dict(self):
        return {"nb_group": self.nb_group, "nb_by_target_cost": self.nb_by_target_cost,
                "sort_items": self.sort_items or 16}


def tuning_label(t):
    """'32/7/s16': targets per warp / by-target cost / sort keys per thread"""
    return f"{t['nb_group']}/{t['nb_by_target_cost']}/s{t.get('sort_items', 16)}"


lib.cs_pipeline_autotune.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                     C.c_void_p]

STAGES = ("keys", "sort", "gather", "build", "link", "geometry", "nbprep", "halos", "neighbors")
COPY_TIMES = ("compaction", "list_copy", "list_copy_wait", "run_start_to_lists_on_host")


class Pipeline:
    """keys -> sort -> gather -> computeOctree -> link -> geometry -> findHalos -> findNeighbors, device resident."""

    def __init__(self, coord_bits=64, key_bits=64, kind=HILBERT, bucket=64, ngmax=200, search_ext=1.0,
                 halo_search_ext=1.0, do_halos=True, do_neighbors=True, max_count=0xFFFFFFFF):
        self.cfg = PipelineConfig(kind, bucket, max_count, ngmax, search_ext, halo_search_ext, int(do_halos),
                                  int(do_neighbors))
        self.coord_bits, self.key_bits = coord_bits, key_bits
        self.handle = C.c_void_p()
        _check(lib.cs_pipeline_create(C.byref(self.handle), coord_bits, key_bits, C.byref(self.cfg)))
        self.result = PipelineResult()

    def __del__(self):
        if getattr(self, "handle", None):
            lib.cs_pipeline_destroy(self.handle)
            self.handle = None

    def run(self, x, y, z, h, box, focus=(0, 0)):
        self._n = x.numel()
        _check(lib.cs_pipeline_run(self.handle, _stream(), _p(x), _p(y), _p(z), _p(h), C.c_size_t(x.numel()),
                                   C.byref(box), C.c_uint64(focus[0]), C.c_uint64(focus[1]), C.byref(self.result)))
        return self.result

    def run_host(self, x, y, z, h, box, focus=(0, 0), nc_out=None, flags_out=None):
        """x..h: pinned (or pageable) host torch tensors; nc_out/flags_out host tensors or None."""
        fcap = flags_out.numel() if flags_out is not None else 0
        self._n = x.numel()
        _check(lib.cs_pipeline_run_host(self.handle, _stream(), _p(x), _p(y), _p(z), _p(h), C.c_size_t(x.numel()),
                                        C.byref(box), C.c_uint64(focus[0]), C.c_uint64(focus[1]), _p(nc_out),
                                        _p(flags_out), C.c_size_t(fcap), C.byref(self.result)))
        return self.result

    def run_host_async(self, x, y, z, h, box, focus=(0, 0), nc_out=None, flags_out=None):
        """as run_host, returning once enqueued; the next call's input copies overlap this run. Keep x..h unchanged
        and nc_out / flags_out unread until wait()."""
        fcap = flags_out.numel() if flags_out is not None else 0
        self._n = x.numel()
        _check(lib.cs_pipeline_run_host_async(self.handle, _stream(), _p(x), _p(y), _p(z), _p(h),
                                              C.c_size_t(x.numel()), C.byref(box), C.c_uint64(focus[0]),
                                              C.c_uint64(focus[1]), _p(nc_out), _p(flags_out), C.c_size_t(fcap),
                                              C.byref(self.result)))
        return self.result

    def run_host_csr(self, x, y, z, h, box, focus, offsets_out, list_out, nc_out=None, flags_out=None,
                     asynchronous=False):
        """as run_host / run_host_async, with the neighbour lists returned as CSR into pinned host tensors:
        offsets_out (int64, n + 1), list_out (int32, capacity); row i = list_out[offsets_out[i]:offsets_out[i+1]]"""
        fcap = flags_out.numel() if flags_out is not None else 0
        self._n = x.numel()
        fn = lib.cs_pipeline_run_host_csr_async if asynchronous else lib.cs_pipeline_run_host_csr
        _check(fn(self.handle, _stream(), _p(x), _p(y), _p(z), _p(h), C.c_size_t(x.numel()), C.byref(box),
                  C.c_uint64(focus[0]), C.c_uint64(focus[1]), _p(nc_out), _p(flags_out), C.c_size_t(fcap),
                  _p(offsets_out), _p(list_out), C.c_size_t(list_out.numel()), C.byref(self.result)))
        return self.result

    def wait(self):
        _check(lib.cs_pipeline_wait(self.handle))

    def step(self, x, y, z, h, box, use_graph=True):
        """one incremental time step (the first of a sequence builds from the root); device tensors"""
        self._n = x.numel()
        _check(lib.cs_pipeline_step(self.handle, _stream(), _p(x), _p(y), _p(z), _p(h), C.c_size_t(x.numel()),
                                    C.byref(box), int(use_graph), C.byref(self.result)))
        return self.result

    def reset_steps(self):
        _check(lib.cs_pipeline_reset_steps(self.handle))

    def graph_replays(self):
        return lib.cs_pipeline_graph_replays(self.handle)

    def stage_times(self):
        ms = (C.c_float * len(STAGES))()
        _check(lib.cs_pipeline_stage_times(self.handle, ms, len(STAGES)))
        return dict(zip(STAGES, list(ms)))

    def copy_times(self):
        """device ms of the last copy-back that returned neighbour lists: the compaction, the list copy to host
        memory, the copy's wait for the previous call's copy, and the run's start to the end of its list copy"""
        ms = (C.c_float * len(COPY_TIMES))()
        _check(lib.cs_pipeline_copy_times(self.handle, ms, len(COPY_TIMES)))
        return dict(zip(COPY_TIMES, list(ms)))

    def set_tuning(self, nb_group=32, nb_by_target_cost=7, sort_items=16):
        t = Tuning(nb_group, nb_by_target_cost, sort_items)
        _check(lib.cs_pipeline_set_tuning(self.handle, C.byref(t)))

    def get_tuning(self):
        t = Tuning()
        _check(lib.cs_pipeline_get_tuning(self.handle, C.byref(t)))
        return t.as_dict()

    def autotune(self, reps=2):
        """reruns the last run's inputs for each candidate tuning (traversal candidates timed on the neighbour stage,
        then sort tile shapes on the sort stage) and keeps the fastest; returns
        {"best": tuning, "tried": [(tuning, ms), ...]}"""
        cap = 16
        best, tried, ms, count = Tuning(), (Tuning * cap)(), (C.c_float * cap)(), C.c_int()
        _check(lib.cs_pipeline_autotune(self.handle, _stream(), int(reps), C.byref(best), tried, ms, cap,
                                        C.byref(count)))
        return {"best": best.as_dict(), "tried": [(tried[k].as_dict(), float(ms[k])) for k in range(count.value)]}

    def device_bytes(self):
        return lib.cs_pipeline_device_bytes(self.handle)

    def outputs(self):
        """torch views of the device results of the last run (no copies)."""
        o = PipelineOutputs()
        _check(lib.cs_pipeline_get_outputs(self.handle, C.byref(o)))
        r = self.result
        n = self._n
        tdt = torch.float64 if self.coord_bits == 64 else torch.float32
        kdt = key_dtype(self.key_bits)
        L, N = r.num_leaves, r.num_nodes
        out = dict(sorted_keys=_wrap(o.sorted_keys, n, kdt), order=_wrap(o.order, n, torch.int32),
                   x=_wrap(o.x, n, tdt), y=_wrap(o.y, n, tdt), z=_wrap(o.z, n, tdt), h=_wrap(o.h, n, tdt),
                   leaves=_wrap(o.leaves, L + 1, kdt), counts=_wrap(o.counts, L, torch.int32),
                   layout=_wrap(o.layout, L + 1, torch.int32), prefixes=_wrap(o.octree.prefixes, N, kdt),
                   child_offsets=_wrap(o.octree.child_offsets, N, torch.int32),
                   parents=_wrap(o.octree.parents, max(1, (N - 1) // 8), torch.int32),
                   level_range=_wrap(o.octree.level_range, max_level(self.key_bits) + 2, torch.int32),
                   internal_to_leaf=_wrap(o.octree.internal_to_leaf, N, torch.int32),
                   leaf_to_internal=_wrap(o.octree.leaf_to_internal, N, torch.int32),
                   centers=_wrap(o.centers, 3 * N, tdt).view(N, 3), sizes=_wrap(o.sizes, 3 * N, tdt).view(N, 3),
                   halo_flags=_wrap(o.halo_flags, N, torch.uint8),
                   neighbor_counts=_wrap(o.neighbor_counts, n, torch.int32))
        if o.neighbors:
            out["neighbors"] = _wrap(o.neighbors, n * self.cfg.ngmax, torch.int32).view(n, self.cfg.ngmax)
        if o.search_centers and r.focus_last > r.focus_first:
            out["search_centers"] = _wrap(o.search_centers, 3 * L, tdt).view(L, 3)
            out["search_sizes"] = _wrap(o.search_sizes, 3 * L, tdt).view(L, 3)
        return out


# ---------------------------------------------------------------------------------------------------------------
# many independent sets (cs_batch_*)
# ---------------------------------------------------------------------------------------------------------------

class BatchConfig(C.Structure):
    _fields_ = [("coord_bits", C.c_int), ("sfc_kind", C.c_int), ("ngmax", C.c_uint), ("search_ext", C.c_float),
                ("do_neighbors", C.c_int)]


class BatchResult(C.Structure):
    _fields_ = [("num_sets", C.c_int32), ("num_leaves", C.c_int32), ("num_nodes", C.c_int32),
                ("iterations", C.c_int32), ("num_particles", C.c_uint64)]


class BatchOutputs(C.Structure):
    _fields_ = [("order", C.c_void_p), ("x", C.c_void_p), ("y", C.c_void_p), ("z", C.c_void_p), ("h", C.c_void_p),
                ("leaves", C.c_void_p), ("counts", C.c_void_p), ("layout", C.c_void_p),
                ("set_leaf_begin", C.c_void_p), ("set_roots", C.c_void_p), ("set_offsets", C.c_void_p),
                ("octree", OctreeView), ("centers", C.c_void_p), ("sizes", C.c_void_p), ("neighbors", C.c_void_p),
                ("neighbor_counts", C.c_void_p)]


lib.cs_batch_device_bytes.restype = C.c_size_t
lib.cs_batch_device_bytes.argtypes = [C.c_void_p]


class Batch:
    """many independent sets: keys -> segmented sort -> one build of every set -> link -> geometry -> neighbours"""

    def __init__(self, coord_bits=32, kind=MORTON, ngmax=100, search_ext=1.0, do_neighbors=True):
        self.cfg = BatchConfig(coord_bits, kind, ngmax, search_ext, int(do_neighbors))
        self.coord_bits = coord_bits
        self.handle = C.c_void_p()
        _check(lib.cs_batch_create(C.byref(self.handle), C.byref(self.cfg)))
        self.result = BatchResult()

    def __del__(self):
        if getattr(self, "handle", None):
            lib.cs_batch_destroy(self.handle)
            self.handle = None

    def set_tuning(self, nb_group=32, nb_by_target_cost=7, sort_items=16):
        t = Tuning(nb_group, nb_by_target_cost, sort_items)
        _check(lib.cs_batch_set_tuning(self.handle, C.byref(t)))

    def run(self, x, y, z, h, offsets, boxes, buckets):
        """x..h: device tensors of all sets concatenated; offsets: S + 1 ints; boxes: S cs_box; buckets: S ints"""
        S = len(boxes)
        off = (C.c_uint32 * (S + 1))(*[int(v) for v in offsets])
        bx = (Box * S)(*boxes)
        bk = (C.c_uint32 * S)(*[int(v) for v in buckets])
        _check(lib.cs_batch_run(self.handle, _stream(), _p(x), _p(y), _p(z), _p(h), off, S, bx, bk,
                                C.byref(self.result)))
        return self.result

    def device_bytes(self):
        return lib.cs_batch_device_bytes(self.handle)

    def outputs(self):
        """torch views of the device results of the last run (no copies)"""
        o = BatchOutputs()
        _check(lib.cs_batch_get_outputs(self.handle, C.byref(o)))
        r = self.result
        n, L, N, S = int(r.num_particles), r.num_leaves, r.num_nodes, r.num_sets
        tdt = torch.float64 if self.coord_bits == 64 else torch.float32
        out = dict(order=_wrap(o.order, n, torch.int32), x=_wrap(o.x, n, tdt), y=_wrap(o.y, n, tdt),
                   z=_wrap(o.z, n, tdt), h=_wrap(o.h, n, tdt), leaves=_wrap(o.leaves, L + 1, torch.int64),
                   counts=_wrap(o.counts, L, torch.int32), layout=_wrap(o.layout, L + 1, torch.int32),
                   set_leaf_begin=_wrap(o.set_leaf_begin, S + 1, torch.int32),
                   set_roots=_wrap(o.set_roots, S, torch.int32), set_offsets=_wrap(o.set_offsets, S + 1, torch.int32),
                   prefixes=_wrap(o.octree.prefixes, N, torch.int64),
                   centers=_wrap(o.centers, 3 * N, tdt).view(N, 3), sizes=_wrap(o.sizes, 3 * N, tdt).view(N, 3),
                   neighbor_counts=_wrap(o.neighbor_counts, n, torch.int32))
        if o.neighbors:
            out["neighbors"] = _wrap(o.neighbors, n * self.cfg.ngmax, torch.int32).view(n, self.cfg.ngmax)
        return out


# ---------------------------------------------------------------------------------------------------------------
# request server (cs_server_*)
# ---------------------------------------------------------------------------------------------------------------

REQ_BUILD, REQ_UPDATE = 0, 1


class ServerConfig(C.Structure):
    _fields_ = [("num_slots", C.c_int), ("hbm_budget_bytes", C.c_uint64), ("coord_bits", C.c_int),
                ("key_bits", C.c_int), ("pipeline", PipelineConfig)]


class Request(C.Structure):
    _fields_ = [("kind", C.c_int), ("tree", C.c_int32), ("x", C.c_void_p), ("y", C.c_void_p), ("z", C.c_void_p),
                ("h", C.c_void_p), ("n", C.c_size_t), ("box", Box)]


class RequestResult(C.Structure):
    _fields_ = [("id", C.c_uint64), ("status", C.c_int), ("num_leaves", C.c_int32),
                ("neighbor_checksum", C.c_uint64), ("queued_ms", C.c_double), ("run_ms", C.c_double),
                ("latency_ms", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("completed", C.c_uint64), ("failed", C.c_uint64), ("particles", C.c_uint64),
                ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("elapsed_s", C.c_double),
                ("device_bytes", C.c_uint64), ("resident_trees", C.c_int)]


class Server:
    """continuous batching of build / update requests from host arrays (numpy) on the current GPU"""

    def __init__(self, num_slots, budget_bytes, coord_bits=64, key_bits=64, kind=HILBERT, bucket=64, ngmax=200,
                 search_ext=1.0):
        pc = PipelineConfig(kind, bucket, 0xFFFFFFFF, ngmax, search_ext, 1.0, 0, 1)
        self.cfg = ServerConfig(num_slots, int(budget_bytes), coord_bits, key_bits, pc)
        self.handle = C.c_void_p()
        _check(lib.cs_server_create(C.byref(self.handle), C.byref(self.cfg)))
        self._inputs = {}  # keeps each request's host arrays alive until it is waited for

    def submit(self, x, y, z, h, box, kind=REQ_BUILD, tree=-1):
        import numpy as np

        arrs = [np.ascontiguousarray(a) for a in (x, y, z, h)]
        req = Request(kind, tree, *[a.ctypes.data for a in arrs], arrs[0].size, box)
        rid = C.c_uint64()
        _check(lib.cs_server_submit(self.handle, C.byref(req), C.byref(rid)))
        self._inputs[rid.value] = arrs
        return rid.value

    def wait(self, rid, counts=True):
        """(RequestResult, neighbour counts as a numpy array or None); raises on a failed request"""
        import numpy as np

        arrs = self._inputs.get(rid)
        nc = np.empty(arrs[0].size, np.uint32) if counts and arrs is not None else None
        res = RequestResult()
        rc = lib.cs_server_wait(self.handle, C.c_uint64(rid), C.byref(res),
                                nc.ctypes.data_as(C.c_void_p) if nc is not None else None)
        self._inputs.pop(rid, None)
        if rc != 0:
            raise CsError(rc, f"request {rid} failed")
        return res, nc

    def stats(self):
        st = ServerStats()
        _check(lib.cs_server_get_stats(self.handle, C.byref(st)))
        return st

    def release_tree(self, tree):
        _check(lib.cs_server_release_tree(self.handle, tree))

    def close(self):
        if getattr(self, "handle", None):
            lib.cs_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        self.close()


def _wrap(ptr, count, dtype):
    """non-owning torch view of device memory held by the library"""
    if count == 0 or not ptr:
        return torch.empty(0, dtype=dtype, device="cuda")
    nbytes = count * torch.empty(0, dtype=dtype).element_size()
    arr = _CudaArray(ptr, nbytes)
    t = torch.as_tensor(arr, device="cuda").view(torch.uint8)[:nbytes]
    return t.view(dtype)


class _CudaArray:
    """exposes a raw device pointer through __cuda_array_interface__ so torch can view it"""

    def __init__(self, ptr, nbytes):
        self.__cuda_array_interface__ = {"shape": (nbytes,), "typestr": "|u1", "data": (int(ptr), False),
                                         "version": 3}



# ---------------------------------------------------------------------------------------------------------------
# around the path: upsweeps, source centres, target groups, SFC gaps, focus tree
# ---------------------------------------------------------------------------------------------------------------

for _name in ("cs_upsweep_workspace_bytes", "cs_group_splits_workspace_bytes", "cs_spanning_tree_workspace_bytes",
              "cs_node_layout_workspace_bytes", "cs_neighbors_csr_workspace_bytes"):
    getattr(lib, _name).restype = C.c_size_t


def _host_i32(a):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.int32))
    return a, a.ctypes.data_as(C.c_void_p)


def upsweep_sum(child_offsets, node_counts, parents=None, level_range=None):
    """upsweepSumGpu in place on node_counts (uint32 as int32, leaf values set): one launch with parents, else level by
    level from level_range (host array)"""
    n = child_offsets.numel()
    lr, lrp = _host_i32(level_range if level_range is not None else [0])
    nl = lr.size - 1 if level_range is not None else 0
    _check(lib.cs_upsweep_sum(_stream(), nl, lrp if level_range is not None else None, _p(child_offsets),
                              _p(parents), n, _p(node_counts), None, C.c_size_t(0)))
    return node_counts


def leaf_source_centers(x, y, z, m, leaf_to_internal_leaves, layout, centers):
    """mass centres of the leaves into centers[num_nodes, 4] (f64 coordinates with f64 or f32 masses, or all f32)"""
    if x.dtype == torch.float64:
        fn = lib.cs_leaf_source_centers_f64 if m.dtype == torch.float64 else lib.cs_leaf_source_centers_f64_m32
    else:
        fn = lib.cs_leaf_source_centers_f32
    _check(fn(_stream(), _p(x), _p(y), _p(z), _p(m), _p(leaf_to_internal_leaves), leaf_to_internal_leaves.numel(),
              _p(layout), _p(centers)))
    return centers


def upsweep_source_centers(child_offsets, centers, parents=None, level_range=None):
    n = child_offsets.numel()
    lr, lrp = _host_i32(level_range if level_range is not None else [0])
    nl = lr.size - 1 if level_range is not None else 0
    fn = lib.cs_upsweep_source_centers_f64 if centers.dtype == torch.float64 else lib.cs_upsweep_source_centers_f32
    _check(fn(_stream(), nl, lrp if level_range is not None else None, _p(child_offsets), _p(parents), n,
              _p(centers), None, C.c_size_t(0)))
    return centers


def group_splits(first, last, x, y, z, h, leaves, layout, box, group_size=32, tol=8.0):
    """computeGroupSplits: returns the group boundaries (num_groups + 1 int32 device tensor)"""
    cap = 2 * ((last - first) // group_size + 2)
    fn = lib.cs_group_splits_f64 if x.dtype == torch.float64 else lib.cs_group_splits_f32
    while True:
        groups = torch.empty(cap, dtype=torch.int32, device=x.device)
        ng = C.c_uint32()
        rc = fn(_stream(), C.c_uint32(first), C.c_uint32(last), _p(x), _p(y), _p(z), _p(h), _p(leaves),
                leaves.numel() - 1, _p(layout), C.byref(box), C.c_uint(group_size), C.c_float(tol), _p(groups),
                C.c_size_t(cap), C.byref(ng), None, C.c_size_t(0))
        if rc == CS_ERR_CAPACITY:
            cap = ng.value + 1
            continue
        _check(rc)
        return groups[: ng.value + 1]


def spanning_tree(keys):
    """computeSpanningTree of sorted keys (first 0, last nodeRange(0)); int32/int64 tensors hold u32/u64 keys"""
    bits = key_bits(keys)
    fn = lib.cs_spanning_tree_u32 if bits == 32 else lib.cs_spanning_tree_u64
    cap = 8 * keys.numel() + 64
    while True:
        out = torch.empty(cap, dtype=keys.dtype, device=keys.device)
        size = C.c_int32()
        rc = fn(_stream(), _p(keys), keys.numel(), _p(out), cap, C.byref(size), None, C.c_size_t(0))
        if rc == CS_ERR_CAPACITY:
            cap = size.value
            continue
        _check(rc)
        return out[: size.value]


def count_sfc_gaps(tree):
    bits = key_bits(tree)
    ops = torch.empty(tree.numel(), dtype=torch.int32, device=tree.device)
    fn = lib.cs_count_sfc_gaps_u32 if bits == 32 else lib.cs_count_sfc_gaps_u64
    _check(fn(_stream(), _p(tree), tree.numel() - 1, _p(ops)))
    return ops[: tree.numel() - 1]


def fill_sfc_gaps(tree, scanned_ops):
    bits = key_bits(tree)
    out = torch.empty(int(scanned_ops[-1]) + 1, dtype=tree.dtype, device=tree.device)
    fn = lib.cs_fill_sfc_gaps_u32 if bits == 32 else lib.cs_fill_sfc_gaps_u64
    _check(fn(_stream(), _p(tree), tree.numel() - 1, _p(scanned_ops), _p(out)))
    return out


def _kf(bits, name):
    return getattr(lib, f"{name}_u{bits}")


def rebalance_decision_essential(prefixes, child_offsets, parents, counts, macs, focus, bucket):
    bits = key_bits(prefixes)
    n = prefixes.numel()
    ops = torch.empty(n, dtype=torch.int32, device=prefixes.device)
    kt = C.c_uint32 if bits == 32 else C.c_uint64
    _check(_kf(bits, "cs_rebalance_decision_essential")(_stream(), _p(prefixes), _p(child_offsets), _p(parents),
                                                        _p(counts), _p(macs), kt(focus[0]), kt(focus[1]),
                                                        C.c_uint(bucket), _p(ops), n))
    return ops


def mac_refine_decision(prefixes, macs, leaf_to_internal_leaves, focus_first, focus_last):
    bits = key_bits(prefixes)
    L = leaf_to_internal_leaves.numel()
    ops = torch.empty(L, dtype=torch.int32, device=prefixes.device)
    _check(_kf(bits, "cs_mac_refine_decision")(_stream(), _p(prefixes), _p(macs), _p(leaf_to_internal_leaves), L,
                                               focus_first, focus_last, _p(ops)))
    return ops


def protect_ancestors(prefixes, parents, ops):
    """in place on ops; returns converged (no op differs from 1)"""
    bits = key_bits(prefixes)
    changed = torch.zeros(1, dtype=torch.int32, device=prefixes.device)
    conv = C.c_int()
    _check(_kf(bits, "cs_protect_ancestors")(_stream(), _p(prefixes), _p(parents), _p(ops), prefixes.numel(),
                                             _p(changed), C.byref(conv)))
    return bool(conv.value)


def enforce_keys(forced_keys, prefixes, child_offsets, parents, ops):
    """in place on ops; returns the status (0 converged, 1 cancelMerge, 2 rebalance, 3 failed)"""
    bits = key_bits(prefixes)
    sdev = torch.zeros(1, dtype=torch.int32, device=prefixes.device)
    st = C.c_int()
    _check(_kf(bits, "cs_enforce_keys")(_stream(), _p(forced_keys), forced_keys.numel(), _p(prefixes),
                                        _p(child_offsets), _p(parents), _p(ops), _p(sdev), C.byref(st)))
    return st.value


def range_count(leaves, counts, leaves_focus, focus_idx, counts_focus=None):
    bits = key_bits(leaves)
    if counts_focus is None:
        counts_focus = torch.zeros(leaves_focus.numel() - 1, dtype=torch.int32, device=leaves.device)
    _check(_kf(bits, "cs_range_count")(_stream(), _p(leaves), leaves.numel(), _p(counts), _p(leaves_focus),
                                       _p(focus_idx), focus_idx.numel(), _p(counts_focus)))
    return counts_focus


def node_layout(focus_leaf_counts, flags, leaf_to_internal_leaves, first, last):
    L = focus_leaf_counts.numel()
    out = torch.empty(L + 1, dtype=torch.int32, device=focus_leaf_counts.device)
    _check(lib.cs_node_layout(_stream(), _p(focus_leaf_counts), L, _p(flags), _p(leaf_to_internal_leaves), first,
                              last, _p(out), None, C.c_size_t(0)))
    return out


# ---------------------------------------------------------------------------------------------------------------
# neighbour-list consumers (ijLoop with an SPH density interaction)
# ---------------------------------------------------------------------------------------------------------------

lib.cs_cluster_nblist_workspace_bytes.restype = C.c_size_t


def _ns_view(tree, layout, centers, sizes, search_ext=1.0):
    return NsView(tree.num_leaves, tree.num_nodes, C.c_void_p(tree.child_offsets.data_ptr()),
                  C.c_void_p(tree.parents.data_ptr()), C.c_void_p(tree.internal_to_leaf.data_ptr()),
                  C.c_void_p(layout.data_ptr()), C.c_void_p(centers.data_ptr()), C.c_void_p(sizes.data_ptr()),
                  search_ext)


def ijloop_density_list(x, y, z, h, m, box, nb, nc, first=0, last=None):
    """density over the ngmax-strided neighbour rows nb (n x ngmax) with counts nc"""
    last = x.numel() if last is None else last
    rho = torch.empty(last - first, dtype=x.dtype, device=x.device)
    fn = lib.cs_ijloop_density_list_f64 if x.dtype == torch.float64 else lib.cs_ijloop_density_list_f32
    _check(fn(_stream(), _p(x), _p(y), _p(z), _p(h), _p(m), C.c_uint32(first), C.c_uint32(last), C.byref(box),
              _p(nb), _p(nc), C.c_uint(nb.shape[1]), _p(rho)))
    return rho


def cluster_nblist(x, y, z, h, box, tree, layout, centers, sizes, key_bits=64, ncmax=256):
    """cluster-pair lists: (lists[n_icl, ncmax], counts[n_icl]); ncmax grows to the largest count when needed"""
    n = x.numel()
    nic = (n + 7) // 8
    view = _ns_view(tree, layout, centers, sizes)
    fn = lib.cs_cluster_nblist_build_f64 if x.dtype == torch.float64 else lib.cs_cluster_nblist_build_f32
    while True:
        lists = torch.empty((nic, ncmax), dtype=torch.int32, device=x.device)
        counts = torch.empty(nic, dtype=torch.int32, device=x.device)
        mx = C.c_int()
        rc = fn(_stream(), _p(x), _p(y), _p(z), _p(h), C.c_size_t(n), C.byref(view), C.byref(box), key_bits,
                C.c_uint(ncmax), _p(lists), _p(counts), None, C.c_size_t(0), C.byref(mx))
        if rc == CS_ERR_CAPACITY:
            ncmax = mx.value
            need = nic * ncmax * 4
            free, _ = torch.cuda.mem_get_info(x.device)
            if need > free:
                raise CsError(CS_ERR_CAPACITY, f"cluster lists: the longest list needs ncmax = {ncmax}, "
                                               f"{need / 2 ** 30:.1f} GiB for {nic} i-clusters ({free / 2 ** 30:.1f} "
                                               f"GiB free)")
            continue
        _check(rc)
        return lists, counts


def ijloop_density_clusters(x, y, z, h, m, lists, counts):
    rho = torch.empty_like(x)
    fn = lib.cs_ijloop_density_clusters_f64 if x.dtype == torch.float64 else lib.cs_ijloop_density_clusters_f32
    _check(fn(_stream(), _p(x), _p(y), _p(z), _p(h), _p(m), C.c_size_t(x.numel()), _p(lists), _p(counts),
              C.c_uint(lists.shape[1]), _p(rho)))
    return rho
