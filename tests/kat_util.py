"""Known-answer inputs from the reference's unit tests, rebuilt in Python.

OctreeMaker mirrors the reference's test helper (tree/cs_util.hpp:136-197): start from the root, divide nodes given
by their octal digit paths, and return the sorted cornerstone key array.
"""
import numpy as np


def max_level(bits):
    return 10 if bits == 32 else 21


def top(bits):
    return 1 << (3 * max_level(bits))


def pad(prefix, length, bits):
    """the reference's pad(): prefix bits shifted to the top of the 30/63 usable key bits"""
    return prefix << (3 * max_level(bits) - length)


class OctreeMaker:
    def __init__(self, bits):
        self.bits = bits
        self.keys = {0}

    def _key(self, digits):
        L = max_level(self.bits)
        return sum(int(d) << (3 * (L - 1 - i)) for i, d in enumerate(digits))

    def divide(self, *digits, level=None):
        digits = list(digits)
        if level is not None:
            digits = (digits + [0] * level)[:level]
        parent = self._key(digits)
        assert parent in self.keys, "node to be divided not present"
        for s in range(1, 8):
            self.keys.add(self._key(digits + [s]))
        return self

    def make_tree(self):
        return np.array(sorted(self.keys) + [top(self.bits)], dtype=np.uint64)


def uniform_level_tree(level, bits):
    """all 8^level nodes of one level (makeUniformNLevelTree)"""
    step = 1 << (3 * (max_level(bits) - level))
    return np.array([i * step for i in range(8 ** level + 1)], dtype=np.uint64)


def check_connectivity(t, bits):
    """every internal node's 8 children tile its key range, and parents[] points back (checkConnectivity)"""
    L = max_level(bits)
    pre = t.prefixes.astype(np.uint64)

    def decode(p):
        p = int(p)
        plen = p.bit_length() - 1
        key = (p ^ (1 << plen)) << (3 * L - plen)
        return key, key + (1 << (3 * L - plen)), plen // 3

    for i in range(t.num_nodes):
        c = int(t.child_offsets[i])
        if c == 0:
            continue
        k1, k2, lvl = decode(pre[i])
        step = (k2 - k1) // 8
        for s in range(8):
            ck1, ck2, clvl = decode(pre[c + s])
            assert ck1 == k1 + s * step and ck2 == ck1 + step and clvl == lvl + 1, (i, s)
        assert int(t.parents[(c - 1) // 8]) == i
    # every leaf is reachable and maps back
    L_ = t.num_leaves
    i2l = t.internal_to_leaf
    l2i = t.leaf_to_internal
    for leaf in range(L_):
        node = int(l2i[t.num_internal + leaf])
        assert int(i2l[node]) == leaf
        assert int(t.child_offsets[node]) == 0


def brute_force_neighbors(x, y, z, h, box_lo, box_hi, periodic):
    """all-to-all reference (test/unit/neighbors/all_to_all.hpp:25-65): PBC distance, r = 2h, j != i,
    lists sorted ascending"""
    n = x.size
    L = np.asarray(box_hi, float) - np.asarray(box_lo, float)
    out = []
    counts = np.zeros(n, np.int64)
    for i in range(n):
        d = [x - x[i], y - y[i], z - z[i]]
        if periodic:
            for k in range(3):
                d[k] = d[k] - L[k] * np.rint(d[k] * (1.0 / L[k]))
        d2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2]
        r = 2 * h[i]
        m = d2 < r * r
        m[i] = False
        idx = np.nonzero(m)[0]
        out.append(idx)
        counts[i] = idx.size
    return out, counts


def outside_leaf_box(res):
    """per sorted particle: True if it lies outside the box of the leaf that its key assigns it to (beyond a relative
    rounding margin of 1e-12), from an oracle pipeline result"""
    tree, layout = res["tree"], res["layout"]
    L = tree.num_leaves if hasattr(tree, "num_leaves") else layout.size - 1
    leaf = np.repeat(np.arange(L), np.diff(layout[: L + 1]).astype(np.int64))
    node = tree.leaf_to_internal[tree.num_internal + leaf]
    p = np.stack([res["x"], res["y"], res["z"]], axis=1)
    c, s = res["centers"][node], res["sizes"][node]
    tol = 1e-12 * (np.abs(c) + s)
    return np.any(np.abs(p - c) > s + tol, axis=1)
