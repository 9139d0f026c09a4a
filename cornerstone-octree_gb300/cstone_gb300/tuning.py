"""Tuning table of the neighbour traversal and the key sort: the autotuner's choices (``Pipeline.autotune``) keyed by coordinate
width, key width, particle count (power of two, rounded) and device name, stored as JSON. A tuning only changes the
speed of a pipeline, never its results."""
import json
import math
import os

DEFAULT = {"nb_group": 32, "nb_by_target_cost": 7, "sort_items": 16}
FIELDS = ("nb_group", "nb_by_target_cost", "sort_items")


def tuning_key(coord_bits, key_bits, n, device):
    """e.g. 'f64/u64/n2^24/NVIDIA GB300'"""
    return f"f{coord_bits}/u{key_bits}/n2^{int(round(math.log2(max(int(n), 1))))}/{device}"


class TuningTable:
    def __init__(self, path=None):
        self.path = path
        self.entries = {}
        if path and os.path.exists(path):
            with open(path) as f:
                data = json.load(f)
            for key, e in data.get("entries", {}).items():
                # entries written before the sort shape was a knob take the default shape
                self.entries[key] = {f: int(e.get(f, DEFAULT[f])) for f in FIELDS}
                self.entries[key]["ms"] = e.get("ms")

    def lookup(self, key):
        e = self.entries.get(key)
        return None if e is None else {f: e[f] for f in FIELDS}

    def store(self, key, tuning, ms=None):
        self.entries[key] = {f: int(tuning.get(f, DEFAULT[f])) for f in FIELDS}
        self.entries[key]["ms"] = ms

    def save(self, path=None):
        path = path or self.path
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump({"version": 1, "entries": self.entries}, f, indent=1, sort_keys=True)
        os.replace(tmp, path)


def tune_pipeline(pipe, table, key, reps=2):
    """Apply the table's tuning for key to pipe, or (no entry) autotune pipe on its last run's inputs and record the
    choice. Returns (tuning, tried or None)."""
    t = table.lookup(key)
    if t is not None:
        pipe.set_tuning(**t)
        return t, None
    r = pipe.autotune(reps)
    ms = dict((f"{c['nb_group']}/{c['nb_by_target_cost']}/s{c['sort_items']}", m) for c, m in r["tried"])
    table.store(key, r["best"], ms)
    return r["best"], r["tried"]
