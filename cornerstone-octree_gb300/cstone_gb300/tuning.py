"""Tuning table of the neighbour traversal: the autotuner's choices (``Pipeline.autotune``) keyed by coordinate
width, key width, particle count (power of two, rounded) and device name, stored as JSON. A tuning only changes the
speed of a pipeline, never its results."""
import json
import math
import os

DEFAULT = {"nb_group": 32, "nb_by_target_cost": 7}


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
                self.entries[key] = {"nb_group": int(e["nb_group"]), "nb_by_target_cost": int(e["nb_by_target_cost"]),
                                     "ms": e.get("ms")}

    def lookup(self, key):
        e = self.entries.get(key)
        return None if e is None else {"nb_group": e["nb_group"], "nb_by_target_cost": e["nb_by_target_cost"]}

    def store(self, key, tuning, ms=None):
        self.entries[key] = {"nb_group": int(tuning["nb_group"]), "nb_by_target_cost": int(tuning["nb_by_target_cost"]),
                             "ms": ms}

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
    ms = dict((f"{c['nb_group']}/{c['nb_by_target_cost']}", m) for c, m in r["tried"])
    table.store(key, r["best"], ms)
    return r["best"], r["tried"]
