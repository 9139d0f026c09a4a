"""The tuning table (JSON) of the autotuner: keys, round trip through a file, lookup of missing entries; and the
tuning entry points exported by the library (no GPU needed)."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "cornerstone-octree_gb300"))

from cstone_gb300 import tuning  # noqa: E402


def test_keys_round_the_count_to_a_power_of_two():
    assert tuning.tuning_key(64, 64, 1 << 24, "GB300") == "f64/u64/n2^24/GB300"
    assert tuning.tuning_key(32, 32, 3_000_000, "GB300") == "f32/u32/n2^22/GB300"
    assert tuning.tuning_key(32, 64, 0, "x") == "f32/u64/n2^0/x"


def test_table_round_trip(tmp_path):
    path = str(tmp_path / "tuning.json")
    t = tuning.TuningTable(path)
    assert t.lookup("f64/u64/n2^24/GB300") is None
    t.store("f64/u64/n2^24/GB300", {"nb_group": 32, "nb_by_target_cost": 7, "sort_items": 12},
            {"32/7/s16": 18.9, "16/7/s16": 25.0})
    t.store("f32/u32/n2^20/GB300", {"nb_group": 16, "nb_by_target_cost": 0})
    t.save()
    data = json.load(open(path))
    assert data["version"] == 1 and len(data["entries"]) == 2
    u = tuning.TuningTable(path)
    assert u.lookup("f64/u64/n2^24/GB300") == {"nb_group": 32, "nb_by_target_cost": 7, "sort_items": 12}
    # a tuning without a sort shape takes the default shape
    assert u.lookup("f32/u32/n2^20/GB300") == {"nb_group": 16, "nb_by_target_cost": 0, "sort_items": 16}
    assert u.entries["f64/u64/n2^24/GB300"]["ms"]["16/7/s16"] == 25.0


def test_table_reads_entries_written_without_the_sort_shape(tmp_path):
    path = str(tmp_path / "old.json")
    json.dump({"version": 1, "entries": {"k": {"nb_group": 16, "nb_by_target_cost": 5, "ms": None}}}, open(path, "w"))
    assert tuning.TuningTable(path).lookup("k") == {"nb_group": 16, "nb_by_target_cost": 5, "sort_items": 16}


def test_tune_pipeline_uses_the_table_before_autotuning():
    class FakePipe:
        def __init__(self):
            self.set, self.tuned = None, 0

        def set_tuning(self, nb_group, nb_by_target_cost, sort_items):
            self.set = (nb_group, nb_by_target_cost, sort_items)

        def autotune(self, reps):
            self.tuned += 1
            return {"best": {"nb_group": 16, "nb_by_target_cost": 5, "sort_items": 12},
                    "tried": [({"nb_group": 32, "nb_by_target_cost": 7, "sort_items": 16}, 2.0),
                              ({"nb_group": 16, "nb_by_target_cost": 5, "sort_items": 16}, 1.0),
                              ({"nb_group": 16, "nb_by_target_cost": 5, "sort_items": 12}, 0.5)]}

    table = tuning.TuningTable()
    p = FakePipe()
    best, tried = tuning.tune_pipeline(p, table, "k")
    assert best == {"nb_group": 16, "nb_by_target_cost": 5, "sort_items": 12} and p.tuned == 1 and len(tried) == 3
    q = FakePipe()
    best, tried = tuning.tune_pipeline(q, table, "k")
    assert tried is None and q.tuned == 0 and q.set == (16, 5, 12)
