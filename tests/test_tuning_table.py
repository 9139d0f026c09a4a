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
    t.store("f64/u64/n2^24/GB300", {"nb_group": 32, "nb_by_target_cost": 7}, {"32/7": 18.9, "16/7": 25.0})
    t.store("f32/u32/n2^20/GB300", {"nb_group": 16, "nb_by_target_cost": 0})
    t.save()
    data = json.load(open(path))
    assert data["version"] == 1 and len(data["entries"]) == 2
    u = tuning.TuningTable(path)
    assert u.lookup("f64/u64/n2^24/GB300") == {"nb_group": 32, "nb_by_target_cost": 7}
    assert u.lookup("f32/u32/n2^20/GB300") == {"nb_group": 16, "nb_by_target_cost": 0}
    assert u.entries["f64/u64/n2^24/GB300"]["ms"]["16/7"] == 25.0


def test_tune_pipeline_uses_the_table_before_autotuning():
    class FakePipe:
        def __init__(self):
            self.set, self.tuned = None, 0

        def set_tuning(self, nb_group, nb_by_target_cost):
            self.set = (nb_group, nb_by_target_cost)

        def autotune(self, reps):
            self.tuned += 1
            return {"best": {"nb_group": 16, "nb_by_target_cost": 5},
                    "tried": [({"nb_group": 32, "nb_by_target_cost": 7}, 2.0),
                              ({"nb_group": 16, "nb_by_target_cost": 5}, 1.0)]}

    table = tuning.TuningTable()
    p = FakePipe()
    best, tried = tuning.tune_pipeline(p, table, "k")
    assert best == {"nb_group": 16, "nb_by_target_cost": 5} and p.tuned == 1 and len(tried) == 2
    q = FakePipe()
    best, tried = tuning.tune_pipeline(q, table, "k")
    assert tried is None and q.tuned == 0 and q.set == (16, 5)
