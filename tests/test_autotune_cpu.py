"""Host logic of the autotuner: a tuning table written by an earlier process
is read back and answers without timing anything (no device needed)."""
import json

from fdfdpy_gb300.autotune import Autotuner


def test_table_file_round_trip(tmp_path):
    path = tmp_path / "tune.json"
    table = {json.dumps([256, 256, "c64tc"]): {"batch": 4, "fused_max_m": 128, "solves_per_s": 1.0,
                                               "candidates": []}}
    path.write_text(json.dumps(table))
    t = Autotuner(path=str(path))
    assert t.batch_for((256, 256), "c64tc") == 4
    assert t.fused_for((256, 256), "c64tc") == 128
    assert (256, 256, "c64tc") in t.table and (128, 128, "c64tc") not in t.table
