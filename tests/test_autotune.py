"""The autotuner's table lookup and knob plumbing (fegb_set_tuning), on CPU:
the library loads without a GPU, and the knobs are host-side integers."""
import pytest

from fe_gpu_gb300 import _native as N
from fe_gpu_gb300 import autotune as A


def test_knobs_set_get_reset(built):
    A.reset()
    assert A.get_knob("dense_form") == -1 and A.get_knob("cg_graph") == 1 and A.get_knob("batch_estimator") == 1
    A.set_knob("cg_cols_per_pass", 8)
    assert A.get_knob("cg_cols_per_pass") == 8
    assert N.lib().fegb_set_tuning(b"cg_cols_per_pass", 5) != 0  # only 0, 4 or 8
    assert N.lib().fegb_set_tuning(b"no_such_knob", 1) != 0
    assert "unknown key" in N.last_error()
    A.reset()
    assert A.get_knob("cg_cols_per_pass") == 0


def test_entry_for_shape_picks_column_class_and_nearest_rows():
    table = {"entries": [
        {"rows": 2_000_000, "column_class": 9, "best": {"dense_form": 0}},
        {"rows": 20_000_000, "column_class": 9, "best": {"dense_form": 1}},
        {"rows": 37_000, "column_class": 8, "best": {"cg_graph": 0}},
    ]}
    assert A.entry_for_shape(150_000_000, 9, table)["best"] == {"dense_form": 1}
    assert A.entry_for_shape(3_000_000, 9, table)["best"] == {"dense_form": 0}
    assert A.entry_for_shape(40_000, 6, table)["best"] == {"cg_graph": 0}
    assert A.entry_for_shape(40_000, 40, table) is None
    assert A.column_class(6) == 8 and A.column_class(9) == 9 and A.column_class(111) == 112


def test_apply_for_shape_sets_then_resets(built):
    table = {"entries": [{"rows": 1000, "column_class": 9, "best": {"dense_form": 0, "cg_cols_per_pass": 4}}]}
    A.apply_for_shape(1000, 9, table)
    assert A.get_knob("dense_form") == 0 and A.get_knob("cg_cols_per_pass") == 4
    A.apply_for_shape(1000, 40, table)  # no entry: defaults
    assert A.get_knob("dense_form") == -1 and A.get_knob("cg_cols_per_pass") == 0


@pytest.mark.parametrize("value", ["off"])
def test_tuning_off_leaves_knobs(built, monkeypatch, value):
    monkeypatch.setenv("FEGB_TUNING", value)
    A.reset()
    A.set_knob("cg_graph", 0)
    assert A.apply_for_shape(1000, 9) is None
    assert A.get_knob("cg_graph") == 0
    A.reset()


def test_every_listed_knob_value_is_accepted_and_the_table_names_known_knobs(built):
    """The autotuner's knob list and the library's agree: every value the
    tuner tries is accepted, and the committed table names only known knobs."""
    import json

    A.reset()
    for key, values in A.KNOBS.items():
        for v in values:
            A.set_knob(key, v)
            assert A.get_knob(key) == v
        A.reset()
    table = json.loads(A.TABLE.read_text())
    for e in table["entries"]:
        for key in e.get("best", {}):
            assert key in A.KNOBS, key
            A.get_knob(key)  # known to the library as well
