"""DataFrame -> .bin converter (tools/dataframe_to_fe_binary.py) on the CPU:
column handling, missing values, the relabelling rule (pandas
factorize(sort=True) + 1, restated with numpy.unique) and the written file
read back by the .bin reader. The integer relabelling is the oracle's here;
tests/test_gpu_convert.py runs the device one."""
import pathlib

import numpy as np
import pytest

from fe_gpu_gb300 import convert as CV
from fe_gpu_gb300.bin_io import load_dataset_from_file
from oracle import oracle as O


def oracle_compact(raw):
    return O.compact_ids(raw)[0]


def factorize_sorted(values):
    _, inv = np.unique(np.asarray(values), return_inverse=True)
    return inv.reshape(-1) + 1


def table(n=500, seed=3):
    rng = np.random.default_rng(seed)
    return {
        "y": rng.normal(size=n),
        "x1": rng.normal(size=n),
        "x2": rng.integers(0, 5, size=n).astype(np.float64),
        "z1": rng.normal(size=n),
        "worker": rng.choice([-7, 3, 1000, 2**30, 42], size=n),            # int codes with gaps and negatives
        "firm": rng.choice(np.array(["acme", "Bolt", "zeta", "a"]), size=n),  # text labels
        "year": rng.choice([2001.0, 1999.0, 2010.0], size=n),              # integral floats
        "big": rng.choice([2**40, -2**35, 5], size=n),                      # int64 beyond int32
        "cl": rng.choice([9, 8, 7], size=n),
        "w": rng.uniform(0.5, 2.0, size=n),
    }


def test_relabel_rule():
    t = table()
    for name in ("worker", "firm", "year", "big", "cl"):
        np.testing.assert_array_equal(CV.relabel_ids(t[name], oracle_compact), factorize_sorted(t[name]))


def test_convert_roundtrip(tmp_path):
    t = table()
    out = tmp_path / "d.bin"
    info = CV.dataframe_to_fe_binary(t, out, y="y", x=["x1", "x2"], fe=["worker", "firm", "year", "big"],
                                     iv=["z1"], cluster="cl", weights="w", compact=oracle_compact)
    assert info == {"n_obs": 500, "n_regressors": 2, "n_fe_dims": 4, "n_instruments": 1, "clustered": True,
                    "weights": True, "precision": "float64"}
    hdr, host = load_dataset_from_file(str(out))
    np.testing.assert_array_equal(host.y, t["y"])
    np.testing.assert_array_equal(host.W, np.column_stack([t["x1"], t["x2"]]))
    np.testing.assert_array_equal(host.Z[:, 0], t["z1"])
    for d, name in enumerate(["worker", "firm", "year", "big"]):
        np.testing.assert_array_equal(host.fe_ids[d], factorize_sorted(t[name]))
    np.testing.assert_array_equal(host.cluster, factorize_sorted(t["cl"]))
    np.testing.assert_array_equal(host.weights, t["w"])
    assert hdr.depvar_name == "y" and hdr.regressor_names == ["x1", "x2"]
    assert hdr.fe_names == ["worker", "firm", "year", "big"] and hdr.instrument_names == ["z1"]
    assert hdr.cluster_name == "cl" and hdr.weight_name == "w" and hdr.n_fe == 4 and hdr.has_weights


def test_float32_and_missing(tmp_path):
    t = table(n=200)
    t["x1"] = t["x1"].copy()
    t["x1"][[3, 50]] = np.nan
    t["firm"] = t["firm"].astype(object)
    t["firm"][7] = None
    with pytest.raises(ValueError, match="missing values"):
        CV.dataframe_to_fe_binary(t, tmp_path / "a.bin", y="y", x=["x1"], fe=["worker", "firm"],
                                  compact=oracle_compact)
    info = CV.dataframe_to_fe_binary(t, tmp_path / "b.bin", y="y", x=["x1"], fe=["worker", "firm"],
                                     precision="float32", drop_missing=True, compact=oracle_compact)
    assert info["n_obs"] == 197 and info["precision"] == "float32"
    keep = np.ones(200, bool)
    keep[[3, 50, 7]] = False
    hdr, host = load_dataset_from_file(str(tmp_path / "b.bin"))
    np.testing.assert_array_equal(host.y, t["y"][keep].astype(np.float32).astype(np.float64))
    np.testing.assert_array_equal(host.fe_ids[1], factorize_sorted(t["firm"][keep].astype(str)))


def test_csv_input(tmp_path):
    t = table(n=60)
    path = tmp_path / "in.csv"
    names = ["y", "x1", "worker", "firm", "year"]
    with open(path, "w") as f:
        f.write(",".join(names) + "\n")
        for i in range(60):
            f.write(",".join(repr(float(t[c][i])) if c in ("y", "x1", "year") else str(t[c][i]) for c in names) + "\n")
    tab = CV.load_table(path, "auto", names)
    assert tab["worker"].dtype == np.int64 and tab["firm"].dtype == object
    CV.dataframe_to_fe_binary(tab, tmp_path / "c.bin", y="y", x=["x1"], fe=["worker", "firm", "year"],
                              compact=oracle_compact)
    hdr, host = load_dataset_from_file(str(tmp_path / "c.bin"))
    np.testing.assert_array_equal(host.y, t["y"])
    for d, name in enumerate(["worker", "firm", "year"]):
        np.testing.assert_array_equal(host.fe_ids[d], factorize_sorted(t[name]))


def test_errors(tmp_path):
    t = table(n=10)
    with pytest.raises(KeyError):
        CV.dataframe_to_fe_binary(t, tmp_path / "e.bin", y="y", x=["nope"], fe=["worker"], compact=oracle_compact)
    with pytest.raises(ValueError):
        CV.dataframe_to_fe_binary(t, tmp_path / "e.bin", y="y", x=["x1"], fe=["worker"], precision="float16",
                                  compact=oracle_compact)
    with pytest.raises(ValueError, match="not numeric"):
        CV.dataframe_to_fe_binary(t, tmp_path / "e.bin", y="firm", x=["x1"], fe=["worker"], compact=oracle_compact)
