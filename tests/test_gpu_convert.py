"""DataFrame -> .bin converter with the relabelling of integer codes on the
GPU (fegb_compact_ids): the ids equal the oracle's and pandas' factorize(sort=True)
+ 1 rule, and a fit from the converted file equals the fit from the table."""
import numpy as np
import pytest

from fe_gpu_gb300 import convert as CV
from fe_gpu_gb300 import fe_gpu_estimate, fe_runtime_config
from fe_gpu_gb300.bin_io import load_dataset_from_file
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_device_relabel_matches_oracle(built):
    rng = np.random.default_rng(5)
    for raw in (rng.integers(-2**31, 2**31 - 1, size=200_000).astype(np.int64),
                rng.choice([3, -9, 7, 2**30], size=50_000),
                np.full(1000, 12), np.array([5])):
        got = CV.relabel_ids(raw)
        np.testing.assert_array_equal(got, O.compact_ids(raw.astype(np.int32))[0])
        _, inv = np.unique(raw, return_inverse=True)
        np.testing.assert_array_equal(got, inv + 1)


def test_convert_then_fit(built, tmp_path):
    rng = np.random.default_rng(8)
    n = 60_000
    worker = rng.integers(0, 4000, size=n) * 7 + 100        # sparse codes
    firm = rng.choice(np.array([f"f{i:03d}" for i in range(300)]), size=n)
    year = rng.integers(1990, 2010, size=n)
    x1, x2 = rng.normal(size=n), rng.normal(size=n)
    y = 0.5 * x1 - 0.25 * x2 + rng.normal(size=n)
    tab = {"y": y, "x1": x1, "x2": x2, "worker": worker, "firm": firm, "year": year}
    out = tmp_path / "t.bin"
    CV.dataframe_to_fe_binary(tab, out, y="y", x=["x1", "x2"], fe=["worker", "firm", "year"])
    hdr, host = load_dataset_from_file(str(out))
    for d, name in enumerate(["worker", "firm", "year"]):
        _, inv = np.unique(tab[name], return_inverse=True)
        np.testing.assert_array_equal(host.fe_ids[d], inv + 1)
    cfg = fe_runtime_config(fe_tolerance=1e-8, fe_max_iterations=100000, cluster_fe_dims=[1, 2],
                            precision="mixed", demean_cg=True)
    res = fe_gpu_estimate(cfg, hdr, host)
    ref = O.gpu_estimate(host.y, host.W, host.fe_ids, tol=1e-11, max_iter=200000, cluster_dims=[1, 2])
    assert res.converged
    assert np.max(np.abs(res.beta - ref.beta) / np.abs(ref.beta)) < 1e-6
    assert np.max(np.abs(res.se - ref.se) / np.abs(ref.se)) < 1e-5
