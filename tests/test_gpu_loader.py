"""The .bin dataset read straight to the device (fegb_load_bin) against the
host reader that restates src/io/fe_data_io.f90: every header variant
(new / old header, FP64 / FP32 values, with and without the precision flag,
META names, cluster ids and weights), bit for bit, plus a truncated file."""
import ctypes as C

import numpy as np
import pytest

from fe_gpu_gb300 import _native as N
from fe_gpu_gb300.bin_io import DeviceDataset, load_dataset_from_file, write_dataset

pytestmark = pytest.mark.gpu


def _back(ptr, dtype, count):
    out = np.empty(count, dtype=dtype)
    if count:
        N.check(N.lib().fe_gpu_runtime_memcpy_dtoh(out.ctypes.data, C.c_void_p(ptr), out.nbytes), "dtoh")
    return out


CASES = [
    dict(precision_flag=0, header="new", write_flag=True, l=2, meta=True, cluster=True, weights=True),
    dict(precision_flag=1, header="new", write_flag=True, l=1, meta=True, cluster=False, weights=False),
    dict(precision_flag=1, header="new", write_flag=False, l=0, meta=False, cluster=False, weights=True),
    dict(precision_flag=0, header="old", write_flag=False, l=0, meta=False, cluster=True, weights=False),
    dict(precision_flag=0, header="new", write_flag=False, l=3, meta=False, cluster=False, weights=False),
]


@pytest.mark.parametrize("case", range(len(CASES)))
def test_device_load_matches_host_reader(built, tmp_path, case):
    c = CASES[case]
    rng = np.random.default_rng(case)
    n, k = (1_500_007 if case < 2 else 100_003), 4  # the first cases span several 32 MB chunks
    y = rng.standard_normal(n)
    W = rng.standard_normal((n, k))
    Z = rng.standard_normal((n, c["l"])) if c["l"] else None
    fe = np.vstack([rng.integers(1, g, n) for g in (500, 40, 7)]).astype(np.int32)
    meta = dict(y="y", x=[f"x{j}" for j in range(k)], iv=[f"z{j}" for j in range(c["l"])],
                fe=["a", "b", "c"]) if c["meta"] else None
    path = tmp_path / "d.bin"
    write_dataset(str(path), y, W, fe, Z=Z, cluster=fe[0] if c["cluster"] else None,
                  weights=np.abs(y) if c["weights"] else None, precision_flag=c["precision_flag"], metadata=meta,
                  header=c["header"], write_flag=c["write_flag"])
    hdr, host = load_dataset_from_file(str(path))
    ds = DeviceDataset(str(path))
    try:
        assert (ds.n, ds.k, ds.l, ds.n_fe) == (hdr.n_obs, hdr.n_regressors, hdr.n_instruments, hdr.n_fe)
        assert ds.header.precision_flag == hdr.precision_flag
        assert ds.header.regressor_names == hdr.regressor_names and ds.header.fe_names == hdr.fe_names
        if c["meta"]:
            assert ds.header.fe_names == ["a", "b", "c"] and ds.header.regressor_names[0] == "x0"
        assert np.array_equal(_back(ds.y, np.float64, n), host.y)
        assert np.array_equal(_back(ds.W, np.float64, n * k).reshape(k, n).T, host.W)
        if hdr.n_instruments:
            l = hdr.n_instruments
            assert np.array_equal(_back(ds.Z, np.float64, n * l).reshape(l, n).T, host.Z)
        for d in range(hdr.n_fe):
            assert np.array_equal(_back(ds.fe_ids[d], np.int32, n), host.fe_ids[d])
        if hdr.has_cluster:
            assert np.array_equal(_back(ds.cluster, np.int32, n), host.cluster)
        if hdr.has_weights:
            assert np.array_equal(_back(ds.weights, np.float64, n), host.weights)
    finally:
        ds.close()


def test_truncated_file_is_an_error(built, tmp_path):
    rng = np.random.default_rng(9)
    n = 1000
    path = tmp_path / "t.bin"
    write_dataset(str(path), rng.standard_normal(n), rng.standard_normal((n, 2)),
                  rng.integers(1, 9, (2, n)).astype(np.int32))
    raw = path.read_bytes()
    path.write_bytes(raw[: len(raw) - 100])
    with pytest.raises(N.FeGpuError):
        DeviceDataset(str(path))
    with pytest.raises(N.FeGpuError):
        DeviceDataset(str(tmp_path / "missing.bin"))
