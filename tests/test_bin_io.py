"""The .bin reader/writer against the reference loader's own test cases
(tests/test_data_loader.f90:17-132)."""
import numpy as np
import pytest

from fe_gpu_gb300.bin_io import (PRECISION_FLOAT32, PRECISION_FLOAT64, FeDataError, load_dataset_from_file,
                                 write_dataset)


def test_case1_old_header_fp64_no_flag(tmp_path):
    # tests/test_data_loader.f90:17-44, 75-102
    p = tmp_path / "case_fp64_noflag.bin"
    y = np.array([1.0, 2.0, -1.0])
    W = np.array([[1.0, 0.5], [0.0, -0.5], [1.0, 2.0]])
    write_dataset(str(p), y, W, np.array([[1, 1, 2]]), cluster=np.array([10, 10, 99]), header="old",
                  write_flag=False)
    assert p.stat().st_size == 24 + 3 * 8 + 6 * 8 + 3 * 4 + 3 * 4
    hdr, host = load_dataset_from_file(str(p))
    assert hdr.n_obs == 3 and hdr.n_regressors == 2 and hdr.n_fe == 1
    assert hdr.has_cluster and not hdr.has_weights
    assert hdr.precision_flag == PRECISION_FLOAT64
    np.testing.assert_allclose(host.y, y, atol=1e-12)
    np.testing.assert_allclose(host.W, W, atol=1e-12)
    assert list(host.fe_ids[0]) == [1, 1, 2]
    assert list(host.cluster) == [10, 10, 99]


def test_case2_new_header_fp32_flag_weights(tmp_path):
    # tests/test_data_loader.f90:46-73, 104-132
    p = tmp_path / "case_fp32_flag.bin"
    write_dataset(str(p), np.array([0.25, 0.75]), np.array([[-1.5], [2.5]]), np.array([[3, 4], [1, 1]]),
                  weights=np.array([1.5, 2.5]), precision_flag=PRECISION_FLOAT32)
    hdr, host = load_dataset_from_file(str(p))
    assert hdr.n_obs == 2 and hdr.n_regressors == 1 and hdr.n_fe == 2
    assert not hdr.has_cluster and hdr.has_weights
    assert hdr.precision_flag == PRECISION_FLOAT32
    np.testing.assert_allclose(host.y, [0.25, 0.75], atol=1e-6)
    np.testing.assert_allclose(host.W[:, 0], [-1.5, 2.5], atol=1e-6)
    assert list(host.fe_ids[0]) == [3, 4] and list(host.fe_ids[1]) == [1, 1]
    np.testing.assert_allclose(host.weights, [1.5, 2.5], atol=1e-6)


def test_metadata_block_and_instruments(tmp_path):
    p = tmp_path / "meta.bin"
    rng = np.random.default_rng(0)
    n = 17
    y, W, Z = rng.standard_normal(n), rng.standard_normal((n, 3)), rng.standard_normal((n, 2))
    fe = np.vstack([rng.integers(1, 5, n), rng.integers(1, 3, n)])
    meta = {"y": "wage", "x": ["a", "b", "c"], "iv": ["z1", "z2"], "fe": ["worker", "firm"], "cluster": "",
            "weights": ""}
    write_dataset(str(p), y, W, fe, Z=Z, metadata=meta)
    hdr, host = load_dataset_from_file(str(p))
    assert hdr.n_instruments == 2 and hdr.metadata_bytes > 0
    assert hdr.depvar_name == "wage" and hdr.regressor_names == ["a", "b", "c"]
    assert hdr.instrument_names == ["z1", "z2"] and hdr.fe_names == ["worker", "firm"]
    np.testing.assert_array_equal(host.Z, Z)
    np.testing.assert_array_equal(host.fe_ids, fe)
    assert host.fe_ids.flags.f_contiguous  # reference host layout: dimension fastest


def test_truncated_and_bad_flag(tmp_path):
    p = tmp_path / "bad.bin"
    p.write_bytes(b"\x00" * 10)
    with pytest.raises(FeDataError):
        load_dataset_from_file(str(p))
    q = tmp_path / "badflag.bin"
    write_dataset(str(q), np.zeros(4), np.zeros((4, 1)), np.ones((1, 4), dtype=np.int32), precision_flag=7)
    with pytest.raises(FeDataError):
        load_dataset_from_file(str(q))
