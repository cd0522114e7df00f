"""Branches of the estimation path that change results, each against the CPU
oracle through the C ABI:

* FE compaction (fegb_compact_ids): 1-based rank among the sorted distinct raw
  codes (tools/dataframe_to_fe_binary.py:87-94), bit-exact, on codes with
  negatives, gaps and the int32 extremes;
* iterated singleton removal (fegb_drop_singletons), the same kept rows;
* multi-way cluster ids on the device (fegb_cluster_ids), bit-exact with the
  restated builder (src/core/cluster_id_builder.c:173-189) including the
  first-appearance ids used when the key span exceeds 2^62
  (cluster_id_builder.c:202-257);
* the column filter of solve_with_column_filter (src/core/fe_pipeline.f90:
  1034-1107): a regressor constant within the groups of an FE is absorbed and
  dropped; rank, dof_model, the zero coefficient and SE of the dropped column
  and the kept coefficients match the oracle;
* the PSD fix of a 3-way clustered covariance (fe_pipeline.f90:1844-1894):
  the device reports it applied, as the oracle does, and the SEs match.

Integer outputs must be equal; coefficients 1e-6 and SEs 1e-5 relative.
"""
import ctypes as C

import numpy as np
import pytest

from fe_gpu_gb300 import _native as N
from fe_gpu_gb300 import fe_gpu_estimate, fe_runtime_config
from fe_gpu_gb300.bin_io import fe_host_arrays
from fe_gpu_gb300.estimator import DeviceBuffer
from oracle import oracle as O

pytestmark = pytest.mark.gpu

BETA_RTOL = 1e-6
SE_RTOL = 1e-5


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))) if a.size else 0.0


def device_compact(raw):
    raw = np.ascontiguousarray(raw, dtype=np.int32)
    n = raw.size
    d_raw = DeviceBuffer.from_array(raw if n else np.zeros(1, np.int32))
    d_out = DeviceBuffer(max(1, n) * 4)
    lv = C.c_int(-1)
    N.check(N.lib().fegb_compact_ids(C.c_void_p(d_raw.ptr), n, C.c_void_p(d_out.ptr), C.byref(lv)),
            "fegb_compact_ids")
    out = d_out.to_array(np.int32, (n,))
    d_raw.free()
    d_out.free()
    return out, lv.value


@pytest.mark.parametrize("case", ["gaps_negatives", "extremes", "all_equal", "single", "large_random"])
def test_compact_ids_matches_oracle(built, case):
    rng = np.random.default_rng(31)
    if case == "gaps_negatives":
        raw = rng.choice(np.array([-7, -3, 0, 2, 5, 11, 100, 2 ** 20], dtype=np.int64), size=5000).astype(np.int32)
    elif case == "extremes":
        raw = np.array([2 ** 31 - 1, -2 ** 31, 0, -1, 1, 2 ** 31 - 1, -2 ** 31, 17], dtype=np.int32)
    elif case == "all_equal":
        raw = np.full(1000, -42, dtype=np.int32)
    elif case == "single":
        raw = np.array([123456], dtype=np.int32)
    else:
        raw = rng.integers(-2 ** 31, 2 ** 31 - 1, size=300_000, dtype=np.int64).astype(np.int32)
        raw[::3] = raw[1::3][: raw[::3].size]  # repeated codes
    got, lv = device_compact(raw)
    ref, rlv = O.compact_ids(raw)
    assert lv == rlv == np.unique(raw).size
    np.testing.assert_array_equal(got, ref)
    # the rank among sorted distinct codes, 1-based
    np.testing.assert_array_equal(got, np.searchsorted(np.unique(raw), raw) + 1)


def test_compact_ids_empty(built):
    got, lv = device_compact(np.zeros(0, np.int32))
    assert got.size == 0 and lv == 0


def _device_ids(fe):
    return [DeviceBuffer.from_array(np.ascontiguousarray(fe[d])) for d in range(fe.shape[0])]


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_drop_singletons_matches_oracle(built, seed):
    rng = np.random.default_rng(seed)
    n = 20_000
    # many small groups so that removal cascades over several rounds
    fe = np.asfortranarray(np.vstack([rng.integers(1, 9001, n), rng.integers(1, 3001, n),
                                      rng.integers(1, 12, n)]).astype(np.int32))
    sizes = fe.max(axis=1).astype(np.int32)
    bufs = _device_ids(fe)
    ptrs = (C.c_void_p * 3)(*[C.c_void_p(b.ptr) for b in bufs])
    d_keep = DeviceBuffer(n)
    nd = C.c_longlong(-1)
    N.check(N.lib().fegb_drop_singletons(ptrs, sizes.ctypes.data_as(C.POINTER(C.c_int)), 3, n,
                                         C.c_void_p(d_keep.ptr), C.byref(nd)), "fegb_drop_singletons")
    keep = d_keep.to_array(np.uint8, (n,)).astype(bool)
    rkeep, rdropped = O.drop_singletons(fe, sizes)
    assert rdropped > 0
    assert nd.value == rdropped
    np.testing.assert_array_equal(keep, rkeep)
    # the kept rows have no singleton group left in any dimension
    for d in range(3):
        cnt = np.bincount(fe[d][keep])
        assert not np.any(cnt == 1)
    for b in bufs + [d_keep]:
        b.free()


def test_fit_with_singleton_removal_matches_oracle_on_kept_rows(built):
    rng = np.random.default_rng(8)
    n = 6000
    fe = np.asfortranarray(np.vstack([rng.integers(1, 2501, n), rng.integers(1, 400, n),
                                      rng.integers(1, 8, n)]).astype(np.int32))
    W = np.asfortranarray(rng.standard_normal((n, 3)))
    y = W @ np.array([0.3, -0.6, 1.1]) + 0.4 * rng.standard_normal(n)
    cfg = fe_runtime_config(fe_tolerance=1e-10, fe_max_iterations=100000, cluster_fe_dims=[1],
                            drop_singletons=True)
    res = fe_gpu_estimate(cfg, None, fe_host_arrays(y=y, W=W, Z=np.zeros((n, 0), order="F"), fe_ids=fe))
    keep, dropped = O.drop_singletons(fe)
    assert res.n_singletons == dropped and res.n_obs_used == n - dropped
    fk = np.asfortranarray(fe[:, keep])
    ref = O.gpu_estimate(y[keep], W[keep], fk, tol=1e-12, max_iter=200000, cluster_dims=[1],
                         sizes=fe.max(axis=1))
    assert rel(res.beta, ref.beta) < BETA_RTOL
    assert rel(res.se, ref.se) < SE_RTOL


def device_cluster_ids(fe, sizes, dims):
    n = fe.shape[1]
    bufs = [DeviceBuffer.from_array(np.ascontiguousarray(fe[d - 1])) for d in dims]
    ptrs = (C.c_void_p * len(dims))(*[C.c_void_p(b.ptr) for b in bufs])
    ss = np.array([sizes[d - 1] for d in dims], dtype=np.int32)
    d_out = DeviceBuffer(max(1, n) * 4)
    nc = C.c_int(-1)
    N.check(N.lib().fegb_cluster_ids(ptrs, ss.ctypes.data_as(C.POINTER(C.c_int)), len(dims), n,
                                     C.c_void_p(d_out.ptr), C.byref(nc)), "fegb_cluster_ids")
    out = d_out.to_array(np.int32, (n,))
    for b in bufs + [d_out]:
        b.free()
    return out, nc.value


@pytest.mark.parametrize("dims", [[1], [2, 3], [1, 3], [1, 2, 3]])
def test_cluster_ids_device_matches_oracle(built, dims):
    rng = np.random.default_rng(41)
    n = 150_000
    fe = np.asfortranarray(np.vstack([rng.integers(1, 20001, n), rng.integers(1, 501, n),
                                      rng.integers(1, 31, n)]).astype(np.int32))
    sizes = fe.max(axis=1)
    got, nc = device_cluster_ids(fe, sizes, dims)
    ref, rnc, st = O.cluster_ids(fe, sizes, dims)
    assert st == 0
    assert nc == rnc
    np.testing.assert_array_equal(got, ref)


def test_cluster_ids_device_first_appearance_above_2_62(built):
    """Three dimensions of 2^21 + 5 levels each: the key span (about 2^63)
    exceeds 2^62, so ids follow first appearance, on the device as in the
    builder."""
    rng = np.random.default_rng(43)
    n = 100_000
    big = 2 ** 21 + 5
    # ids drawn from a few hundred values each so that tuples repeat
    fe = np.asfortranarray(np.vstack([rng.choice(np.arange(big - 300, big + 1), n),
                                      rng.integers(1, 40, n), rng.choice([1, 7, big], n)]).astype(np.int32))
    sizes = np.array([big, big, big], dtype=np.int64)
    got, nc = device_cluster_ids(fe, sizes, [1, 2, 3])
    ref, rnc, st = O.cluster_ids(fe, sizes, [1, 2, 3])
    assert st == 0
    assert nc == rnc
    np.testing.assert_array_equal(got, ref)
    # first appearance: the first row is cluster 1 and new ids appear in order
    assert got[0] == 1
    assert np.all(np.diff(np.maximum.accumulate(got)) <= 1)
    first = np.unique(got, return_index=True)[1]
    assert np.all(np.diff(first) > 0)


@pytest.mark.parametrize("precision,cg", [("fp64", False), ("mixed", True), ("mixed", False)])
def test_column_filter_drops_absorbed_regressor(built, precision, cg):
    """A regressor constant within each individual is absorbed by the
    individual FE; its demeaned column is zero up to rounding and the filter
    drops it."""
    rng = np.random.default_rng(17)
    n_id, n_years = 800, 8
    ids = np.repeat(np.arange(1, n_id + 1), n_years).astype(np.int32)
    year = np.tile(np.arange(1, n_years + 1), n_id).astype(np.int32)
    n = ids.size
    firm = rng.integers(1, 60, n).astype(np.int32)
    x1 = rng.standard_normal(n)
    absorbed = rng.standard_normal(n_id)[ids - 1] * 3.0 + 5.0  # constant within each id
    x3 = rng.standard_normal(n)
    W = np.asfortranarray(np.column_stack([x1, absorbed, x3]))
    y = 0.8 * x1 - 0.3 * x3 + rng.standard_normal(n_id)[ids - 1] + 0.5 * rng.standard_normal(n)
    fe = np.asfortranarray(np.vstack([ids, firm, year]))
    host = fe_host_arrays(y=y, W=W, Z=np.zeros((n, 0), order="F"), fe_ids=fe)
    cfg = fe_runtime_config(fe_tolerance=1e-10, fe_max_iterations=100000, cluster_fe_dims=[1, 2],
                            precision=precision, demean_cg=cg)
    res = fe_gpu_estimate(cfg, None, host)
    ref = O.gpu_estimate(y, W, fe, tol=1e-12, max_iter=200000, cluster_dims=[1, 2])
    assert res.converged
    assert ref.stats["dof_model"] == 2 and ref.stats["rank"] == 2
    assert res.dof_model == ref.stats["dof_model"]
    assert res.rank == ref.stats["rank"]
    assert res.dof_resid == ref.stats["dof_resid"]
    assert res.beta[1] == 0.0 and res.se[1] == 0.0
    assert ref.beta[1] == 0.0 and ref.se[1] == 0.0
    keep = [0, 2]
    assert rel(res.beta[keep], ref.beta[keep]) < BETA_RTOL
    assert rel(res.se[keep], ref.se[keep]) < SE_RTOL


@pytest.mark.parametrize("precision,cg", [("fp64", False), ("mixed", True)])
@pytest.mark.parametrize("seed", [0, 5])
def test_psd_fix_applied_matches_oracle(built, precision, cg, seed):
    """3-way clustering with 5 and 3 clusters in two dimensions: the
    inclusion-exclusion covariance has a negative eigenvalue, the fix clamps
    it (device Jacobi eigensolver) and the SEs match the oracle's."""
    rng = np.random.default_rng(seed)
    n = 400
    fe = np.asfortranarray(np.vstack([rng.integers(1, 41, n), rng.integers(1, 6, n),
                                      rng.integers(1, 4, n)]).astype(np.int32))
    W = np.asfortranarray(rng.standard_normal((n, 4)))
    y = W @ np.array([0.5, -1.0, 0.2, 0.1]) + rng.standard_normal(n)
    host = fe_host_arrays(y=y, W=W, Z=np.zeros((n, 0), order="F"), fe_ids=fe)
    cfg = fe_runtime_config(fe_tolerance=1e-10, fe_max_iterations=100000, cluster_fe_dims=[1, 2, 3],
                            precision=precision, demean_cg=cg)
    res = fe_gpu_estimate(cfg, None, host)
    ref = O.gpu_estimate(y, W, fe, tol=1e-12, max_iter=200000, cluster_dims=[1, 2, 3])
    assert ref.stats["psd_fix_applied"] == 1
    assert res.psd_fix_applied
    assert res.dof_resid == ref.stats["dof_resid"]
    assert rel(res.beta, ref.beta) < BETA_RTOL
    assert rel(res.se, ref.se) < SE_RTOL
