"""Formula expansion on the device against the oracle: levels
(fegb_design_levels) and expanded columns (fegb_build_design) bit for bit,
and a 2SLS fit with categorical regressors and instruments through the
formula front end against the oracle's GPU-convention estimator on the
oracle-expanded matrices."""
import numpy as np
import pytest

from fe_gpu_gb300.bin_io import fe_dataset_header, fe_host_arrays
from fe_gpu_gb300.formula import (build_columns, device_levels, fe_gpu_estimate_formula, parse_formula_string,
                                  plan_design, prepare_formula)
from oracle import design_ref as D
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _to_device(a):
    from fe_gpu_gb300.estimator import DeviceBuffer

    return DeviceBuffer.from_array(np.asfortranarray(a, dtype=np.float64))


def test_levels_match_oracle(built):
    rng = np.random.default_rng(3)
    n = 200_003
    cols = [
        rng.integers(-5, 6, n).astype(float),                         # few levels, negatives
        rng.integers(0, 500, n).astype(float),                        # more than 40 levels: first 40 by appearance
        np.where(rng.random(n) < 0.3, rng.random(n) * 10, rng.integers(1, 8, n)),  # non-integers mixed in
        rng.integers(1, 21, n) + rng.choice([0.0, 4e-7, -4e-7, 0.5], n),  # within / beyond the 1e-6 tolerance
        np.full(n, 7.0),                                              # one level
        np.concatenate([[3e9, -3e9], rng.integers(1, 4, n - 2).astype(float)]),  # beyond int32
    ]
    for c in cols:
        b = _to_device(c)
        assert device_levels(b.ptr, n) == D.collect_levels(c)
    assert device_levels(_to_device(np.array([0.5, 1.5])).ptr, 2) == []


def _nls_like(n=60_000, seed=11):
    rng = np.random.default_rng(seed)
    hours = rng.normal(37, 10, n)
    ttl_exp = rng.gamma(2, 3, n)
    union = (rng.random(n) < 0.25).astype(float)
    tenure = rng.exponential(5, n)
    wks_ue = rng.poisson(2, n).astype(float)
    ind_code = rng.integers(1, 13, n).astype(float)
    msp = (rng.random(n) < 0.5).astype(float)
    wks_work = rng.normal(50, 5, n)
    ids = [rng.integers(1, 3001, n), rng.integers(1, 14, n), rng.integers(1, 13, n)]
    hours = hours + 0.3 * wks_work + 0.1 * ind_code
    y = (0.02 * hours + 0.03 * ttl_exp + 0.1 * union + 0.01 * tenure - 0.001 * wks_ue + 0.05 * (ind_code == 4)
         - 0.02 * msp + rng.normal(0, 0.3, n))
    W = np.column_stack([hours, ttl_exp, union, tenure, wks_ue, ind_code, msp])
    Z = np.column_stack([wks_work, ind_code])
    fe = np.vstack(ids).astype(np.int32)
    hdr = fe_dataset_header(n_obs=n, n_regressors=7, n_instruments=2, n_fe=3, depvar_name="ln_wage",
                            regressor_names=["hours", "ttl_exp", "union", "tenure", "wks_ue", "ind_code", "msp"],
                            instrument_names=["wks_work", "ind_code"], fe_names=["idcode", "occ_code", "year"])
    return hdr, fe_host_arrays(y=y, W=np.asfortranarray(W), Z=np.asfortranarray(Z), fe_ids=np.asfortranarray(fe))


def _oracle_design(plan, host):
    src = {}
    for j in range(host.W.shape[1]):
        src[("W", j)] = host.W[:, j]
    for j in range(host.Z.shape[1]):
        src[("Z", j)] = host.Z[:, j]
    W = D.expand(src, [c.factors for c in plan.regressors])
    Z = D.expand(src, [c.factors for c in plan.instruments]) if plan.instruments is not None else host.Z
    return W, Z


FORMULAS = [
    "ln_wage ~ hours ttl_exp union tenure wks_ue i.1.ind_code&&i.2.msp tenure&wks_ue, fe(idcode occ_code year) "
    "cluster(idcode occ_code year)",
    "ln_wage ~ hours i.2.msp ttl_exp union tenure wks_ue (hours i.2.msp ~ wks_work i.1.ind_code), "
    "fe(idcode occ_code year) cluster(idcode occ_code)",
]


@pytest.mark.parametrize("formula", FORMULAS)
def test_device_design_matches_oracle_bitwise(built, formula):
    hdr, host = _nls_like()
    ff, cfg = prepare_formula(formula, hdr, host)
    W_ref, Z_ref = _oracle_design(ff.plan, host)
    W_dev = ff.buffers["W"].to_array(np.float64, (ff.n, ff.k), order="F")
    assert np.array_equal(W_dev, W_ref)
    if ff.plan.instruments is not None:
        Z_dev = ff.buffers["Z"].to_array(np.float64, (ff.n, ff.l), order="F")
        assert np.array_equal(Z_dev, Z_ref)


@pytest.mark.parametrize("formula", FORMULAS)
@pytest.mark.parametrize("precision,cg", [("fp64", False), ("mixed", True)])
def test_formula_fit_matches_oracle(built, formula, precision, cg):
    from fe_gpu_gb300.estimator import fe_runtime_config

    hdr, host = _nls_like()
    cfg = fe_runtime_config(fe_tolerance=1e-8, fe_max_iterations=100000, precision=precision, demean_cg=cg)
    res = fe_gpu_estimate_formula(formula, hdr, host, cfg)
    ff = res.formula
    W_ref, Z_ref = _oracle_design(ff.plan, host)
    fe = host.fe_ids[np.array(ff.binding.fe_selection) - 1]
    ref = O.gpu_estimate(host.y, W_ref, fe, Z=Z_ref, tol=1e-12, max_iter=200000,
                         cluster_dims=ff.binding.cluster_fe_dims, iv_regressors=ff.plan.iv_regressors,
                         iv_instruments=ff.plan.iv_instrument_cols)
    assert res.coef_names == ff.plan.regressor_names
    assert res.is_iv == bool(ref.stats["is_iv"])
    assert res.n_instruments == ref.stats["n_instruments"]
    assert res.dof_model == ref.stats["dof_model"] and res.dof_resid == ref.stats["dof_resid"]
    ok = ref.se > 0
    assert np.max(np.abs(res.beta - ref.beta) / np.maximum(np.abs(ref.beta), 1e-300)) < 1e-6
    assert np.max(np.abs(res.se[ok] - ref.se[ok]) / ref.se[ok]) < 1e-5
