"""Parity of the CUDA estimator (through the C ABI) with the CPU oracle.

Tolerances (the parity bar of the estimation path, at fe-tol 1e-8 on both
sides unless stated): coefficients 1e-6 relative, standard errors 1e-5
relative; ids, degrees of freedom and cluster counts exactly equal.
"""
import numpy as np
import pytest

from fe_gpu_gb300 import fe_gpu_estimate, fe_gpu_within_transform, fe_runtime_config
from fe_gpu_gb300.bin_io import fe_host_arrays
from fe_gpu_gb300.synth import nls_panel, worker_firm_panel
from oracle import oracle as O

pytestmark = pytest.mark.gpu

BETA_RTOL = 1e-6
SE_RTOL = 1e-5


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))) if a.size else 0.0


def six_row_case():
    # tests/test_gpu_regression.f90:49-83
    W = np.array([[1.0, -2.0], [1.5, 0.5], [-0.5, 1.0], [-1.0, -1.5], [0.25, 0.75], [2.0, 1.25]])
    fe = np.asfortranarray(np.array([[1, 1, 2, 2, 3, 3], [1, 2, 1, 2, 1, 2]], dtype=np.int32))
    y = W @ np.array([1.5, -0.75]) + np.array([0.5, -0.25, 0.8])[fe[0] - 1] + np.array([-0.4, 0.2])[fe[1] - 1]
    return fe_host_arrays(y=y, W=np.asfortranarray(W), Z=np.zeros((6, 0), order="F"), fe_ids=fe)


@pytest.mark.parametrize("method", ["ap", "cg"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_reference_regression_known_answer(built, method, precision):
    # tests/test_gpu_regression.f90: beta = (1.5, -0.75) to 1e-8 at fe_tol 1e-10
    host = six_row_case()
    cfg = fe_runtime_config(fe_tolerance=1e-10, fe_max_iterations=500, precision=precision,
                            demean_cg=(method == "cg"))
    res = fe_gpu_estimate(cfg, None, host)
    assert res.converged
    assert res.solver_info == 0
    np.testing.assert_allclose(res.beta, [1.5, -0.75], atol=1e-8, rtol=0)


@pytest.mark.parametrize("method", ["ap", "cg"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_reference_demean_known_answer(built, method, precision):
    # tests/test_gpu_demean.f90:43-125: group means < 1e-6 after tol 1e-8, 200 iterations
    y = np.array([1.0, 2.0, 3.0, -2.0, -1.0, 0.5])
    W = np.asfortranarray(np.array([[1.0, 0.0], [1.5, -2.0], [-0.5, 1.0], [-1.0, 0.5], [2.0, 1.5], [-0.5, -1.0]]))
    fe = np.array([[1, 1, 2, 2, 3, 3], [1, 2, 1, 2, 1, 2]], dtype=np.int32)
    host = fe_host_arrays(y=y, W=W, Z=np.zeros((6, 0), order="F"), fe_ids=fe)
    conv, iters, mu = fe_gpu_within_transform(fe_runtime_config(fe_tolerance=1e-8, fe_max_iterations=200,
                                                                precision=precision, demean_cg=(method == "cg")),
                                              host)
    assert conv
    for d in range(2):
        for g in range(1, fe[d].max() + 1):
            m = fe[d] == g
            assert abs(host.y[m].mean()) < 1e-6
            for j in range(2):
                assert abs(host.W[m, j].mean()) < 1e-6


def test_demean_matches_oracle_symmetric_scheme(built):
    hdr, host = nls_panel(n_ids=300, seed=7)
    y0, W0 = host.y.copy(), host.W.copy(order="F")
    cfg = fe_runtime_config(fe_tolerance=1e-8, fe_max_iterations=10000)
    conv, iters, mu = fe_gpu_within_transform(cfg, host)
    oy, oW, _, oit, oconv, omu = O.demean_symmetric(y0, W0, host.fe_ids, 1e-8, 10000)
    assert conv and oconv
    # same scheme, same decisions: iteration counts agree and values to rounding
    assert abs(iters - oit) <= 1
    np.testing.assert_allclose(host.y, oy, atol=1e-9)
    np.testing.assert_allclose(host.W, oW, atol=1e-9)


@pytest.mark.parametrize("method", ["ap", "cg"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("clusters", [[], [1], [1, 3], [1, 2, 3]])
def test_nls_panel_gpu_conventions(built, method, precision, clusters):
    hdr, host = nls_panel(n_ids=1500, seed=11)
    cfg = fe_runtime_config(fe_tolerance=1e-8, fe_max_iterations=20000, cluster_fe_dims=clusters,
                            precision=precision, demean_cg=(method == "cg"))
    res = fe_gpu_estimate(cfg, hdr, host)
    ref = O.gpu_estimate(host.y, host.W, host.fe_ids, tol=1e-12, max_iter=200000, cluster_dims=clusters)
    assert res.converged
    assert rel(res.beta, ref.beta) < BETA_RTOL
    assert rel(res.se, ref.se) < SE_RTOL
    assert res.dof_resid == ref.stats["dof_resid"]
    assert res.dof_fes == ref.stats["dof_fes"]
    assert res.dof_model == ref.stats["dof_model"]
    assert abs(res.r2 - ref.stats["r2"]) < 1e-8
    assert abs(res.r2_within - ref.stats["r2_within"]) < 1e-8


@pytest.mark.parametrize("clusters", [[], [1, 2, 3]])
def test_nls_panel_cpu_conventions(built, clusters):
    hdr, host = nls_panel(n_ids=1500, seed=12)
    cfg = fe_runtime_config(fe_tolerance=1e-8, fe_max_iterations=20000, cluster_fe_dims=clusters,
                            se_convention="cpu")
    res = fe_gpu_estimate(cfg, hdr, host)
    ref = O.cpu_estimate(host.y, host.W, host.fe_ids, tol=1e-12, max_iter=200000, cluster_dims=clusters)
    assert rel(res.beta, ref.beta) < BETA_RTOL
    assert rel(res.se, ref.se) < SE_RTOL
    assert res.dof_resid == ref.stats["dof_resid"]


@pytest.mark.parametrize("method", ["ap", "cg"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_worker_firm_small(built, method, precision):
    hdr, host = worker_firm_panel(n_workers=20000, n_firms=2000, n_periods=10, switch_prob=0.1, seed=5)
    cfg = fe_runtime_config(fe_tolerance=1e-8, fe_max_iterations=20000, cluster_fe_dims=[1, 2, 3],
                            precision=precision, demean_cg=(method == "cg"))
    res = fe_gpu_estimate(cfg, hdr, host)
    ref = O.gpu_estimate(host.y, host.W, host.fe_ids, tol=1e-11, max_iter=200000, cluster_dims=[1, 2, 3])
    assert res.converged
    assert rel(res.beta, ref.beta) < BETA_RTOL
    assert rel(res.se, ref.se) < SE_RTOL
    assert res.dof_resid == ref.stats["dof_resid"]


def iv_case(n=6000, seed=3):
    rng = np.random.default_rng(seed)
    g = [200, 40, 6]
    fe = np.asfortranarray(np.vstack([rng.integers(1, gd + 1, n) for gd in g]).astype(np.int32))
    z = rng.standard_normal((n, 3))
    u = rng.standard_normal(n)
    x_end = z @ np.array([0.6, 0.3, -0.2]) + 0.5 * u + rng.standard_normal(n)
    x_ex = rng.standard_normal((n, 2))
    y = 0.8 * x_end + x_ex @ np.array([0.3, -0.4]) + u + 0.2 * fe[0] / 200.0
    W = np.asfortranarray(np.column_stack([x_end, x_ex]))
    return fe_host_arrays(y=y, W=W, Z=np.asfortranarray(z), fe_ids=fe)


@pytest.mark.parametrize("method", ["ap", "cg"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("clusters", [[], [1, 2]])
def test_iv_gpu_conventions(built, method, precision, clusters):
    host = iv_case()
    cfg = fe_runtime_config(fe_tolerance=1e-8, fe_max_iterations=20000, cluster_fe_dims=clusters,
                            iv_regressors=[1], precision=precision, demean_cg=(method == "cg"))
    res = fe_gpu_estimate(cfg, None, host)
    ref = O.gpu_estimate(host.y, host.W, host.fe_ids, Z=host.Z, tol=1e-12, max_iter=200000, cluster_dims=clusters,
                         iv_regressors=[1])
    assert res.is_iv and ref.stats["is_iv"]
    assert res.n_instruments == ref.stats["n_instruments"]
    assert rel(res.beta, ref.beta) < BETA_RTOL
    assert rel(res.se, ref.se) < SE_RTOL


@pytest.mark.parametrize("method", ["ap", "cg"])
def test_deterministic_bitwise(built, method):
    hdr, host = worker_firm_panel(n_workers=5000, n_firms=700, n_periods=8, switch_prob=0.2, seed=9)
    cfg = fe_runtime_config(fe_tolerance=1e-8, fe_max_iterations=20000, cluster_fe_dims=[1, 2], precision="mixed",
                            demean_cg=(method == "cg"))
    a = fe_gpu_estimate(cfg, hdr, host)
    b = fe_gpu_estimate(cfg, hdr, host)
    assert a.fe_iterations == b.fe_iterations
    assert np.array_equal(a.beta, b.beta)
    assert np.array_equal(a.se, b.se)



def many_group_case(n=40000, g=(3000, 400, 90), k=3, seed=13):
    # every FE dimension above the dense count-matrix limit (64 groups), or, with
    # k > 31, every dimension swept (C > 32): the CG's Schur form then sweeps
    # two dimensions besides the eliminated one
    rng = np.random.default_rng(seed)
    fe = np.asfortranarray(np.vstack([rng.integers(1, gd + 1, n) for gd in g]).astype(np.int32))
    W = np.asfortranarray(rng.standard_normal((n, k)))
    eff = sum(rng.normal(0, 0.5, gd)[fe[d] - 1] for d, gd in enumerate(g))
    y = W @ rng.standard_normal(k) + eff + rng.standard_normal(n)
    return fe_host_arrays(y=y, W=W, Z=np.zeros((n, 0), order="F"), fe_ids=fe)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("g,k", [((3000, 400, 90), 3), ((3000, 400, 30), 33)])
def test_cg_schur_two_swept_dimensions(built, precision, g, k):
    host = many_group_case(g=g, k=k)
    cfg = fe_runtime_config(fe_tolerance=1e-8, fe_max_iterations=20000, cluster_fe_dims=[1, 2],
                            precision=precision, demean_cg=True)
    res = fe_gpu_estimate(cfg, None, host)
    ref = O.gpu_estimate(host.y, host.W, host.fe_ids, tol=1e-11, max_iter=200000, cluster_dims=[1, 2])
    assert res.converged and res.solver_info == 0
    # the operator and its Schur-diagonal preconditioner are exact: a handful of
    # iterations (8 here); an operator that misses the primary's cross-chunk
    # group sums took 300-700 and still converged
    assert res.fe_iterations < 60
    assert rel(res.beta, ref.beta) < BETA_RTOL
    assert rel(res.se, ref.se) < SE_RTOL


def test_verify_fp64_reports_per_coefficient_errors(built):
    """verify_fp64: the mixed-precision fit carries, per coefficient and SE,
    its relative error against the plain FP64 form on the same inputs; both
    fits are within the parity bar of the oracle."""
    hdr, host = worker_firm_panel(n_workers=20000, n_firms=2000, n_periods=10, switch_prob=0.1, seed=6)
    cfg = fe_runtime_config(fe_tolerance=1e-8, fe_max_iterations=20000, cluster_fe_dims=[1, 2, 3],
                            precision="mixed", demean_cg=True, verify_fp64=True)
    res = fe_gpu_estimate(cfg, hdr, host)
    assert res.beta_rel_err_vs_fp64 is not None and res.se_rel_err_vs_fp64 is not None
    assert res.beta_rel_err_vs_fp64.shape == res.beta.shape and res.se_rel_err_vs_fp64.shape == res.se.shape
    np.testing.assert_allclose(res.beta_rel_err_vs_fp64,
                               np.abs(res.beta - res.beta_fp64) / np.abs(res.beta_fp64), rtol=1e-12, atol=0)
    assert np.max(res.beta_rel_err_vs_fp64) < BETA_RTOL
    assert np.max(res.se_rel_err_vs_fp64) < SE_RTOL
    ref = O.gpu_estimate(host.y, host.W, host.fe_ids, tol=1e-11, max_iter=200000, cluster_dims=[1, 2, 3])
    assert rel(res.beta_fp64, ref.beta) < BETA_RTOL
    assert rel(res.se_fp64, ref.se) < SE_RTOL
