"""Pins of the CPU oracle (test infrastructure) before it is trusted as the
checker of the CUDA path:

* the reference's own known-answer tests (tests/test_gpu_regression.f90,
  tests/test_gpu_demean.f90);
* the reference's compiled multi-way cluster-id builder
  (src/core/cluster_id_builder.c, built into oracle/_ref where the reference
  tree is present): bit-identical ids;
* independent numpy restatements of the estimator formulas
  (src/core/fe_pipeline.f90): explicit-dummy least squares, homoskedastic and
  Cameron-Gelbach-Miller clustered covariances, the PSD fix;
* the committed golden fixture of the reference's synthetic generator.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = Path(__file__).resolve().parent / "golden"


def six_row():
    W = np.array([[1.0, -2.0], [1.5, 0.5], [-0.5, 1.0], [-1.0, -1.5], [0.25, 0.75], [2.0, 1.25]])
    fe = np.array([[1, 1, 2, 2, 3, 3], [1, 2, 1, 2, 1, 2]], dtype=np.int32)
    y = W @ np.array([1.5, -0.75]) + np.array([0.5, -0.25, 0.8])[fe[0] - 1] + np.array([-0.4, 0.2])[fe[1] - 1]
    return y, W, fe


@pytest.mark.parametrize("conv", ["cpu", "gpu"])
def test_regression_known_answer(conv):
    y, W, fe = six_row()
    fn = O.cpu_estimate if conv == "cpu" else O.gpu_estimate
    r = fn(y, W, fe, tol=1e-10, max_iter=500)
    assert r.stats["converged"] and r.stats["solver_info"] == 0
    np.testing.assert_allclose(r.beta, [1.5, -0.75], atol=1e-8, rtol=0)


@pytest.mark.parametrize("scheme", ["forward", "symmetric"])
def test_demean_known_answer(scheme):
    y = np.array([1.0, 2.0, 3.0, -2.0, -1.0, 0.5])
    W = np.array([[1.0, 0.0], [1.5, -2.0], [-0.5, 1.0], [-1.0, 0.5], [2.0, 1.5], [-0.5, -1.0]])
    fe = np.array([[1, 1, 2, 2, 3, 3], [1, 2, 1, 2, 1, 2]], dtype=np.int32)
    if scheme == "forward":
        yd, Wd, it, conv, mu = O.demean_forward(y, W, fe, 1e-8, 200)
    else:
        yd, Wd, _, it, conv, mu = O.demean_symmetric(y, W, fe, 1e-8, 200)
    assert conv
    for d in range(2):
        for g in range(1, 4 if d == 0 else 3):
            m = fe[d] == g
            assert abs(yd[m].mean()) < 1e-6 and np.all(np.abs(Wd[m].mean(axis=0)) < 1e-6)


def random_ids(rng, n, sizes):
    return np.asfortranarray(np.vstack([rng.integers(1, s + 1, n) for s in sizes]).astype(np.int32))


@pytest.mark.parametrize("sizes,subset", [((50, 7, 3), [1, 2]), ((50, 7, 3), [3, 1]), ((50, 7, 3), [1, 2, 3]),
                                          ((1000, 1000, 1000), [2, 3, 1]), ((4, 4, 4), [2])])
def test_cluster_ids_match_reference_builder(sizes, subset):
    if O.ref_lib() is None:
        pytest.skip("reference cluster builder not built here (reference tree absent)")
    rng = np.random.default_rng(len(subset) * 7 + sizes[0])
    fe = random_ids(rng, 5000, sizes)
    ours, nc, st = O.cluster_ids(fe, sizes, subset)
    ref, rnc, rst = O.cluster_ids(fe, sizes, subset, use_reference=True)
    assert st == 0 and rst == 0
    assert nc == rnc
    np.testing.assert_array_equal(ours, ref)


def test_cluster_ids_first_appearance_matches_reference_builder():
    # span above 2^62 switches the reference to first-appearance (hash) ids
    if O.ref_lib() is None:
        pytest.skip("reference cluster builder not built here (reference tree absent)")
    rng = np.random.default_rng(3)
    big = 2_000_000_000
    fe = np.asfortranarray(np.vstack([rng.integers(1, 40, 3000), rng.integers(1, 40, 3000),
                                      rng.integers(1, 40, 3000)]).astype(np.int32))
    sizes = [big, big, big]
    ours, nc, st = O.cluster_ids(fe, sizes, [1, 2, 3])
    ref, rnc, rst = O.cluster_ids(fe, sizes, [1, 2, 3], use_reference=True)
    assert st == 0 and rst == 0 and nc == rnc
    np.testing.assert_array_equal(ours, ref)


def test_cluster_ids_are_sorted_key_ranks():
    rng = np.random.default_rng(1)
    sizes = (30, 5, 4)
    fe = random_ids(rng, 2000, sizes)
    ids, nc, st = O.cluster_ids(fe, sizes, [2, 1])
    key = (fe[1].astype(np.int64) - 1) + (fe[0].astype(np.int64) - 1) * sizes[1]
    u, inv = np.unique(key, return_inverse=True)
    np.testing.assert_array_equal(ids, inv + 1)
    assert nc == u.size


def test_compaction_and_group_sizes():
    raw = np.array([17, -3, 17, 5, 99, -3, 5], dtype=np.int32)
    out, lv = O.compact_ids(raw)
    u, inv = np.unique(raw, return_inverse=True)  # = pandas factorize(sort=True)
    np.testing.assert_array_equal(out, inv + 1)
    assert lv == u.size
    fe = np.array([[1, 4, 2], [3, 3, 1]], dtype=np.int32)
    np.testing.assert_array_equal(O.group_sizes(fe), [4, 3])
    with pytest.raises(ValueError):
        O.group_sizes(np.array([[1, 0, 2]], dtype=np.int32))


def test_singletons_fixpoint():
    fe = np.array([[1, 1, 2, 3, 3, 4], [1, 2, 2, 1, 1, 2]], dtype=np.int32)
    keep, dropped = O.drop_singletons(fe)
    # row 2 (group 2 of dim 1) and row 5 (group 4) are singletons; after removing them
    # dim 2 group 2 keeps rows 1; row 1 then becomes a singleton in dim 2 ... iterate
    rows = np.ones(6, bool)
    changed = True
    while changed:
        changed = False
        for d in range(2):
            vals, cnt = np.unique(fe[d][rows], return_counts=True)
            single = set(vals[cnt == 1])
            for i in np.nonzero(rows)[0]:
                if fe[d][i] in single:
                    rows[i] = False
                    changed = True
    np.testing.assert_array_equal(keep, rows)
    assert dropped == int((~rows).sum())


def dummies(ids):
    g = ids.max()
    D = np.zeros((ids.size, g))
    D[np.arange(ids.size), ids - 1] = 1.0
    return D


def small_panel(seed=0, n=400):
    rng = np.random.default_rng(seed)
    fe = random_ids(rng, n, (40, 6, 5))
    W = rng.standard_normal((n, 3))
    y = W @ np.array([0.5, -1.0, 0.25]) + rng.standard_normal(n) + 0.3 * fe[0] / 40
    return y, np.asfortranarray(W), fe


def test_fwl_coefficients_and_homoskedastic_se():
    y, W, fe = small_panel()
    n, k = W.shape
    D = np.hstack([dummies(fe[0]), dummies(fe[1])[:, 1:], dummies(fe[2])[:, 1:]])
    X = np.hstack([W, D])
    coef, *_ = np.linalg.lstsq(X, y, rcond=None)
    r = O.gpu_estimate(y, W, fe, tol=1e-13, max_iter=100000)
    np.testing.assert_allclose(r.beta, coef[:k], rtol=1e-9, atol=1e-12)
    # homoskedastic SE with the GPU-path dof (fe_pipeline.f90:1171-1198)
    resid = y - X @ coef
    G = O.group_sizes(fe)
    df = n - (k + int(np.sum(G - 1)) + 1)
    Wt = W - D @ np.linalg.lstsq(D, W, rcond=None)[0]
    V = resid @ resid / df * np.linalg.inv(Wt.T @ Wt)
    np.testing.assert_allclose(r.se, np.sqrt(np.diag(V)), rtol=1e-9)
    assert r.stats["dof_resid"] == df
    # CPU path: sigma^2 = RSS / (N - K) (fe_pipeline.f90:185-187)
    rc = O.cpu_estimate(y, W, fe, tol=1e-13, max_iter=100000)
    np.testing.assert_allclose(rc.beta, coef[:k], rtol=1e-9, atol=1e-12)
    Vc = resid @ resid / (n - k) * np.linalg.inv(Wt.T @ Wt)
    np.testing.assert_allclose(rc.se, np.sqrt(np.diag(Vc)), rtol=1e-9)


def cgm_numpy(resid, Wt, fe, dims, scalar):
    Qi = np.linalg.inv(Wt.T @ Wt)
    V = np.zeros_like(Qi)
    for mask in range(1, 1 << len(dims)):
        sub = [dims[j] for j in range(len(dims)) if mask & (1 << j)]
        key = np.zeros(fe.shape[1], dtype=np.int64)
        for d in sub:
            key = key * (fe[d - 1].max() + 1) + fe[d - 1]
        _, cid = np.unique(key, return_inverse=True)
        S = np.zeros((cid.max() + 1, Wt.shape[1]))
        np.add.at(S, cid, resid[:, None] * Wt)
        V += (1 if len(sub) % 2 else -1) * Qi @ (S.T @ S) @ Qi
    return V * scalar


@pytest.mark.parametrize("dims", [[1], [1, 3], [1, 2, 3]])
def test_clustered_se_formulas(dims):
    y, W, fe = small_panel(seed=5)
    n, k = W.shape
    D = np.hstack([dummies(fe[0]), dummies(fe[1])[:, 1:], dummies(fe[2])[:, 1:]])
    Wt = W - D @ np.linalg.lstsq(D, W, rcond=None)[0]
    yt = y - D @ np.linalg.lstsq(D, y, rcond=None)[0]
    beta = np.linalg.solve(Wt.T @ Wt, Wt.T @ yt)
    resid = yt - Wt @ beta
    G = O.group_sizes(fe)
    gmin = min(int(G[d - 1]) for d in dims)
    # GPU path scalar: (N-1)/(N-K-1) * G/(G-1) when clustering on an FE dim (fe_pipeline.f90:1348-1360)
    V = cgm_numpy(resid, Wt, fe, dims, (n - 1) / (n - k - 1) * gmin / (gmin - 1))
    w, vec = np.linalg.eigh(V)
    Vp = (vec * np.maximum(w, 0)) @ vec.T
    r = O.gpu_estimate(y, W, fe, tol=1e-13, max_iter=100000, cluster_dims=dims)
    np.testing.assert_allclose(r.beta, beta, rtol=1e-9)
    np.testing.assert_allclose(r.se, np.sqrt(np.diag(Vp)), rtol=1e-8)
    assert r.stats["dof_resid"] == gmin - 1
    # CPU path scalar: (N-1)/(N-K) * G/(G-1), no PSD fix (fe_pipeline.f90:466-480)
    Vc = cgm_numpy(resid, Wt, fe, dims, (n - 1) / (n - k) * gmin / (gmin - 1))
    rc = O.cpu_estimate(y, W, fe, tol=1e-13, max_iter=100000, cluster_dims=dims)
    np.testing.assert_allclose(rc.se, np.sqrt(np.clip(np.diag(Vc), 0, None)), rtol=1e-8)


def test_iv_two_stage_least_squares():
    rng = np.random.default_rng(9)
    n = 500
    fe = random_ids(rng, n, (30, 4))
    z = rng.standard_normal((n, 2))
    u = rng.standard_normal(n)
    xe = z @ [0.7, -0.4] + 0.5 * u + rng.standard_normal(n)
    xx = rng.standard_normal(n)
    y = 1.2 * xe - 0.3 * xx + u
    W = np.asfortranarray(np.column_stack([xe, xx]))
    D = np.hstack([dummies(fe[0]), dummies(fe[1])[:, 1:]])

    def tilde(a):
        return a - D @ np.linalg.lstsq(D, a, rcond=None)[0]

    Wt, yt, Zt = tilde(W), tilde(y), tilde(z)
    Za = np.column_stack([Wt[:, 1], Zt])
    Xh = Za @ np.linalg.solve(Za.T @ Za, Za.T @ Wt)
    beta = np.linalg.solve(Xh.T @ Wt, Xh.T @ yt)
    r = O.gpu_estimate(y, W, fe, Z=np.asfortranarray(z), tol=1e-13, max_iter=100000, iv_regressors=[1])
    assert r.stats["is_iv"] and r.stats["n_instruments"] == 3
    np.testing.assert_allclose(r.beta, beta, rtol=1e-8)


def test_psd_fix_and_cholesky():
    A = np.array([[2.0, 1.9, 0.0], [1.9, 1.0, 0.3], [0.0, 0.3, 1.5]])
    fixed, applied = O.psd_fix(A)
    w, v = np.linalg.eigh(A)
    assert applied and w.min() < 0
    np.testing.assert_allclose(fixed, (v * np.maximum(w, 0)) @ v.T, atol=1e-12)
    Q = np.array([[4.0, 1.0, 0.5], [1.0, 3.0, 0.2], [0.5, 0.2, 2.0]])
    b = np.array([1.0, -2.0, 0.5])
    beta, Qi, info = O.chol_solve_invert(Q, b)
    assert info == 0
    np.testing.assert_allclose(beta, np.linalg.solve(Q, b), rtol=1e-13)
    np.testing.assert_allclose(Qi, np.linalg.inv(Q), rtol=1e-13)


def test_reference_generator_fixture():
    """fe_gpu_gb300.synth.reference_panel reproduces the reference's own
    generator output (fixture made by tests/golden/make_fixtures.py)."""
    from fe_gpu_gb300.synth import reference_panel

    fx = np.load(GOLDEN / "reference_generator_small.npz")
    meta = json.loads(str(fx["meta"]))
    hdr, host, coeffs = reference_panel(**meta)
    np.testing.assert_array_equal(host.fe_ids, fx["fe_ids"])
    np.testing.assert_allclose(host.W, fx["W"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(host.y, fx["y"], rtol=1e-15, atol=1e-14)
    np.testing.assert_allclose(coeffs, fx["coeffs"], rtol=0, atol=0)
