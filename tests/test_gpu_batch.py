"""Batched specifications (fegb_estimate_batch) against the same fits run
one by one and against the oracle: uneven sizes, 1-3 FE dimensions, 2-24
regressors, OLS and 2SLS, 1-3-way clustering; both the batched estimation of
each column class (default) and the specification-by-specification path
(knob batch_estimator = 0)."""
import numpy as np
import pytest

from fe_gpu_gb300.estimator import (DeviceBuffer, fe_batch_spec, fe_gpu_estimate_batch, fe_gpu_estimate_device,
                                    fe_runtime_config)
from fe_gpu_gb300.synth import batch_specs
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _upload(specs):
    bufs, out = [], []
    for host, extra in specs:
        n = host.y.shape[0]
        by = DeviceBuffer.from_array(host.y)
        bW = DeviceBuffer.from_array(np.asfortranarray(host.W))
        bZ = DeviceBuffer.from_array(np.asfortranarray(host.Z)) if host.Z.shape[1] else None
        bf = [DeviceBuffer.from_array(np.ascontiguousarray(host.fe_ids[d])) for d in range(host.fe_ids.shape[0])]
        bufs.append((by, bW, bZ, bf))
        out.append(fe_batch_spec(n=n, k=host.W.shape[1], l=host.Z.shape[1], d_y=by.ptr, d_W=bW.ptr,
                                 d_Z=bZ.ptr if bZ else None, d_fe_ids=[b.ptr for b in bf],
                                 cluster_fe_dims=extra["cluster_fe_dims"], iv_regressors=extra["iv_regressors"]))
    return bufs, out


def rel(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


@pytest.mark.parametrize("batched", [1, 0])
@pytest.mark.parametrize("precision,cg", [("fp64", False), ("mixed", True)])
def test_batch_matches_single_fits_and_oracle(built, precision, cg, batched):
    from fe_gpu_gb300 import autotune as A

    specs = batch_specs(n_specs=12, total_rows=300_000, row_range=(2_000, 60_000), seed=1)
    assert sum(1 for _, e in specs if e["iv_regressors"]) >= 3
    bufs, dspecs = _upload(specs)
    cfg = fe_runtime_config(fe_tolerance=1e-8, fe_max_iterations=100000, precision=precision, demean_cg=cg)
    A.reset()
    A.set_knob("batch_estimator", batched)
    try:
        batch = fe_gpu_estimate_batch(cfg, dspecs)
    finally:
        A.reset()
    assert len(batch) == len(specs)
    for (host, extra), sp, rb in zip(specs, dspecs, batch):
        c1 = fe_runtime_config(fe_tolerance=1e-8, fe_max_iterations=100000, precision=precision, demean_cg=cg,
                               cluster_fe_dims=extra["cluster_fe_dims"], iv_regressors=extra["iv_regressors"])
        rs = fe_gpu_estimate_device(c1, sp.n, sp.k, sp.l, sp.d_y, sp.d_W, sp.d_Z, sp.d_fe_ids)
        ref = O.gpu_estimate(host.y, host.W, host.fe_ids, Z=host.Z, tol=1e-12, max_iter=200000,
                             cluster_dims=extra["cluster_fe_dims"], iv_regressors=extra["iv_regressors"])
        assert rb.converged
        for r in (rs,):
            assert rb.dof_model == r.dof_model and rb.dof_fes == r.dof_fes and rb.dof_resid == r.dof_resid
            assert rb.is_iv == r.is_iv and rb.n_instruments == r.n_instruments
        assert rb.is_iv == bool(ref.stats["is_iv"])
        assert rb.dof_resid == ref.stats["dof_resid"]
        assert rel(rb.beta, ref.beta) < 1e-6
        assert rel(rb.se, ref.se) < 1e-5
        assert abs(rb.r2 - rs.r2) < 1e-7 and abs(rb.r2_within - rs.r2_within) < 1e-7
        assert rb.psd_fix_applied == r.psd_fix_applied
        assert abs(rb.tss_total - rs.tss_total) <= 1e-9 * abs(rs.tss_total)
        assert abs(rb.rss - rs.rss) <= 1e-7 * abs(rs.rss)


def test_batch_64_specs_match_oracle(built):
    """64 specifications (the batched estimator's path) against the oracle."""
    specs = batch_specs(n_specs=64, total_rows=1_500_000, row_range=(2_000, 80_000), seed=3)
    bufs, dspecs = _upload(specs)
    cfg = fe_runtime_config(fe_tolerance=1e-8, fe_max_iterations=100000, precision="mixed", demean_cg=True)
    from fe_gpu_gb300 import autotune as A

    A.reset()
    A.set_knob("batch_estimator", 1)
    try:
        batch = fe_gpu_estimate_batch(cfg, dspecs)
    finally:
        A.reset()
    for (host, extra), rb in zip(specs, batch):
        ref = O.gpu_estimate(host.y, host.W, host.fe_ids, Z=host.Z, tol=1e-12, max_iter=200000,
                             cluster_dims=extra["cluster_fe_dims"], iv_regressors=extra["iv_regressors"])
        assert rb.converged
        assert rb.dof_resid == ref.stats["dof_resid"] and rb.dof_model == ref.stats["dof_model"]
        assert rel(rb.beta, ref.beta) < 1e-6
        assert rel(rb.se, ref.se) < 1e-5


def test_batch_rejects_bad_specs(built):
    from fe_gpu_gb300 import _native as N

    specs = batch_specs(n_specs=2, total_rows=10_000, row_range=(2_000, 8_000), seed=1)
    bufs, dspecs = _upload(specs)
    cfg = fe_runtime_config(drop_singletons=True)
    with pytest.raises(N.FeGpuError):
        fe_gpu_estimate_batch(cfg, dspecs)
