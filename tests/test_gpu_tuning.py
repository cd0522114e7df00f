"""Every value of every launch-shape knob gives the same fit, within the
parity bar, as the defaults: the knobs select between equivalent kernel forms
(count-matrix pass on tensor or CUDA cores, CG operator sweep columns per
pass, split-FP32 Gram threshold, CG loop as a graph or host-driven)."""
import numpy as np
import pytest

from fe_gpu_gb300 import autotune as A
from fe_gpu_gb300 import fe_gpu_estimate, fe_runtime_config
from fe_gpu_gb300.synth import worker_firm_panel
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def panel():
    return worker_firm_panel(n_workers=20000, n_firms=2000, n_periods=12, switch_prob=0.1, seed=9)


@pytest.mark.parametrize("key,value", [(k, v) for k, vs in A.KNOBS.items() for v in vs])
def test_knob_values_agree_with_oracle(built, panel, key, value):
    hdr, host = panel
    cfg = fe_runtime_config(fe_tolerance=1e-8, fe_max_iterations=20000, cluster_fe_dims=[1, 2, 3],
                            precision="mixed", demean_cg=True)
    A.reset()
    A.set_knob(key, value)
    try:
        res = fe_gpu_estimate(cfg, hdr, host, tune=False)
    finally:
        A.reset()
    ref = O.gpu_estimate(host.y, host.W, host.fe_ids, tol=1e-11, max_iter=200000, cluster_dims=[1, 2, 3])
    assert res.converged
    assert np.max(np.abs(res.beta - ref.beta) / np.abs(ref.beta)) < 1e-6
    assert np.max(np.abs(res.se - ref.se) / np.abs(ref.se)) < 1e-5
    assert res.dof_resid == ref.stats["dof_resid"]
