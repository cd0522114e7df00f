"""The reference's own 150M-row panel against the reference's printed fit.

The panel is regenerated with fe_gpu_gb300.synth.reference_panel (the
reference generator restated; checked bit for bit against the generator at
small size in test_oracle_golden.py) with the generator's default seed, and
fitted like the reference's log run (fe-tol 1e-8, FEs worker/firm/time,
clustered on all three). The printed values carry 7 significant digits, so
coefficients and SEs are compared to 1e-6 relative.

The case needs about 25 GB of host memory and half a minute of generation
and fitting. It runs whenever the host has at least 48 GB available
(MemAvailable), unless FEGB_MASSIVE=0; FEGB_MASSIVE=1 forces it.
"""
import json
import os
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = json.loads((Path(__file__).resolve().parent / "golden" / "massive_panel_log.json").read_text())


def _mem_available_gb() -> float:
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) / 1e6
    except OSError:
        pass
    return 0.0


def _massive_enabled() -> bool:
    flag = os.environ.get("FEGB_MASSIVE")
    if flag is not None:
        return flag == "1"
    return _mem_available_gb() >= 48.0


@pytest.fixture(scope="module")
def massive_panel():
    from fe_gpu_gb300.synth import reference_panel

    g = GOLD["generator"]
    return reference_panel(workers=g["workers"], firms=g["firms"], periods=g["periods"],
                           extra_vars=g["extra_vars"], seed=g["seed"])


@pytest.mark.skipif(not _massive_enabled(), reason="needs 48 GB of available host memory (150M rows)")
@pytest.mark.parametrize("precision,cg", [("mixed", True), ("fp64", False)])
def test_massive_panel_matches_reference_log(built, massive_panel, precision, cg):
    from fe_gpu_gb300 import fe_gpu_estimate, fe_runtime_config

    hdr, host, coeffs = massive_panel
    # the generator printed its drawn extra coefficients
    assert list(coeffs) == GOLD["generator_printed_extra_coefficients"]
    cfg = fe_runtime_config(fe_tolerance=GOLD["fit"]["fe_tol"], fe_max_iterations=100000,
                            cluster_fe_dims=GOLD["fit"]["cluster_dims"], precision=precision, demean_cg=cg)
    res = fe_gpu_estimate(cfg, hdr, host)
    print("beta", list(res.beta), "se", list(res.se), "iters", res.fe_iterations, "time", res.stats["time_total"])
    assert res.converged
    np.testing.assert_allclose(res.beta, GOLD["beta"], rtol=1e-6)
    np.testing.assert_allclose(res.se, GOLD["se"], rtol=1e-6)
    assert res.dof_model == GOLD["dof_model"]
    assert res.dof_resid == GOLD["dof_resid"]
    assert abs(res.r2 - GOLD["r2"]) < 1e-5
    assert abs(res.r2_adj - GOLD["r2_adj"]) < 1e-5
    assert abs(res.r2_within - GOLD["r2_within"]) < 1e-5
