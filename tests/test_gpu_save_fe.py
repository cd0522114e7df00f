"""--save-fe on the device (fegb_reconstruct_fe) against the oracle's
restatement of reconstruct_and_save_fixed_effects: same FE values (both
converged to the tolerance), same counts, same sweep count."""
import numpy as np
import pytest

from fe_gpu_gb300.bin_io import fe_host_arrays
from fe_gpu_gb300.estimator import fe_gpu_estimate, fe_gpu_reconstruct_fe, fe_runtime_config, write_fe_outputs
from fe_gpu_gb300.synth import worker_firm_panel
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [0, 1])
def test_reconstruction_matches_oracle(built, seed, tmp_path):
    hdr, host = worker_firm_panel(n_workers=3000, n_firms=300, n_periods=8, switch_prob=0.2, seed=seed)
    cfg = fe_runtime_config(fe_tolerance=1e-10, fe_max_iterations=100000)
    res = fe_gpu_estimate(cfg, hdr, host)
    v, c, it, mu = fe_gpu_reconstruct_fe(cfg, host, res.beta)
    rv, rc, rit, rmu = O.reconstruct_fe(host.y, host.W, host.fe_ids, res.beta, tol=1e-10, max_iter=100000)
    assert mu < 1e-10
    assert abs(it - rit) <= 1
    scale = max(np.max(np.abs(x)) for x in rv)
    for d in range(len(rv)):
        assert np.array_equal(c[d], rc[d])
        assert np.max(np.abs(v[d] - rv[d])) < 1e-8 * scale
    paths = write_fe_outputs(str(tmp_path / "fe"), v, c)
    assert len(paths) == host.fe_ids.shape[0]
    lines = open(paths[0]).read().splitlines()
    assert lines[0] == "level_id,fe_value" and len(lines) == 1 + int((c[0] > 0).sum())
