"""bench.py's reference arm (the oracle port on the host cores) prints one JSON
line with the contract's keys; run here on the small nls panel."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.timeout(300)
def test_reference_arm_json_line(built):
    env = dict(os.environ, OMP_NUM_THREADS="2")
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload", "nls_panel",
                          "--steps", "1", "--warmup", "0"], cwd=ROOT, env=env, capture_output=True, text=True,
                         timeout=280)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]
    assert d["config"]["workload"].startswith("nls_panel")
    # the line reports what was fitted: config.rows is the sample's row count,
    # and ms_per_step the measured time of one fit of it (the value's inverse)
    from fe_gpu_gb300.synth import nls_panel

    rows = nls_panel(seed=20261203)[1].y.shape[0]
    assert d["config"]["rows"] == rows
    assert abs(d["ms_per_step"] - rows / d["value"] * 1e3) <= 1e-6 * d["ms_per_step"]
    assert d["steps"] == 1 and len(d["config"]["step_seconds_all"]) == 1
    assert abs(d["config"]["step_seconds_all"][0] * 1e3 - d["ms_per_step"]) <= 1e-6 * d["ms_per_step"]


def test_sample_of_150m_workload_is_bounded():
    """The CPU sample of the 150M-row workload is the same design at 1/200
    (25,000 workers x 30 periods = 750k rows over 5,000 firms)."""
    sys.path.insert(0, str(ROOT))
    import bench

    w = bench.WORKLOADS["worker_firm_150M"]
    assert w["cpu_sample_div"] == 200
    assert bench.workload_rows("worker_firm_150M") == 150_000_000
    assert w["n_workers"] // w["cpu_sample_div"] * w["n_periods"] == 750_000
