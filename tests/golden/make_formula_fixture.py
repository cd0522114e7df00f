"""Builds formula_expansion_log.json from the reference's own example run:
the six fe_gpu formulas of Examples/01TESTS_fe_gpu_small.sh and, for each,
the coefficient names, estimator line, endogenous columns and dof printed in
Examples/01TESTS_fe_gpu_small_output.txt. Run where the reference source tree
is present, with FE_GPU_REFERENCE naming its root."""
import json
import os
import re
from pathlib import Path

if not os.environ.get("FE_GPU_REFERENCE"):
    raise SystemExit("set FE_GPU_REFERENCE to the root of the reference source tree")
REF = Path(os.environ["FE_GPU_REFERENCE"])
OUT = Path(__file__).resolve().parent / "formula_expansion_log.json"


def main():
    sh = (REF / "Examples/01TESTS_fe_gpu_small.sh").read_text().splitlines()
    formulas = [re.search(r'--formula "([^"]+)"', ln).group(1) for ln in sh
                if "build/src/fe_gpu" in ln and "--formula" in ln and not ln.lstrip().startswith("#")]
    log = (REF / "Examples/01TESTS_fe_gpu_small_output.txt").read_text().splitlines()
    runs = []
    cur = None
    in_table = 0
    for no, ln in enumerate(log, 1):
        if ln.startswith("Loaded dataset header:"):
            cur = {"log_line": no, "names": []}
            runs.append(cur)
            in_table = 0
            continue
        if cur is None:
            continue
        m = re.match(r"Estimator: (.*)$", ln)
        if m:
            cur["estimator"] = m.group(1).strip()
            mi = re.search(r"with (\d+) instruments", ln)
            cur["n_instruments"] = int(mi.group(1)) if mi else 0
        m = re.match(r"Endogenous regressors \(--iv-cols\): \[(.*)\]", ln)
        if m:
            cur["endogenous"] = m.group(1).split(",")
        if re.match(r"\s+-{10,}", ln):
            in_table += 1
            continue
        if in_table == 1:
            parts = ln.split()
            if len(parts) == 7:
                cur["names"].append(parts[0])
        m = re.match(r"\s+dof \(model\): (\d+), dof \(residuals\): (\d+)", ln)
        if m:
            cur["dof_model"] = int(m.group(1))
            cur["dof_resid"] = int(m.group(2))
    assert len(runs) == len(formulas), (len(runs), len(formulas))
    for r, f in zip(runs, formulas):
        r["formula"] = f
        r.setdefault("endogenous", [])
    OUT.write_text(json.dumps({"source": "Examples/01TESTS_fe_gpu_small.sh and _output.txt (fe_gpu runs)",
                               "raw_regressors": ["hours", "ttl_exp", "union", "tenure", "wks_ue", "ind_code", "msp"],
                               "raw_instruments": ["wks_work", "ind_code"],
                               "levels": {"ind_code": list(range(1, 13)), "msp": [0, 1]},
                               "runs": runs}, indent=1) + "\n")
    print(f"wrote {OUT} ({len(runs)} runs)")


if __name__ == "__main__":
    main()
