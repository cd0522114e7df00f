"""Autotuner of the library's launch-shape knobs (fegb_set_tuning).

The knobs select, for a problem shape, between equivalent forms of the hot
kernels: the count-matrix pass on the tensor cores or the CUDA cores, the
number of table columns one CG operator sweep carries per pass (4, 8 or all),
the output size from which Gram products use the split-FP32 form, whether
the CG loop runs as a CUDA graph, and whether operator sweeps of streams with
short groups run one thread per group. None changes the result beyond rounding.

    python -m fe_gpu_gb300.autotune [--out PATH] [--repeats R] [--quick]

times every candidate of every knob (coordinate descent: one knob at a time,
the others at their best so far) on seeded synthetic panels of a few shape
classes, and writes the winners to a JSON table (default
fe_gpu_gb300/tuning_gb300.json, committed with the package). A fit applies the
entry of the nearest shape class (same column class, nearest log row count)
before it runs, through apply_for_shape(); FEGB_TUNING=off skips that, and
FEGB_TUNING=<path> reads another table.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import time
from pathlib import Path
from typing import Optional

from . import _native as N

TABLE = Path(__file__).resolve().parent / "tuning_gb300.json"

KNOBS = {
    "dense_form": [1, 0],
    "cg_cols_per_pass": [0, 8, 4],
    "split_gram_pairs_per_col": [3, 1, 8],
    "cg_graph": [1, 0],
    "cg_short_groups": [1, 0],
}


def set_knob(key: str, value: int) -> None:
    N.check(N.lib().fegb_set_tuning(key.encode(), int(value)), "fegb_set_tuning")


def get_knob(key: str) -> int:
    import ctypes as C

    v = C.c_int(0)
    N.check(N.lib().fegb_get_tuning(key.encode(), C.byref(v)), "fegb_get_tuning")
    return v.value


def reset() -> None:
    N.check(N.lib().fegb_reset_tuning(), "fegb_reset_tuning")


def column_class(columns: int) -> int:
    """Columns (1 + k + l) bucketed as the kernels' register tiles are: 4, 8,
    9, 12, 16, then multiples of 16."""
    for c in (4, 8, 9, 12, 16):
        if columns <= c:
            return c
    return (columns + 15) // 16 * 16


# ---------------------------------------------------------------- applying

_table_cache: dict = {}


def _load_table(path: Path) -> Optional[dict]:
    key = str(path)
    if key not in _table_cache:
        try:
            _table_cache[key] = json.loads(path.read_text())
        except (OSError, ValueError):
            _table_cache[key] = None
    return _table_cache[key]


def active_table() -> Optional[dict]:
    """The table fits apply: FEGB_TUNING=<path>, else the packaged one; None
    with FEGB_TUNING=off or when there is no table."""
    src = os.environ.get("FEGB_TUNING", "")
    if src.lower() == "off":
        return None
    return _load_table(Path(src) if src else TABLE)


def entry_for_shape(rows: int, columns: int, table: Optional[dict] = None) -> Optional[dict]:
    """The table entry of the same column class with the nearest log row
    count (None without a table or an entry of that column class)."""
    if table is None:
        table = active_table()
    if not table:
        return None
    cc = column_class(columns)
    best, best_d = None, math.inf
    for e in table.get("entries", []):
        if e.get("column_class") != cc:
            continue
        d = abs(math.log(max(rows, 1)) - math.log(max(e.get("rows", 1), 1)))
        if d < best_d:
            best, best_d = e, d
    return best


def apply_for_shape(rows: int, columns: int, table: Optional[dict] = None) -> Optional[dict]:
    """With a table: every knob back to its default, then the knobs of the
    matching entry. Returns the entry applied, or None. Without a table (or
    with FEGB_TUNING=off) the knobs are left as they are."""
    if table is None:
        table = active_table()
    if not table:
        return None
    e = entry_for_shape(rows, columns, table)
    reset()
    if e is None:
        return None
    for k, v in e.get("best", {}).items():
        if k in KNOBS:
            set_knob(k, v)
    return e


# ------------------------------------------------------------------ tuning

def _shapes(quick: bool):
    from .synth import nls_panel, worker_firm_panel

    out = [("nls_panel", lambda: nls_panel(seed=20261203))]
    out.append(("worker_firm_2M", lambda: worker_firm_panel(n_workers=100_000, n_firms=10_000, n_periods=20,
                                                            switch_prob=0.1, n_reg=8, seed=20261204)))
    if not quick:
        out.append(("worker_firm_20M", lambda: worker_firm_panel(n_workers=1_000_000, n_firms=100_000,
                                                                 n_periods=20, switch_prob=0.1, n_reg=8,
                                                                 seed=20261204)))
        out.append(("worker_firm_30M_5pct", lambda: worker_firm_panel(n_workers=1_000_000, n_firms=200_000,
                                                                      n_periods=30, switch_prob=0.05, n_reg=8,
                                                                      tenure_sick=True, seed=20261206)))
    return out


def _time_fit(fit, repeats: int) -> float:
    best = math.inf
    for _ in range(repeats):
        t0 = time.perf_counter()
        fit()
        best = min(best, time.perf_counter() - t0)
    return best


def tune(repeats: int = 3, quick: bool = False, log=print) -> dict:
    """Coordinate descent over KNOBS for each shape class; returns the table."""
    import numpy as np

    from .estimator import DeviceBuffer, fe_gpu_estimate_device, fe_runtime_config

    entries = []
    for name, make in _shapes(quick):
        hdr, host = make()
        n, k = host.W.shape
        n_fe = host.fe_ids.shape[0]
        by = DeviceBuffer.from_array(host.y)
        bW = DeviceBuffer.from_array(np.asfortranarray(host.W))
        bf = [DeviceBuffer.from_array(np.ascontiguousarray(host.fe_ids[d])) for d in range(n_fe)]
        cfg = fe_runtime_config(fe_tolerance=1e-8, fe_max_iterations=100000, cluster_fe_dims=[1, 2, 3],
                                precision="mixed", demean_cg=True)

        def fit():
            return fe_gpu_estimate_device(cfg, n, k, 0, by.ptr, bW.ptr, None, [b.ptr for b in bf],
                                          tune=False)

        reset()
        best = {key: get_knob(key) for key in KNOBS}
        ref = fit()  # warm-up, and the reference result of the default knobs
        timings = {}
        for key, cands in KNOBS.items():
            results = {}
            for v in cands:
                for k2, v2 in best.items():
                    set_knob(k2, v2)
                set_knob(key, v)
                r = fit()
                dbeta = float(np.max(np.abs(r.beta - ref.beta) / np.maximum(np.abs(ref.beta), 1e-300)))
                if not r.converged or dbeta > 1e-6:
                    log(f"{name}: {key}={v} rejected (converged {r.converged}, beta rel diff {dbeta:.2e})")
                    continue
                results[v] = _time_fit(fit, repeats)
            timings[key] = {str(v): t for v, t in results.items()}
            if results:
                best[key] = min(results, key=results.get)
            log(f"{name}: {key} -> {best[key]} ({', '.join(f'{v}: {t * 1e3:.2f} ms' for v, t in results.items())})")
        entries.append({"workload": name, "rows": int(n), "columns": int(1 + k),
                        "column_class": column_class(1 + k), "groups": [int(host.fe_ids[d].max()) for d in range(n_fe)],
                        "best": best, "seconds_per_fit": timings})
        for b in [by, bW] + bf:
            b.free()
        reset()
    return {"device": _device_name(), "repeats": repeats, "knobs": KNOBS, "entries": entries,
            "timing": "host wall time of one whole fit (mixed CG, 3-way clusters), best of the repeats"}


def _device_name() -> str:
    try:
        import torch

        return torch.cuda.get_device_name(0)
    except Exception:  # noqa: BLE001 - the name is informational
        return "unknown"


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--out", default=str(TABLE))
    ap.add_argument("--repeats", type=int, default=3)
    ap.add_argument("--quick", action="store_true", help="the small shape classes only")
    args = ap.parse_args(argv)
    N.check(N.lib().fe_gpu_runtime_is_available(), "no CUDA device")
    table = tune(repeats=args.repeats, quick=args.quick)
    Path(args.out).write_text(json.dumps(table, indent=1) + "\n")
    print("wrote", args.out)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
