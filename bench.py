#!/usr/bin/env python3
"""Benchmark of the fixed-effects estimation path on GB300.

One step = one whole fit (FE preparation, within-transform to fe-tol 1e-8,
normal equations, 3-way clustered SEs) of the workload below, with its inputs
already resident in HBM. The default workload is the 150M-row worker-firm
panel (5,000,000 workers x 30 periods, 1,000,000 firms with Pareto(1.5) sizes,
5% mobility per period, tenure + sick + 6 regressors, FEs worker/firm/time,
3-way clustering), fitted in the mixed-precision form; the plain FP64 forms
are timed beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload NAME]

Prints one JSON line (rank 0). Under torchrun each rank fits its own replica
of the panel (weak scaling, no collective on the data path).

The CPU legs (cpu_baseline, and --impl reference) fit a bounded sample of the
workload: the same panel design with the workers and firms divided by the
workload's sample divisor (1/200 of the 150M panel: 25,000 workers x 30
periods over 5,000 firms, 750k rows). The GPU fits the same sample too, so the
line carries a like-for-like rate and the per-coefficient errors of the GPU
fit against the CPU oracle on identical inputs.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

from fe_gpu_gb300 import replicas

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "fit time & demean GB/s (of ~8 TB/s): FP32-mixed+batched vs plain FP64 @ tol 1e-8"
UNIT = "rows/s"

WORKLOADS = {
    "worker_firm_20M": dict(n_workers=1_000_000, n_firms=100_000, n_periods=20, switch_prob=0.1, n_reg=8,
                            seed=20261204, cpu_sample_div=20,
                            desc="1M workers x 20 periods, 100k Pareto(1.5) firms, 10% switching, "
                                 "8 regressors, FEs worker/firm/time, 3-way clustered SEs"),
    "worker_firm_150M": dict(n_workers=5_000_000, n_firms=1_000_000, n_periods=30, switch_prob=0.05, n_reg=8,
                             tenure_sick=True, seed=20261206, cpu_sample_div=200,
                             desc="5M workers x 30 periods, 1M Pareto(1.5) firms, 5% mobility, tenure/sick + 6 "
                                  "regressors, FEs worker/firm/time, 3-way clustered SEs"),
    "worker_firm_2M": dict(n_workers=100_000, n_firms=10_000, n_periods=20, switch_prob=0.1, n_reg=8,
                           seed=20261204, cpu_sample_div=2, desc="small case of the 20M panel for profiling"),
    "worker_firm_5M": dict(n_workers=250_000, n_firms=25_000, n_periods=20, switch_prob=0.1, n_reg=8,
                           seed=20261204, cpu_sample_div=5, desc="quarter-size case of the 20M panel for ncu captures (360 MB of "
                                                "FP64 rows, above L2)"),
    "nls_panel": dict(generator="nls", seed=20261203, cpu_sample_div=1,
                      desc="nlswork-shaped unbalanced panel: 4,700 ids with U{1..15} consecutive years of 15, "
                           "13 Zipf(1.1) occupations, 5 regressors, FEs id/occupation/year, 3-way clustered SEs"),
}


# 2SLS with categorical expansion: the formula is expanded on the device
# (90 regressors, 20 instruments) and fitted with 2-way clustered SEs.
FORMULA_WORKLOADS = {
    "iv_10M": dict(n=10_000_000, g=(500_000, 50_000, 30), seed=20261205,
                   desc="10M rows, FEs 500k/50k/30 uniform; 2SLS: continuous + 4-level categorical (base 2) "
                        "endogenous, continuous + 20-level instrument, i.a&&i.b (20x4), x1&x2, 6 exogenous; "
                        "2-way clustered; formula expanded on the device to 90 regressors and 20 instruments"),
    "iv_1M": dict(n=1_000_000, g=(50_000, 5_000, 30), seed=20261205, desc="small case of iv_10M for profiling"),
}


# Batched specifications: many independent regressions fitted together.
BATCH_WORKLOADS = {
    "batch_512": dict(n_specs=512, total_rows=100e6, seed=20261207,
                      desc="512 independent specifications, rows log-uniform in [5k, 2M] (about 100M in total), "
                           "1-3 FEs with levels ~ rows^0.7, 2-24 regressors, 75% OLS / 25% 2SLS (1-2 endogenous), "
                           "1-3-way clustering; one within-transform per column-count class"),
    "batch_64": dict(n_specs=64, total_rows=4e6, seed=20261207, desc="small case of batch_512 for profiling"),
}


def dist_env():
    return replicas.dist_env()


def make_panel(name, scale=1):
    """The workload's panel; scale > 1 divides the workers and firms of a
    worker-firm panel (the bounded CPU sample). The nls panel is small enough
    to be used whole."""
    from fe_gpu_gb300.synth import nls_panel, worker_firm_panel

    w = dict(WORKLOADS[name])
    w.pop("desc")
    w.pop("cpu_sample_div", None)
    if w.pop("generator", None) == "nls":
        return nls_panel(seed=w["seed"])
    if scale > 1:
        w["n_workers"] = max(1000, w["n_workers"] // scale)
        w["n_firms"] = max(100, w["n_firms"] // scale)
    return worker_firm_panel(**w)


def sample_of(name):
    """(header, host arrays, description) of the bounded CPU sample of a
    workload: the same design with the workers and firms divided by the
    workload's sample divisor; the nls panel whole."""
    w = WORKLOADS[name]
    div = w.get("cpu_sample_div", 1)
    hdr, host = make_panel(name, scale=div)
    if w.get("generator") == "nls" or div == 1:
        what = "the whole panel"
    else:
        what = (f"1/{div} of the panel: {max(1000, w['n_workers'] // div)} workers x {w['n_periods']} periods, "
                f"{max(100, w['n_firms'] // div)} firms, same design and seed")
    return hdr, host, what


def workload_rows(name):
    w = WORKLOADS[name]
    if w.get("generator") == "nls":
        return make_panel(name)[1].y.shape[0]
    return w["n_workers"] * w["n_periods"]


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.idx = device_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.idx)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, power, reasons = [], None, [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
                power.append(float(parts[3]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm), "power_w_max": max(power) if power else None}


def measured_hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            v = json.load(f).get("hbm_gbs")
        if v:
            return float(v), "measured"
    except (OSError, ValueError):
        pass
    return 6800.0, "fallback"


def oracle_fit(host, threads):
    """The oracle (C restatement of the reference CPU estimator) on one panel,
    with the CPU path's conventions; returns (result, seconds)."""
    from oracle import oracle as O

    os.environ["OMP_NUM_THREADS"] = str(threads)
    t0 = time.perf_counter()
    r = O.cpu_estimate(host.y, host.W, host.fe_ids, tol=1e-8, max_iter=100000, cluster_dims=[1, 2, 3])
    return r, time.perf_counter() - t0


def cpu_baseline(name, threads, sample=None):
    """The oracle on the workload's bounded sample (about 10-20 s of CPU work
    on the host's cores). Returns the baseline entry and the oracle result."""
    hdr, host, what = sample if sample is not None else sample_of(name)
    r, dt = oracle_fit(host, threads)
    n = host.y.shape[0]
    entry = {"value": n / dt, "unit": UNIT, "cores": threads, "kind": "port",
             "sample": f"{n} rows ({what}), whole fit with the reference CPU conventions, "
                       f"{r.stats['fe_iterations']} AP iterations, {dt:.2f} s on {threads} host threads",
             "rows": n, "seconds": dt}
    return entry, r


def run_reference(args):
    """The reference's CPU path (the oracle port: the reference itself needs a
    Fortran compiler and LAPACK) on the workload's bounded sample, with all
    host threads. Each step fits the whole sample; ms_per_step is the measured
    time of one such fit, and config.rows the rows it fitted."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    sample = sample_of(args.workload)
    hdr, host, what = sample
    n = host.y.shape[0]
    secs = []
    r = None
    for i in range(args.warmup + args.steps):
        r, dt = oracle_fit(host, threads)
        if i >= args.warmup:
            secs.append(dt)
    step_s = float(np.median(secs)) if secs else float("nan")
    value = n / step_s
    w = WORKLOADS[args.workload]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": f"{args.workload} sample ({what})", "description": w["desc"], "rows": n,
                   "full_workload_rows": workload_rows(args.workload), "fe_tol": 1e-8,
                   "sampled": True, "step_seconds_all": secs},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{n} rows ({what}), whole fit with the reference CPU conventions, "
                                   f"{r.stats['fe_iterations'] if r else 0} AP iterations per fit, "
                                   f"median {step_s:.2f} s per fit on {threads} host threads"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def knob_values():
    """The launch-shape knobs in force (after the autotuner's table or --knob)."""
    from fe_gpu_gb300 import autotune

    return {k: autotune.get_knob(k) for k in list(autotune.KNOBS) + ["batch_estimator"]}


def rel_errors(got, ref):
    got, ref = np.asarray(got, dtype=np.float64), np.asarray(ref, dtype=np.float64)
    return [float(v) for v in np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + sorted(FORMULA_WORKLOADS) + sorted(BATCH_WORKLOADS),
                    default="worker_firm_150M")
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--method", choices=["cg", "ap"], default="cg",
                    help="within-transform of the headline form (the FP64 comparison always uses AP)")
    ap.add_argument("--fp64-steps", type=int, default=1,
                    help="timed steps of each plain FP64 form (AP and CG; no warm-up of their own)")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--file", choices=["auto", "on", "off"], default="auto",
                    help=".bin file leg (write the panel once, load it to the device, fit); auto: panels up to "
                         "50M rows")
    ap.add_argument("--profile-case", action="store_true",
                    help="one fit per (precision, method) and exit (for ncu captures)")
    ap.add_argument("--case", default="all", help="with --profile-case: mixed-cg, fp64-cg, mixed-ap, fp64-ap or all")
    ap.add_argument("--knob", action="append", default=[],
                    help="key=value: set a launch-shape knob (fegb_set_tuning) for every fit of the run; the "
                         "autotuner's table is not applied then")
    args = ap.parse_args()
    if args.knob and args.impl == "ours":
        from fe_gpu_gb300 import autotune

        os.environ["FEGB_TUNING"] = "off"
        autotune.reset()
        for kv in args.knob:
            key, val = kv.split("=", 1)
            autotune.set_knob(key.strip(), int(val))
    if args.impl == "reference":
        return run_reference(args)
    if args.workload in FORMULA_WORKLOADS:
        return run_formula(args)
    if args.workload in BATCH_WORKLOADS:
        return run_batch(args)

    import torch

    from fe_gpu_gb300 import _native
    from fe_gpu_gb300.estimator import fe_gpu_estimate, fe_gpu_estimate_device, fe_runtime_config

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    replicas.init(world)
    _native.check(_native.lib().fe_gpu_runtime_is_available(), "no CUDA device")
    stream = torch.cuda.Stream()

    hdr, host = make_panel(args.workload)
    n, k = host.W.shape
    n_fe = host.fe_ids.shape[0]
    dev = torch.device("cuda", local)
    d_y = torch.from_numpy(host.y).to(dev)
    d_W = torch.from_numpy(np.ascontiguousarray(host.W.T)).to(dev)  # column-major n x k
    d_ids = [torch.from_numpy(np.ascontiguousarray(host.fe_ids[d])).to(dev) for d in range(n_fe)]
    torch.cuda.synchronize()

    def cfg_for(precision, method=None):
        method = args.method if method is None else method
        return fe_runtime_config(fe_tolerance=1e-8, fe_max_iterations=100000, cluster_fe_dims=[1, 2, 3],
                                 precision=precision, demean_cg=(method == "cg"))

    def fit(precision, profile=False, method=None):
        return fe_gpu_estimate_device(cfg_for(precision, method), n, k, 0, d_y.data_ptr(), d_W.data_ptr(), None,
                                      [t.data_ptr() for t in d_ids], stream=stream.cuda_stream, profile=profile)

    if args.profile_case:
        for p, m in (("mixed", "cg"), ("fp64", "cg"), ("mixed", "ap"), ("fp64", "ap")):
            if args.case != "all" and args.case != f"{p}-{m}":
                continue
            # per-launch events (host-driven loop), so every kernel launch is visible to a profiler
            r = fit(p, profile=True, method=m)
            print(p, m, r.fe_iterations, r.stats["outer_iterations"], r.stats["time_total"], flush=True)
        return 0

    def barrier():
        replicas.barrier(world)

    def timed(precision, steps, profile, method=None):
        res = None
        barrier()
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        launches0 = _native.lib().fegb_kernel_launches()
        ev0.record(stream)
        results = []
        for _ in range(steps):
            res = fit(precision, profile, method)
            results.append(res)
        ev1.record(stream)
        torch.cuda.synchronize()
        barrier()
        launches = _native.lib().fegb_kernel_launches() - launches0
        ms = ev0.elapsed_time(ev1) / steps
        ms = replicas.max_over_ranks(ms, world, dev)
        return ms, results, launches

    for _ in range(args.warmup):
        fit(args.precision)
    sampler = ClockSampler(local)
    sampler.start()
    ms, results, launches = timed(args.precision, args.steps, True)
    clocks = sampler.stop()
    last = results[-1]

    # plain FP64 forms beside it (the reference's AP scheme, and CG), timed
    # without warm-up fits of their own: one FP64 AP fit of the 150M panel
    # takes about a minute
    fp64_ms = fp64cg_ms = None
    fp64_res = fp64cg_res = None
    if args.fp64_steps > 0:
        fp64cg_ms, fr, _ = timed("fp64", args.fp64_steps, False, method="cg")
        fp64cg_res = fr[-1]
        fp64_ms, fr, _ = timed("fp64", args.fp64_steps, False, method="ap")
        fp64_res = fr[-1]

    # end to end through the host-buffer C ABI, inputs in pinned host memory
    pin_y = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
    pin_y[:] = host.y
    pin_W = torch.empty(n * k, dtype=torch.float64, pin_memory=True).numpy().reshape(k, n).T
    pin_W[:] = host.W
    pin_ids = torch.empty(n * n_fe, dtype=torch.int32, pin_memory=True).numpy().reshape(n, n_fe).T
    pin_ids[:] = host.fe_ids
    from fe_gpu_gb300.bin_io import fe_host_arrays

    hp = fe_host_arrays(y=pin_y, W=pin_W, Z=np.zeros((n, 0), order="F"), fe_ids=pin_ids)
    fe_gpu_estimate(cfg_for(args.precision), hdr, hp, stream=stream.cuda_stream)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_each = []
    for _ in range(args.e2e_steps):
        t1 = time.perf_counter()
        er = fe_gpu_estimate(cfg_for(args.precision), hdr, hp, stream=stream.cuda_stream)
        e2e_each.append(time.perf_counter() - t1)
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / args.e2e_steps
    e2e_s = replicas.max_over_ranks(e2e_s, world, dev)
    h2d = pin_y.nbytes + n * k * 8 + n * n_fe * 4
    d2h = 2 * k * 8

    # .bin file leg: the panel written once in the fe_gpu format, then loaded
    # straight to the device (fegb_load_bin) and fitted from there
    file_leg = None
    file_on = args.file == "on" or (args.file == "auto" and n <= 50_000_000)
    if file_on and rank == 0:
        import tempfile

        from fe_gpu_gb300.bin_io import DeviceDataset, write_dataset

        with tempfile.TemporaryDirectory(dir=os.environ.get("TMPDIR")) as td:
            path = os.path.join(td, "panel.bin")
            write_dataset(path, host.y, host.W, host.fe_ids, metadata=dict(
                y="y", x=[f"x{j + 1}" for j in range(k)], fe=["worker", "firm", "time"]))
            size = os.path.getsize(path)
            DeviceDataset(path).close()  # first touch (page cache)
            t0 = time.perf_counter()
            ds = DeviceDataset(path)
            load_s = time.perf_counter() - t0
            t1 = time.perf_counter()
            fr = fe_gpu_estimate_device(cfg_for(args.precision), ds.n, ds.k, 0, ds.y, ds.W, None, ds.fe_ids,
                                        stream=stream.cuda_stream)
            torch.cuda.synchronize()
            fit_s = time.perf_counter() - t1
            ds.close()
            file_leg = {"file_bytes": size, "load_s": load_s, "load_gbs": size / load_s / 1e9,
                        "fit_after_load_s": fit_s, "rows_per_s_from_file": n / (load_s + fit_s),
                        "beta_equal_to_resident_fit": bool(np.array_equal(fr.beta, last.beta))}

    # roofline of the dominant sweep-kernel family, timed live in the timed steps
    roofline = roofline_of(results, args.workload, elements_per_sweep=n * (1 + k))
    demean_gbs = last.stats["demean_bytes"] / last.stats["time_demean"] / 1e9 if last.stats["time_demean"] else None

    value = world * n / (ms / 1e3)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32-sweeps+f64" if args.precision == "mixed" else "f64", "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "description": WORKLOADS[args.workload]["desc"], "rows": n,
                   "columns": 1 + k, "fe_tol": 1e-8, "precision": args.precision, "within_transform": args.method,
                   "l2": "inputs larger than L2 (%.2f GB of FP64 data per fit)" % (n * (1 + k) * 8 / 1e9),
                   "parallelism": f"replicas x{world}", "knobs": knob_values()},
        "fit_time_s": ms / 1e3,
        "fit_breakdown_s": {key: last.stats[key] for key in ("time_prep", "time_demean", "time_regression",
                                                              "time_se")},
        "fe_iterations": last.fe_iterations, "outer_iterations": last.stats["outer_iterations"],
        "projections": last.stats["projections"],
        "demean_gbs_algorithmic": demean_gbs,
        "rows_x_cols_demeaned_per_s": (last.stats["projections"] * n * (1 + k) / last.stats["time_demean"]
                                       if last.stats["time_demean"] else None),
        "fp64_ap_fit_time_s": fp64_ms / 1e3 if fp64_ms else None,
        "fp64_fe_iterations": fp64_res.fe_iterations if fp64_res else None,
        "speedup_vs_plain_fp64_ap": (fp64_ms / ms) if fp64_ms else None,
        "fp64_cg_fit_time_s": fp64cg_ms / 1e3 if fp64cg_ms else None,
        "fp64_cg_fe_iterations": fp64cg_res.fe_iterations if fp64cg_res else None,
        "speedup_vs_plain_fp64_cg": (fp64cg_ms / ms) if fp64cg_ms else None,
        "fp64_timed_steps": args.fp64_steps,
        "beta_max_rel_diff_mixed_vs_fp64": (max(rel_errors(last.beta, fp64_res.beta)) if fp64_res else None),
        "se_max_rel_diff_mixed_vs_fp64": (max(rel_errors(last.se, fp64_res.se)) if fp64_res else None),
        "coefficients_vs_fp64_ap": ({"names": last.coef_names, "beta": [float(b) for b in last.beta],
                                     "se": [float(v) for v in last.se],
                                     "beta_rel_err": rel_errors(last.beta, fp64_res.beta),
                                     "se_rel_err": rel_errors(last.se, fp64_res.se)} if fp64_res else None),
        "e2e": {"value": world * n / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "seconds_per_step": e2e_s, "seconds_each": e2e_each,
                "last_breakdown_s": {key: er.stats[key] for key in ("time_h2d", "time_prep", "time_demean",
                                                                     "time_regression", "time_se", "time_total")}},
        "gpu_launches": int(launches / args.steps) * args.steps,
        "bin_file": file_leg,
        "roofline": roofline,
        "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu_baseline:
        # the CPU oracle and the GPU on the same bounded sample: a like-for-like
        # rate, and the GPU fit's per-coefficient errors against the oracle
        # (CPU conventions on both sides)
        sample = sample_of(args.workload)
        entry, oref = cpu_baseline(args.workload, os.cpu_count() or 1, sample)
        line["cpu_baseline"] = {k2: v for k2, v in entry.items() if k2 not in ("seconds", "rows")}
        line["parity_vs_oracle"] = parity_on_sample(sample, oref, entry, stream)
    if rank == 0:
        print(json.dumps(line), flush=True)
    replicas.finish(world)
    return 0


def parity_on_sample(sample, oref, cpu_entry, stream):
    """Fits the CPU baseline's sample on the GPU (headline mixed CG form and
    plain FP64 AP, CPU SE conventions, from pinned-free host arrays through
    fegb_estimate_host) and compares every coefficient and SE with the
    oracle's, and the integer outputs exactly."""
    import torch

    from fe_gpu_gb300.estimator import fe_gpu_estimate, fe_runtime_config

    hdr, host, what = sample
    n = host.y.shape[0]
    out = {"sample": what, "rows": n, "tolerance": {"beta_rel": 1e-6, "se_rel": 1e-5},
           "oracle": "C restatement of the reference CPU estimator (fe_pipeline.f90:71-513)",
           "oracle_fe_iterations": oref.stats["fe_iterations"]}
    for label, precision, cg in (("mixed_cg", "mixed", True), ("fp64_ap", "fp64", False)):
        cfg = fe_runtime_config(fe_tolerance=1e-8, fe_max_iterations=100000, cluster_fe_dims=[1, 2, 3],
                                precision=precision, demean_cg=cg, se_convention="cpu")
        fe_gpu_estimate(cfg, hdr, host, stream=stream.cuda_stream)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fe_gpu_estimate(cfg, hdr, host, stream=stream.cuda_stream)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        be = rel_errors(r.beta, oref.beta)
        sv = rel_errors(r.se, oref.se)
        out[label] = {"beta_rel_err": be, "se_rel_err": sv, "max_beta_rel": max(be), "max_se_rel": max(sv),
                      "dof_resid_equal": int(r.dof_resid) == int(oref.stats["dof_resid"]),
                      "converged": bool(r.converged), "fe_iterations": r.fe_iterations,
                      "fit_s_host_arrays": dt, "rows_per_s_host_arrays": n / dt,
                      "vs_cpu_baseline_same_sample": (n / dt) / cpu_entry["value"]}
    out["pass"] = all(out[lb]["max_beta_rel"] < 1e-6 and out[lb]["max_se_rel"] < 1e-5 and out[lb]["dof_resid_equal"]
                      for lb in ("mixed_cg", "fp64_ap"))
    return out


FAMILIES = ["segment sweep fp64", "segment sweep fp32", "small-G sweep fp64", "small-G sweep fp32",
            "CG operator segment sweep fp64", "CG operator segment sweep fp32",
            "CG operator dense small-G products fp64", "CG operator dense small-G products fp32"]
ALG_BYTES = {
    "segment": ("N (4 + C s) per read-only sweep (one id and one row read per position; the FP64 mean passes "
                "of the mixed form are read-only), N C s more when the rows are written back, 4 N for the "
                "traversal permutation of a gathered sweep"),
    "cg": "N (4 (1 + S) + S C s): destination and S swept source ids, S gathered FE-table rows",
    "dense": "G_e (4 G_s + C s) per product: count-matrix rows and FE-table rows read once",
}


# Nominal dense FP64 rate of the part (1.25 TFLOP/s, an FMA counted as two):
# an FP64 addition takes one FMA issue slot, so 625 G additions/s.
FP64_ADDS_PEAK_NOMINAL = 625.0


def roofline_of(results, workload, elements_per_sweep=None):
    """Roofline entry of the dominant sweep family. For the FP64 sweep families
    (one FP64 addition per element) elements_per_sweep = N x C also gives the
    FP64-pipe rate, the bound that sits below HBM for them on this part."""
    secs = [sum(r.stats["prof_seconds"][i] for r in results) for i in range(8)]
    nlaunch = [sum(r.stats["prof_launches"][i] for r in results) for i in range(8)]
    nbytes = [sum(r.stats["prof_bytes"][i] for r in results) for i in range(8)]
    top = int(np.argmax(secs))
    peak, peak_kind = measured_hbm_peak()
    achieved = nbytes[top] / secs[top] / 1e9 if secs[top] > 0 else 0.0
    traffic = TRAFFIC_PER_LAUNCH.get((workload, FAMILIES[top]))
    fp64 = None
    if elements_per_sweep and top in (0, 2) and secs[top] > 0:
        gadds = elements_per_sweep * nlaunch[top] / secs[top] / 1e9
        fp64 = {"adds_per_launch": elements_per_sweep, "achieved_gadds_per_s": gadds,
                "peak_gadds_per_s_nominal": FP64_ADDS_PEAK_NOMINAL, "frac": gadds / FP64_ADDS_PEAK_NOMINAL}
    return {"bound": "hbm", "kernel": FAMILIES[top], "achieved": achieved, "peak": peak, "peak_source": peak_kind,
            "fp64_pipe": fp64,
            "unit": "GB/s", "frac": achieved / peak if peak else None, "traffic": traffic,
            # the captured DRAM bytes per launch over this run's average launch time
            "traffic_gbs": (traffic / (secs[top] / max(1, nlaunch[top])) / 1e9) if traffic and secs[top] else None,
            "traffic_frac": (traffic / (secs[top] / max(1, nlaunch[top])) / 1e9 / peak)
                            if traffic and secs[top] and peak else None,
            "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum per launch, " +
                               TRAFFIC_SOURCE[(workload, FAMILIES[top])]) if traffic is not None else None,
            "alg_bytes_definition": ALG_BYTES["segment" if top < 4 else ("cg" if top < 6 else "dense")],
            "launches": nlaunch[top], "avg_launch_ms": secs[top] / max(1, nlaunch[top]) * 1e3,
            "alg_bytes_per_launch": nbytes[top] / max(1, nlaunch[top]),
            "all_families": {FAMILIES[i]: {"launches": nlaunch[i], "seconds": secs[i],
                                           "gbs": (nbytes[i] / secs[i] / 1e9) if secs[i] else None}
                             for i in range(8) if nlaunch[i]}}


def run_formula(args):
    """Formula workloads: each step expands the formula on the device from the
    resident raw columns and fits it (the plain FP64 AP form beside it); e2e
    runs the whole formula fit from pinned host arrays."""
    import torch

    from fe_gpu_gb300 import _native
    from fe_gpu_gb300.estimator import fe_runtime_config
    from fe_gpu_gb300.formula import RawDevice, expand_formula, fe_gpu_estimate_formula, fit_formula
    from fe_gpu_gb300.synth import iv_formula_panel

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    replicas.init(world)
    w = FORMULA_WORKLOADS[args.workload]
    hdr, host, formula = iv_formula_panel(n=w["n"], g=w["g"], seed=w["seed"])
    n = host.y.shape[0]
    stream = torch.cuda.Stream()
    raw = RawDevice(hdr, host)

    def cfg_for(precision, method):
        return fe_runtime_config(fe_tolerance=1e-8, fe_max_iterations=100000, precision=precision,
                                 demean_cg=(method == "cg"))

    def step(precision, method, profile=False):
        ff, cfg2 = expand_formula(formula, raw, cfg_for(precision, method), stream.cuda_stream)
        res = fit_formula(ff, cfg2, hdr, stream.cuda_stream, profile)
        ff.buffers["W"].free()
        if ff.plan.instruments is not None:
            ff.buffers["Z"].free()
        return res

    def barrier():
        replicas.barrier(world)

    def timed(precision, method, steps, profile):
        barrier()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = _native.lib().fegb_kernel_launches()
        ev0.record(stream)
        results = [step(precision, method, profile) for _ in range(steps)]
        ev1.record(stream)
        torch.cuda.synchronize()
        barrier()
        ms = ev0.elapsed_time(ev1) / steps
        ms = replicas.max_over_ranks(ms, world, torch.device("cuda", local))
        return ms, results, _native.lib().fegb_kernel_launches() - l0

    if args.profile_case:
        for p, m in (("mixed", "cg"), ("fp64", "cg"), ("mixed", "ap"), ("fp64", "ap")):
            if args.case != "all" and args.case != f"{p}-{m}":
                continue
            r = step(p, m)
            print(p, m, r.fe_iterations, r.stats["outer_iterations"], r.stats["time_total"], flush=True)
        return 0

    for _ in range(args.warmup):
        step(args.precision, args.method)
    sampler = ClockSampler(local)
    sampler.start()
    ms, results, launches = timed(args.precision, args.method, args.steps, True)
    clocks = sampler.stop()
    last = results[-1]
    fp64_ms, fp64_res = None, None
    if args.fp64_steps > 0:
        step("fp64", "ap")
        fp64_ms, fr, _ = timed("fp64", "ap", args.fp64_steps, False)
        fp64_res = fr[-1]

    # end to end from pinned host arrays through the formula front end
    def pinned(a, dtype):
        t = torch.empty(a.size, dtype=dtype, pin_memory=True).numpy()
        return t

    from fe_gpu_gb300.bin_io import fe_host_arrays

    py = pinned(host.y, torch.float64)
    py[:] = host.y
    pW = pinned(host.W, torch.float64).reshape(host.W.shape[1], n).T
    pW[:] = host.W
    pZ = pinned(host.Z, torch.float64).reshape(host.Z.shape[1], n).T
    pZ[:] = host.Z
    pf = pinned(host.fe_ids, torch.int32).reshape(n, host.fe_ids.shape[0]).T
    pf[:] = host.fe_ids
    hp = fe_host_arrays(y=py, W=pW, Z=pZ, fe_ids=pf)
    fe_gpu_estimate_formula(formula, hdr, hp, cfg_for(args.precision, args.method), stream.cuda_stream)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        er = fe_gpu_estimate_formula(formula, hdr, hp, cfg_for(args.precision, args.method), stream.cuda_stream)
    torch.cuda.synchronize()
    e2e_s = replicas.max_over_ranks((time.perf_counter() - t0) / args.e2e_steps, world, torch.device("cuda", local))
    k = len(last.beta)
    line = {
        "metric": METRIC, "value": world * n / (ms / 1e3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32-sweeps+f64" if args.precision == "mixed" else "f64", "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "description": w["desc"], "rows": n, "formula": formula,
                   "regressors": k, "instruments": last.formula.l, "columns": 1 + k + last.formula.l,
                   "fe_tol": 1e-8, "precision": args.precision, "within_transform": args.method,
                   "l2": "inputs larger than L2", "parallelism": f"replicas x{world}"},
        "fit_time_s": ms / 1e3,
        "fit_breakdown_s": {key: last.stats[key] for key in ("time_prep", "time_demean", "time_regression",
                                                              "time_se")},
        "fe_iterations": last.fe_iterations, "outer_iterations": last.stats["outer_iterations"],
        "is_iv": last.is_iv, "n_instruments": last.n_instruments,
        "fp64_ap_fit_time_s": fp64_ms / 1e3 if fp64_ms else None,
        "speedup_vs_plain_fp64_ap": (fp64_ms / ms) if fp64_ms else None,
        "beta_max_rel_diff_mixed_vs_fp64": (float(np.max(np.abs(last.beta - fp64_res.beta) /
                                                         np.abs(fp64_res.beta))) if fp64_res else None),
        "se_max_rel_diff_mixed_vs_fp64": (float(np.max(np.abs(last.se - fp64_res.se) / np.abs(fp64_res.se)))
                                          if fp64_res else None),
        "e2e": {"value": world * n / e2e_s, "unit": UNIT, "h2d_bytes_per_step": raw.h2d_bytes,
                "d2h_bytes_per_step": 2 * k * 8, "seconds_per_step": e2e_s},
        "gpu_launches": int(launches / args.steps) * args.steps,
        "roofline": roofline_of(results, args.workload),
        "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = formula_cpu_baseline(os.cpu_count() or 1)
    if rank == 0:
        print(json.dumps(line), flush=True)
    replicas.finish(world)
    return 0


def run_batch(args):
    """Batched specifications: one step fits every specification with
    fegb_estimate_batch (inputs resident in HBM); beside it the same
    specifications as sequential plain FP64 fits; e2e adds the host-to-device
    copies of every specification from pinned memory."""
    import torch

    from fe_gpu_gb300 import _native
    from fe_gpu_gb300.estimator import (DeviceBuffer, fe_batch_spec, fe_gpu_estimate_batch, fe_gpu_estimate_device,
                                        fe_runtime_config)
    from fe_gpu_gb300.synth import batch_specs

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    replicas.init(world)
    w = BATCH_WORKLOADS[args.workload]
    specs = batch_specs(n_specs=w["n_specs"], total_rows=w["total_rows"], seed=w["seed"])
    stream = torch.cuda.Stream()
    rows = sum(h.y.shape[0] for h, _ in specs)

    def upload():
        bufs, out = [], []
        for host, extra in specs:
            by = DeviceBuffer.from_array(host.y)
            bW = DeviceBuffer.from_array(np.asfortranarray(host.W))
            bZ = DeviceBuffer.from_array(np.asfortranarray(host.Z)) if host.Z.shape[1] else None
            bf = [DeviceBuffer.from_array(np.ascontiguousarray(host.fe_ids[d])) for d in range(host.fe_ids.shape[0])]
            bufs.append((by, bW, bZ, bf))
            out.append(fe_batch_spec(n=host.y.shape[0], k=host.W.shape[1], l=host.Z.shape[1], d_y=by.ptr,
                                     d_W=bW.ptr, d_Z=bZ.ptr if bZ else None, d_fe_ids=[b.ptr for b in bf],
                                     cluster_fe_dims=extra["cluster_fe_dims"], iv_regressors=extra["iv_regressors"]))
        return bufs, out

    bufs, dspecs = upload()
    h2d = sum(h.y.nbytes + h.W.nbytes + h.Z.nbytes + h.fe_ids.nbytes for h, _ in specs)
    cfg = fe_runtime_config(fe_tolerance=1e-8, fe_max_iterations=100000, precision=args.precision,
                            demean_cg=(args.method == "cg"))

    def barrier():
        replicas.barrier(world)

    def timed(fn, steps):
        barrier()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = _native.lib().fegb_kernel_launches()
        ev0.record(stream)
        out = [fn() for _ in range(steps)]
        ev1.record(stream)
        torch.cuda.synchronize()
        barrier()
        ms = ev0.elapsed_time(ev1) / steps
        ms = replicas.max_over_ranks(ms, world, torch.device("cuda", local))
        return ms, out, _native.lib().fegb_kernel_launches() - l0

    def batch_fit(profile=False):
        return fe_gpu_estimate_batch(cfg, dspecs, stream=stream.cuda_stream, profile=profile)

    def sequential_fp64():
        out = []
        for (host, extra), sp in zip(specs, dspecs):
            c1 = fe_runtime_config(fe_tolerance=1e-8, fe_max_iterations=100000, precision="fp64", demean_cg=False,
                                   cluster_fe_dims=extra["cluster_fe_dims"], iv_regressors=extra["iv_regressors"])
            out.append(fe_gpu_estimate_device(c1, sp.n, sp.k, sp.l, sp.d_y, sp.d_W, sp.d_Z, sp.d_fe_ids,
                                              stream=stream.cuda_stream))
        return out

    if args.profile_case:
        r = batch_fit()
        print("batch", len(r), r[0].fe_iterations, flush=True)
        return 0

    for _ in range(args.warmup):
        batch_fit()
    sampler = ClockSampler(local)
    sampler.start()
    ms, outs, launches = timed(lambda: batch_fit(True), args.steps)
    clocks = sampler.stop()
    last = outs[-1]
    seq_ms, seq = None, None
    if args.fp64_steps > 0:
        seq_ms, so, _ = timed(sequential_fp64, 1)
        seq = so[-1]
    # e2e: every step copies each specification's inputs from pinned host
    # memory into device buffers (allocated once, as a serving process keeps
    # them) with asynchronous copies on the fit's stream, then runs the batched
    # fit, whose results come back to the host
    pinned, dev = [], []
    for host, _ in specs:
        hs, ds = [], []
        arrays = [(host.y, torch.float64), (np.asfortranarray(host.W).reshape(-1, order="F"), torch.float64),
                  (np.asfortranarray(host.Z).reshape(-1, order="F"), torch.float64)]
        arrays += [(np.ascontiguousarray(host.fe_ids[d]), torch.int32) for d in range(host.fe_ids.shape[0])]
        for a, dt in arrays:
            t = torch.empty(max(1, a.size), dtype=dt, pin_memory=True)
            t[:a.size] = torch.from_numpy(np.ascontiguousarray(a).reshape(-1))
            hs.append(t)
            ds.append(torch.empty(max(1, a.size), dtype=dt, device=torch.device("cuda", local)))
        pinned.append(hs)
        dev.append(ds)
    e2e_specs = []
    for (host, extra), ds in zip(specs, dev):
        n, k, l, nfe = host.y.shape[0], host.W.shape[1], host.Z.shape[1], host.fe_ids.shape[0]
        e2e_specs.append(fe_batch_spec(n=n, k=k, l=l, d_y=ds[0].data_ptr(), d_W=ds[1].data_ptr(),
                                       d_Z=ds[2].data_ptr() if l else None,
                                       d_fe_ids=[ds[3 + d].data_ptr() for d in range(nfe)],
                                       cluster_fe_dims=extra["cluster_fe_dims"],
                                       iv_regressors=extra["iv_regressors"]))

    def e2e_step():
        with torch.cuda.stream(stream):
            for hs, ds in zip(pinned, dev):
                for h, d in zip(hs, ds):
                    d.copy_(h, non_blocking=True)
        return fe_gpu_estimate_batch(cfg, e2e_specs, stream=stream.cuda_stream)

    e2e_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = replicas.max_over_ranks((time.perf_counter() - t0) / args.e2e_steps, world, torch.device("cuda", local))
    ktot = sum(h.W.shape[1] for h, _ in specs)
    diffs_b = [float(np.max(np.abs(a.beta - b.beta) / np.maximum(np.abs(b.beta), 1e-300))) for a, b in zip(last, seq)] \
        if seq else []
    diffs_s = [float(np.max(np.abs(a.se - b.se) / np.maximum(np.abs(b.se), 1e-300))) for a, b in zip(last, seq)] \
        if seq else []
    line = {
        "metric": METRIC, "value": world * rows / (ms / 1e3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32-sweeps+f64" if args.precision == "mixed" else "f64", "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "description": w["desc"], "specs": len(specs), "rows": rows,
                   "fe_tol": 1e-8, "precision": args.precision, "within_transform": args.method,
                   "l2": "inputs larger than L2", "parallelism": f"replicas x{world}", "knobs": knob_values()},
        "fit_time_s": ms / 1e3,
        "specs_per_s": len(specs) / (ms / 1e3),
        "iv_specs": sum(1 for r in last if r.is_iv),
        "fe_iterations_max": max(r.fe_iterations for r in last),
        "sequential_fp64_time_s": seq_ms / 1e3 if seq_ms else None,
        "speedup_vs_sequential_fp64": (seq_ms / ms) if seq_ms else None,
        "beta_max_rel_diff_vs_sequential_fp64": max(diffs_b) if diffs_b else None,
        "se_max_rel_diff_vs_sequential_fp64": max(diffs_s) if diffs_s else None,
        "e2e": {"value": world * rows / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": 2 * ktot * 8, "seconds_per_step": e2e_s},
        "gpu_launches": int(launches / args.steps) * args.steps,
        "roofline": roofline_of([r for step_results in outs for r in step_results], args.workload),
        "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    replicas.finish(world)
    return 0


def formula_cpu_baseline(threads):
    """The oracle's GPU-convention estimator (2SLS; the reference CPU path has
    no 2SLS) on a bounded sample: the same design at 500k rows, expanded with
    the oracle's numpy restatement."""
    from fe_gpu_gb300.formula import parse_formula_string, plan_design
    from fe_gpu_gb300.synth import iv_formula_panel
    from oracle import design_ref as D
    from oracle import oracle as O

    hdr, host, formula = iv_formula_panel(n=500_000, g=(25_000, 2_500, 30), seed=20261205)
    spec = parse_formula_string(formula)
    src = {("W", j): host.W[:, j] for j in range(host.W.shape[1])}
    src.update({("Z", j): host.Z[:, j] for j in range(host.Z.shape[1])})
    os.environ["OMP_NUM_THREADS"] = str(threads)
    t0 = time.perf_counter()
    plan = plan_design(spec, hdr.regressor_names, hdr.instrument_names, lambda m, c: D.collect_levels(src[(m, c)]))
    W = D.expand(src, [c.factors for c in plan.regressors])
    Z = D.expand(src, [c.factors for c in plan.instruments])
    r = O.gpu_estimate(host.y, W, host.fe_ids, Z=Z, tol=1e-8, max_iter=100000, cluster_dims=[1, 2],
                       iv_regressors=plan.iv_regressors, iv_instruments=plan.iv_instrument_cols)
    dt = time.perf_counter() - t0
    n = host.y.shape[0]
    return {"value": n / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n} rows (FEs 25k/2.5k/30), same formula: numpy expansion + oracle 2SLS fit with the "
                      f"reference GPU conventions, {r.stats['fe_iterations']} AP iterations, {dt:.2f} s"}


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the
# dominant kernel family, from the ncu captures summarised in profiles/:
# - CG operator sweep: cg_rows_worker_firm_20M.md (mean of the worker and firm
#   operator sweeps of one fit);
# - FP64 segment sweep: fp64_sweeps_worker_firm_5M.md (the tuple row sweep at
#   5M rows, times 4: the traffic is row data).
# Other workloads were not captured.
TRAFFIC_PER_LAUNCH: dict = {
    ("worker_firm_20M", "CG operator segment sweep fp32"): 7.65e+07,
    ("worker_firm_20M", "segment sweep fp64"): 2.027e+09,
    ("worker_firm_150M", "CG operator segment sweep fp32"): 1.0725e+09,
}
TRAFFIC_SOURCE = {
    ("worker_firm_20M", "CG operator segment sweep fp32"):
        "profiles/dram_cg_operator_worker_firm_20M.md (full-size one-pass capture, two iterations)",
    ("worker_firm_20M", "segment sweep fp64"): "profiles/fp64_sweeps_worker_firm_5M.md (5M-row capture scaled by rows)",
    ("worker_firm_150M", "CG operator segment sweep fp32"):
        "profiles/dram_cg_operator_worker_firm_150M.md (full-size one-pass capture, two iterations)",
}


if __name__ == "__main__":
    sys.exit(main())
