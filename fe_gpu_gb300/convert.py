"""Tabular data -> fe_gpu binary dataset (tools/dataframe_to_fe_binary.py).

    python -m fe_gpu_gb300.convert INPUT --output OUT.bin --y Y --x X1,X2 --fe A,B,C
        [--iv Z1,Z2] [--cluster CL] [--weights W] [--precision float64|float32]
        [--drop-missing] [--summary] [--verbose] [--input-format auto|csv|parquet|pickle]

does what the reference's converter does (tools/dataframe_to_fe_binary.py:186-277):
load the named columns, drop rows with a missing value in any of them when
asked (else refuse missing values), relabel every FE column and the cluster
column to 1-based dense ids in the order of their sorted distinct values
(pandas.factorize(sort=True) + 1, :87-94), and write the header, the columns,
the ids and the META block of names (:123-176) with bin_io.write_dataset.

The relabelling of integer codes runs on the GPU (fegb_compact_ids: a radix
sort, a flag pass and a scan per column); codes that are not integers (text
labels, fractional floats) or that fall outside the int32 range are ranked on
the host first, which is already their dense 1-based id. pandas is optional:
a table is anything whose columns can be read by name (a dict of arrays, a
numpy structured array, a pandas or pyarrow table); CSV files are parsed with
the csv module, parquet needs pyarrow, pickle files hold such a table.
"""
from __future__ import annotations

import argparse
import csv
import ctypes as C
import json
import pathlib
import pickle
import sys
import time
from typing import Callable, Optional, Sequence

import numpy as np

from .bin_io import write_dataset

PRECISION_FLAGS = {"float64": 0, "float32": 1}  # tools/dataframe_to_fe_binary.py:19-22


def device_compact(raw: np.ndarray) -> np.ndarray:
    """1-based rank of each int32 code among the sorted distinct codes, on the
    GPU (fegb_compact_ids)."""
    from . import _native as N
    from .estimator import DeviceBuffer

    raw = np.ascontiguousarray(raw, dtype=np.int32)
    n = raw.shape[0]
    if n == 0:
        return np.zeros(0, np.int32)
    d_raw = DeviceBuffer.from_array(raw)
    d_out = DeviceBuffer(4 * n)
    try:
        levels = C.c_int(0)
        N.check(N.lib().fegb_compact_ids(C.c_void_p(d_raw.ptr), n, C.c_void_p(d_out.ptr), C.byref(levels)),
                "fegb_compact_ids")
        return d_out.to_array(np.int32, (n,))
    finally:
        d_raw.free()
        d_out.free()


def _int32_codes(a: np.ndarray) -> Optional[np.ndarray]:
    """The column as int32 codes when every value is an integer in the int32
    range (integer dtypes, booleans, integral floats), else None."""
    if a.dtype.kind == "b":
        return a.astype(np.int32)
    if a.dtype.kind in "iu":
        if a.size and (a.min() < np.iinfo(np.int32).min or a.max() > np.iinfo(np.int32).max):
            return None
        return a.astype(np.int32)
    if a.dtype.kind == "f":
        if not np.all(np.isfinite(a)) or not np.all(a == np.floor(a)):
            return None
        if a.size and (a.min() < np.iinfo(np.int32).min or a.max() > np.iinfo(np.int32).max):
            return None
        return a.astype(np.int32)
    return None


def relabel_ids(values, compact: Callable[[np.ndarray], np.ndarray] = device_compact) -> np.ndarray:
    """Dense 1-based ids in the order of the sorted distinct values
    (tools/dataframe_to_fe_binary.py:87-94). Integer codes go to `compact`
    (the GPU); other values are ranked on the host."""
    a = np.asarray(values)
    codes = _int32_codes(a)
    if codes is not None:
        return np.asarray(compact(codes), dtype=np.int32)
    if a.dtype.kind == "O":
        if any(v is None or (isinstance(v, float) and np.isnan(v)) for v in a):
            raise ValueError("FE or cluster column contains missing values after cleaning")
        a = a.astype(str) if all(isinstance(v, str) for v in a) else a
    _, inv = np.unique(a, return_inverse=True)
    return (inv.reshape(-1) + 1).astype(np.int32)


# ------------------------------------------------------------------ tables

def column(table, name: str) -> np.ndarray:
    """One named column of a table as a 1-D numpy array."""
    if isinstance(table, dict):
        if name not in table:
            raise KeyError(f"column {name!r} not found")
        return np.asarray(table[name])
    if isinstance(table, np.ndarray) and table.dtype.names:
        return np.asarray(table[name])
    if hasattr(table, "column") and hasattr(table, "num_rows"):  # pyarrow.Table
        return table.column(name).to_numpy()
    col = table[name]  # pandas.DataFrame and alike
    return col.to_numpy() if hasattr(col, "to_numpy") else np.asarray(col)


def _parse_text_column(cells: list) -> np.ndarray:
    """A CSV column: integers when every cell is an integer, numbers (empty
    or NA cells: NaN) when every non-empty cell parses as one, else text
    (empty cells: None)."""
    vals = np.empty(len(cells), dtype=np.float64)
    for i, c in enumerate(cells):
        c = c.strip()
        if c == "" or c.lower() in ("na", "nan"):
            vals[i] = np.nan
            continue
        try:
            vals[i] = float(c)
        except ValueError:
            return np.array([c.strip() or None for c in cells], dtype=object)
    if vals.size and not np.isnan(vals).any() and np.all(vals == np.floor(vals)) and np.all(np.abs(vals) < 2**53):
        return vals.astype(np.int64)
    return vals


def read_csv(path: pathlib.Path, columns: Sequence[str]) -> dict:
    with open(path, newline="") as f:
        rd = csv.reader(f)
        header = next(rd)
        idx = {}
        for name in columns:
            if name not in header:
                raise KeyError(f"column {name!r} not found in {path}")
            idx[name] = header.index(name)
        cells = {name: [] for name in columns}
        for row in rd:
            if not row:
                continue
            for name, j in idx.items():
                cells[name].append(row[j] if j < len(row) else "")
    return {name: _parse_text_column(cells[name]) for name in columns}


def load_table(path: pathlib.Path, fmt: str, columns: Sequence[str]):
    """tools/dataframe_to_fe_binary.py:63-84 without pandas."""
    if fmt == "auto":
        suf = path.suffix.lower()
        fmt = "parquet" if suf in (".parquet", ".pq") else ("pickle" if suf in (".pkl", ".pickle") else "csv")
    cols = list(dict.fromkeys(columns))
    if fmt == "csv":
        return read_csv(path, cols)
    if fmt == "parquet":
        try:
            import pyarrow.parquet as pq
        except ImportError as e:
            raise RuntimeError("parquet input needs pyarrow") from e
        return pq.read_table(path, columns=cols)
    if fmt == "pickle":
        with open(path, "rb") as f:
            return pickle.load(f)
    raise ValueError(f"unsupported format: {fmt}")


def missing_mask(a: np.ndarray) -> np.ndarray:
    if a.dtype.kind == "f":
        return np.isnan(a)
    if a.dtype.kind == "O":
        return np.array([v is None or (isinstance(v, float) and np.isnan(v)) for v in a], dtype=bool)
    return np.zeros(a.shape[0], dtype=bool)


# ---------------------------------------------------------------- convert

def dataframe_to_fe_binary(table, output, *, y: str, x: Sequence[str], fe: Sequence[str],
                           iv: Sequence[str] = (), cluster: Optional[str] = None, weights: Optional[str] = None,
                           precision: str = "float64", drop_missing: bool = False,
                           compact: Callable[[np.ndarray], np.ndarray] = device_compact, log=None) -> dict:
    """Writes `table` as an fe_gpu binary dataset (tools/dataframe_to_fe_binary.py:186-277)
    and returns its summary."""
    if precision not in PRECISION_FLAGS:
        raise ValueError(f"precision must be one of {sorted(PRECISION_FLAGS)}")
    if not x:
        raise ValueError("at least one regressor is required")
    if not fe:
        raise ValueError("at least one FE column is required")
    log = log or (lambda msg: None)
    names = [y] + list(x) + list(fe) + list(iv) + ([cluster] if cluster else []) + ([weights] if weights else [])
    names = list(dict.fromkeys(names))
    cols = {name: column(table, name) for name in names}
    n = {a.shape[0] for a in cols.values()}
    if len(n) != 1:
        raise ValueError("columns differ in length")
    miss = np.zeros(next(iter(n)), dtype=bool)
    for a in cols.values():
        miss |= missing_mask(a)
    if miss.any():
        if not drop_missing:
            raise ValueError("Dataset contains missing values; rerun with --drop-missing")
        keep = ~miss
        cols = {k: v[keep] for k, v in cols.items()}
        log(f"Dropped {int(miss.sum())} rows containing missing values")
    n_obs = next(iter(cols.values())).shape[0]
    if n_obs == 0:
        raise ValueError("No observations remain after processing")

    def num(name):
        a = cols[name]
        if a.dtype.kind not in "biuf":
            raise ValueError(f"column {name!r} is not numeric")
        return a.astype(np.float64)

    yv = num(y)
    W = np.asfortranarray(np.column_stack([num(c) for c in x]))
    Z = np.asfortranarray(np.column_stack([num(c) for c in iv])) if iv else None
    t0 = time.perf_counter()
    fe_ids = np.stack([relabel_ids(cols[c], compact) for c in fe], axis=0)
    log(f"Relabeled FE columns in {time.perf_counter() - t0:.3f} s")
    cl = relabel_ids(cols[cluster], compact) if cluster else None
    wv = num(weights) if weights else None
    meta = {"y": y, "x": list(x), "iv": list(iv), "fe": list(fe), "cluster": cluster or "",
            "weights": weights or ""}
    write_dataset(str(output), yv, W, fe_ids, Z=Z, cluster=cl, weights=wv,
                  precision_flag=PRECISION_FLAGS[precision], metadata=meta)
    return {"n_obs": int(n_obs), "n_regressors": int(W.shape[1]), "n_fe_dims": int(fe_ids.shape[0]),
            "n_instruments": int(0 if Z is None else Z.shape[1]), "clustered": cluster is not None,
            "weights": weights is not None, "precision": precision}


def _columns_arg(value: str):
    items = [c.strip() for c in value.split(",") if c.strip()]
    if not items:
        raise argparse.ArgumentTypeError("At least one column must be provided")
    return items


def _optional_columns_arg(value: str):
    return [c.strip() for c in (value or "").split(",") if c.strip()]


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description="Convert tabular data to the fe_gpu binary format.")
    ap.add_argument("input", type=pathlib.Path)
    ap.add_argument("--input-format", choices=["auto", "csv", "parquet", "pickle"], default="auto")
    ap.add_argument("--output", type=pathlib.Path, required=True)
    ap.add_argument("--y", required=True)
    ap.add_argument("--x", required=True, type=_columns_arg)
    ap.add_argument("--fe", required=True, type=_columns_arg)
    ap.add_argument("--iv", type=_optional_columns_arg, default=[])
    ap.add_argument("--cluster", default=None)
    ap.add_argument("--weights", default=None)
    ap.add_argument("--precision", choices=list(PRECISION_FLAGS), default="float64")
    ap.add_argument("--drop-missing", action="store_true")
    ap.add_argument("--summary", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--workers", type=int, default=None, help="accepted for compatibility; the relabelling runs on the GPU")
    args = ap.parse_args(argv)
    log = (lambda m: print(m, file=sys.stderr)) if args.verbose else None
    names = [args.y] + args.x + args.fe + args.iv + ([args.cluster] if args.cluster else []) + (
        [args.weights] if args.weights else [])
    table = load_table(args.input, args.input_format, names)
    info = dataframe_to_fe_binary(table, args.output, y=args.y, x=args.x, fe=args.fe, iv=args.iv,
                                  cluster=args.cluster, weights=args.weights, precision=args.precision,
                                  drop_missing=args.drop_missing, log=log)
    if args.summary:
        print(json.dumps(info, indent=2))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
