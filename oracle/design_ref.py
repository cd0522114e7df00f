"""TEST INFRASTRUCTURE ONLY -- not part of the product path.

numpy restatement of the reference's per-row formula expansion, the checker
for fegb_design_levels / fegb_build_design:

* collect_levels  -- collect_levels_for_column (src/src_main.f90:1390-1435):
                     scan the column in row order, keep values within 1e-6 of
                     nint(x), stop at the 40th distinct value, sort ascending.
* design_column   -- a dummy is 1.0 where int(nint(x)) == level
                     (append_main_term_columns :1209-1227, build_factor_block
                     :1356-1377); interaction columns multiply factor blocks
                     left to right (append_interaction_columns :1286-1300).
* expand          -- the whole expanded matrix for a list of factor recipes.

Fortran nint rounds halves away from zero; it is restated exactly as
trunc(x) + sign(x) * (|x - trunc(x)| >= 0.5).
"""
from __future__ import annotations

import numpy as np

MAX_CATEGORIES = 40
CATEGORY_TOL = 1.0e-6


def nint(x: np.ndarray) -> np.ndarray:
    x = np.asarray(x, dtype=np.float64)
    t = np.trunc(x)
    return t + np.sign(x) * (np.abs(x - t) >= 0.5)


def _int32_ok(r: np.ndarray) -> np.ndarray:
    return np.abs(r) <= 2147483647.0


def collect_levels(col: np.ndarray, max_levels: int = MAX_CATEGORIES) -> list:
    x = np.asarray(col, dtype=np.float64)
    r = nint(x)
    ok = _int32_ok(r) & (np.abs(x - r) <= CATEGORY_TOL)
    vals = r[ok].astype(np.int64)
    if vals.size == 0:
        return []
    uniq, first = np.unique(vals, return_index=True)
    order = np.argsort(first, kind="stable")[:max_levels]
    return sorted(int(v) for v in uniq[order])


def dummy(col: np.ndarray, level: int) -> np.ndarray:
    r = nint(col)
    return np.where(_int32_ok(r) & (r == level), 1.0, 0.0)


def design_column(sources: dict, factors) -> np.ndarray:
    """factors: [(matrix, col, level_or_None)]; sources[(matrix, col)] -> column."""
    out = None
    for (m, c, lv) in factors:
        f = sources[(m, c)] if lv is None else dummy(sources[(m, c)], lv)
        out = f.copy() if out is None else out * f
    return out


def expand(sources: dict, columns) -> np.ndarray:
    n = len(next(iter(sources.values())))
    out = np.zeros((n, len(columns)), order="F")
    for j, factors in enumerate(columns):
        out[:, j] = design_column(sources, factors)
    return out
