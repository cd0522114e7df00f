"""The FP64 group-sum sweeps behind the within-transform's group means
(fegb_test_group_sums), segment and small-G forms, against numpy in FP64.

Tolerance: |gpu - numpy| <= 1e-13 * sum |x| over the group (the two differ
only in the order of the FP64 additions)."""
import ctypes as C

import numpy as np
import pytest

from fe_gpu_gb300 import _native as N

pytestmark = pytest.mark.gpu


def ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def run(X, gid, G, small_g):
    X = np.ascontiguousarray(X, dtype=np.float64)
    gid = np.ascontiguousarray(gid, dtype=np.int32)
    n, cols = X.shape
    out = np.zeros((G, cols), dtype=np.float64)
    st = N.lib().fegb_test_group_sums(ptr(X), n, cols, ptr(gid), G, small_g, ptr(out))
    N.check(st, "fegb_test_group_sums")
    return out


def reference(X, gid, G):
    s = np.zeros((G, X.shape[1]))
    a = np.zeros((G, X.shape[1]))
    np.add.at(s, gid, X)
    np.add.at(a, gid, np.abs(X))
    return s, a


def case(form, n, G, cols, seed):
    rng = np.random.default_rng(seed)
    if form == "segment":
        # Pareto-like group sizes: some groups span many 256-row chunks, some are empty at the end
        sizes = np.maximum(1, (rng.pareto(1.2, G) * 5).astype(np.int64))
        gid = np.repeat(np.arange(G), sizes)[:n]
        gid = np.concatenate([gid, np.full(max(0, n - gid.size), G - 1)]).astype(np.int32)
    else:
        gid = rng.integers(0, G, n).astype(np.int32)
    X = rng.standard_normal((n, cols)) + 3.0
    return X, gid


@pytest.mark.parametrize("form,G,cols", [("segment", 5000, 9), ("segment", 37, 1), ("segment", 200_003, 3),
                                         ("small", 20, 9), ("small", 60, 3)])
def test_group_sums_match_numpy(built, form, G, cols):
    X, gid = case(form, 200_003, G, cols, seed=G + cols)
    out = run(X, gid, G, form == "small")
    ref, mag = reference(X, gid, G)
    assert np.all(np.abs(out - ref) <= 1e-13 * mag)


@pytest.mark.parametrize("form", ["segment", "small"])
def test_group_sums_wide_range_and_nonfinite(built, form):
    # magnitudes from 2^-50 to 2^100 and a non-finite value: FP64 additions take them all
    X, gid = case(form, 50_000, 20, 4, seed=7)
    X[:, 1] *= 2.0 ** 100
    X[:, 2] *= 2.0 ** -50
    X[1234, 3] = np.inf
    out = run(X, gid, 20, form == "small")
    ref, mag = reference(X, gid, 20)
    fin = np.isfinite(ref)
    assert np.all(np.abs(out[fin] - ref[fin]) <= 1e-13 * mag[fin])
    assert np.array_equal(np.isinf(out), np.isinf(ref))
