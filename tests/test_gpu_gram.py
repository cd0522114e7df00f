"""Gram products behind the normal equations and the single-row cluster
meats (X'X over n rows) against an FP64 numpy reference: the split-FP32
(double-single) rows kernel up to 10 columns, the register-blocked kernel for
wider matrices (4 x 4 output blocks per thread, ragged last block) and the
FP64 form."""
import ctypes as C

import numpy as np
import pytest

from fe_gpu_gb300 import _native as N

pytestmark = pytest.mark.gpu


def gram(X, split):
    X = np.ascontiguousarray(X, dtype=np.float64)
    n, a = X.shape
    out = np.zeros((a, a), order="F")
    N.check(N.lib().fegb_test_gram(X.ctypes.data, n, a, split, out.ctypes.data), "fegb_test_gram")
    return out


@pytest.mark.parametrize("n,a", [(100_000, 7), (250_000, 11), (100_003, 111), (50_000, 90), (4096, 33), (70_001, 200)])
def test_gram_matches_fp64(built, n, a):
    rng = np.random.default_rng(a)
    X = rng.normal(size=(n, a)) * rng.uniform(0.1, 10.0, size=a)
    X[:, 0] += 3.0  # a column with a large mean
    ref = X.T @ X
    for split in (1, 0):
        got = gram(X, split)
        np.testing.assert_allclose(got, got.T, rtol=0, atol=0)
        scale = np.sqrt(np.outer(np.diag(ref), np.diag(ref)))
        err = np.max(np.abs(got - ref) / scale)
        # double-single products: about 2^-44 of each sum of |products|
        assert err < (1e-11 if split else 1e-13), (split, err)
