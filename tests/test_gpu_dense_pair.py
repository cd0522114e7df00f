"""The CG operator's dense count-matrix pass (fegb_test_dense_pair) against
numpy in FP64: the FP32 CUDA-core form and the tensor-core form (tcgen05,
BF16 pieces, FP32 accumulation in tensor memory), plain, accumulating and
Schur forms, ragged sizes (partial tiles of 128 groups, blocks without
groups, small dimensions above 32 groups, columns that are not a multiple of
8, counts up to 255, group counts aligned or not). Shapes the tensor-core form
does not take (C > 16) check its fallback to the CUDA-core form.

Tolerance: 5e-6 of the largest magnitude, for FP32 accumulation of sums of up
to a few hundred terms."""
import ctypes as C

import numpy as np
import pytest

from fe_gpu_gb300 import _native as N

pytestmark = pytest.mark.gpu


def row_stride(cols):
    # the CG tables' FP32 row stride: 32-byte multiples, 16-column multiples above 16
    return (cols + 7) // 8 * 8 if cols <= 16 else (cols + 15) // 16 * 16


def ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def run(counts, pe, ps, ld, cols, sums=None, group_counts=None, extra_in=None, accumulate=0, tensor_cores=1):
    ge, gs = counts.shape
    small = np.zeros((gs, cols), dtype=np.float64)
    extra = None if extra_in is None else extra_in.copy()
    table = np.zeros((ge, ld), dtype=np.float32) if sums is not None else None
    st = N.lib().fegb_test_dense_pair(ptr(counts), ge, gs, ptr(pe), ptr(ps), ld, cols, ptr(sums), ptr(group_counts),
                                      accumulate, tensor_cores, ptr(small), ptr(extra), ptr(table))
    N.check(st, "fegb_test_dense_pair")
    return small, extra, table


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("tensor_cores", [1, 0])
@pytest.mark.parametrize("ge,gs,cols,maxc", [(5000, 20, 9, 1), (3001, 33, 3, 7), (700, 7, 17, 255), (64, 64, 32, 3),
                                             (200_000, 30, 9, 1), (100_003, 30, 16, 255), (129, 64, 1, 2),
                                             (77_777, 64, 12, 40), (2, 1, 9, 3)])
def test_dense_pair_matches_numpy(built, tensor_cores, ge, gs, cols, maxc):
    rng = np.random.default_rng(ge + gs + cols)
    ld = row_stride(cols)
    counts = rng.integers(0, maxc + 1, size=(ge, gs)).astype(np.uint8)
    pe = np.zeros((ge, ld), dtype=np.float32)
    ps = np.zeros((gs, ld), dtype=np.float32)
    pe[:, :cols] = rng.standard_normal((ge, cols))
    ps[:, :cols] = rng.standard_normal((gs, cols))
    nf = counts.astype(np.float64)
    ref_small = -(nf.T @ pe[:, :cols].astype(np.float64))
    ref_extra = nf @ ps[:, :cols].astype(np.float64)
    # plain: both sides, overwrite
    small, extra, _ = run(counts, pe, ps, ld, cols, extra_in=np.zeros((ge, cols), np.float32),
                          tensor_cores=tensor_cores)
    assert rel(small, ref_small) < 5e-6
    assert rel(extra, ref_extra) < 5e-6
    # accumulate into the values passed in
    base = rng.standard_normal((ge, cols)).astype(np.float32)
    _, extra2, _ = run(counts, pe, ps, ld, cols, extra_in=base, accumulate=1, tensor_cores=tensor_cores)
    assert rel(extra2, base + ref_extra) < 5e-6
    # Schur form: u = (sums - N ps) / n written to the table and used as pe
    sums = rng.standard_normal((ge, cols)).astype(np.float32) * 5
    gcount = rng.integers(0, 40, size=ge).astype(np.int32)
    small3, _, table = run(counts, None, ps, ld, cols, sums=sums, group_counts=gcount, tensor_cores=tensor_cores)
    u = np.where(gcount[:, None] > 0, (sums.astype(np.float64) - ref_extra) / np.maximum(gcount, 1)[:, None], 0.0)
    assert rel(table[:, :cols], u) < 5e-6
    assert np.all(table[:, cols:] == 0)
    assert rel(small3, -(nf.T @ u)) < 5e-6
