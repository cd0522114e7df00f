"""The kernel-level C ABI (include/fe_gpu_runtime.h, the reference's
src/gpu/fe_gpu_runtime.h:14-131) on the device, entry point by entry point,
against numpy restatements of the reference kernels' semantics
(src/gpu/fe_gpu_runtime.cu, src/gpu/fe_gpu_linalg.cu): group sums by 1-based
ids (ids <= 0 skipped), means by the reciprocal count, subtraction,
over-relaxed mixing, cross products, residuals, cluster scores and meat,
column copies and multi-way cluster ids."""
import ctypes as C

import numpy as np
import pytest

from fe_gpu_gb300 import _native as N
from fe_gpu_gb300.estimator import DeviceBuffer
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def dev(a):
    return DeviceBuffer.from_array(np.asfortranarray(a))


def host(b, dtype, shape, order="F"):
    return b.to_array(dtype, shape, order=order)


def ok(st, what):
    N.check(st, what)


def test_runtime_init_and_memory(built):
    lib = N.lib()
    assert lib.fe_gpu_runtime_is_available() == 0
    info = N.FeGpuDeviceInfo()
    ok(lib.fe_gpu_runtime_init(0, C.byref(info)), "init")
    assert info.multiprocessor_count > 0 and info.total_global_mem > 0
    a = np.arange(1000, dtype=np.float64)
    b = dev(a)
    c = DeviceBuffer(a.nbytes)
    ok(lib.fe_gpu_runtime_memcpy_dtod(c.ptr, b.ptr, a.nbytes), "dtod")
    assert np.array_equal(host(c, np.float64, (1000,)), a)
    ok(lib.fe_gpu_runtime_memset(c.ptr, 0, a.nbytes), "memset")
    assert not host(c, np.float64, (1000,)).any()


def test_linear_algebra(built):
    lib = N.lib()
    rng = np.random.default_rng(1)
    n, k = 50_001, 7
    W = rng.standard_normal((n, k))
    y = rng.standard_normal(n)
    dW, dy = dev(W), dev(y)
    # syrk: upper triangle of alpha W'W + beta Q
    Q0 = rng.standard_normal((k, k))
    dQ = dev(Q0)
    ok(lib.fe_gpu_syrk(n, k, 0.5, dW.ptr, n, 2.0, dQ.ptr), "syrk")
    Q = host(dQ, np.float64, (k, k))
    ref = 0.5 * W.T @ W + 2.0 * Q0
    iu = np.triu_indices(k)
    assert np.allclose(Q[iu], ref[iu], rtol=1e-12, atol=1e-9)
    # gemv: b = alpha W'y + beta b
    b0 = rng.standard_normal(k)
    db = dev(b0)
    ok(lib.fe_gpu_gemv(n, k, 1.5, dW.ptr, n, dy.ptr, -1.0, db.ptr), "gemv")
    assert np.allclose(host(db, np.float64, (k,)), 1.5 * W.T @ y - b0, rtol=1e-12, atol=1e-9)
    # residual and dot
    beta = rng.standard_normal(k)
    dbeta, dr = dev(beta), DeviceBuffer(8 * n)
    ok(lib.fe_gpu_residual(n, k, dW.ptr, n, dbeta.ptr, dy.ptr, dr.ptr), "residual")
    r = host(dr, np.float64, (n,))
    assert np.allclose(r, y - W @ beta, rtol=1e-13, atol=1e-12)
    out = C.c_double(0)
    ok(lib.fe_gpu_dot(n, dr.ptr, dr.ptr, C.byref(out)), "dot")
    assert abs(out.value - r @ r) < 1e-10 * (r @ r)
    # gemm, both code paths
    A = rng.standard_normal((6000, 5))
    B = rng.standard_normal((6000, 3))
    dA, dB, dC = dev(A), dev(B), DeviceBuffer(8 * 15)
    ok(lib.fe_gpu_gemm(b"T", b"N", 5, 3, 6000, 1.0, dA.ptr, 6000, dB.ptr, 6000, 0.0, dC.ptr, 5), "gemm tn")
    assert np.allclose(host(dC, np.float64, (5, 3)), A.T @ B, rtol=1e-12, atol=1e-10)
    M1, M2 = rng.standard_normal((4, 6)), rng.standard_normal((6, 5))
    d1, d2, d3 = dev(M1), dev(M2), DeviceBuffer(8 * 20)
    ok(lib.fe_gpu_gemm(b"N", b"N", 4, 5, 6, 2.0, d1.ptr, 4, d2.ptr, 6, 0.0, d3.ptr, 4), "gemm nn")
    assert np.allclose(host(d3, np.float64, (4, 5)), 2.0 * M1 @ M2, rtol=1e-13, atol=1e-13)


def test_demeaning_kernels(built):
    lib = N.lib()
    rng = np.random.default_rng(2)
    n, G, k, l = 100_003, 977, 3, 2
    ids = rng.integers(1, G + 1, n).astype(np.int32)
    ids[rng.random(n) < 0.01] = 0  # skipped rows
    ids[ids == 5] = 6               # group 5 empty
    y = rng.standard_normal(n)
    W = rng.standard_normal((n, k))
    Z = rng.standard_normal((n, l))
    dy, dW, dZ, dids = dev(y), dev(W), dev(Z), dev(ids)
    sy, sW, sZ = dev(np.zeros(G)), dev(np.zeros(G * k)), dev(np.zeros(G * l))
    cnt = dev(np.zeros(G, np.int32))
    ok(lib.fe_gpu_fe_accumulate(dy.ptr, dW.ptr, dZ.ptr, dids.ptr, n, G, k, l, n, sy.ptr, sW.ptr, sZ.ptr, cnt.ptr),
       "accumulate")
    m = ids > 0
    g = ids[m] - 1
    ref_y = np.bincount(g, weights=y[m], minlength=G)
    ref_W = np.stack([np.bincount(g, weights=W[m, j], minlength=G) for j in range(k)], 1)
    ref_Z = np.stack([np.bincount(g, weights=Z[m, j], minlength=G) for j in range(l)], 1)
    ref_c = np.bincount(g, minlength=G)
    assert np.array_equal(host(cnt, np.int32, (G,)), ref_c)
    assert np.allclose(host(sy, np.float64, (G,)), ref_y, rtol=1e-12, atol=1e-12)
    assert np.allclose(host(sW, np.float64, (G, k), order="C"), ref_W, rtol=1e-12, atol=1e-12)
    assert np.allclose(host(sZ, np.float64, (G, l), order="C"), ref_Z, rtol=1e-12, atol=1e-12)
    # the same sums in a fixed order: a second call adds bitwise-identical values
    a1 = host(sW, np.float64, (G * k,))
    ok(lib.fe_gpu_fe_accumulate(dy.ptr, dW.ptr, dZ.ptr, dids.ptr, n, G, k, l, n, sy.ptr, sW.ptr, sZ.ptr, cnt.ptr),
       "accumulate again")
    assert np.array_equal(host(sW, np.float64, (G * k,)), a1 + a1)
    assert np.array_equal(host(cnt, np.int32, (G,)), 2 * ref_c)
    # means: sums times the reciprocal count (empty groups give 0)
    ok(lib.fe_gpu_fe_compute_means(sy.ptr, sW.ptr, sZ.ptr, cnt.ptr, G, k, l), "means")
    c2 = 2 * ref_c
    inv = np.where(c2 > 0, 1.0 / np.maximum(c2, 1), 0.0)
    my = host(sy, np.float64, (G,))
    mW = host(sW, np.float64, (G, k), order="C")
    assert np.allclose(my, 2 * ref_y * inv, rtol=1e-12, atol=1e-14)
    assert np.allclose(mW, 2 * ref_W * inv[:, None], rtol=1e-12, atol=1e-14)
    # subtract: rows with id <= 0 untouched
    mZ = host(sZ, np.float64, (G, l), order="C")
    ok(lib.fe_gpu_fe_subtract(dy.ptr, dW.ptr, dZ.ptr, dids.ptr, n, k, l, n, sy.ptr, sW.ptr, sZ.ptr, 1.0), "subtract")
    ey = y.copy()
    ey[m] -= my[g]
    eW = W.copy()
    eW[m] -= mW[g]
    eZ = Z.copy()
    eZ[m] -= mZ[g]
    assert np.array_equal(host(dy, np.float64, (n,)), ey)
    assert np.array_equal(host(dW, np.float64, (n, k)), eW)
    assert np.array_equal(host(dZ, np.float64, (n, l)), eZ)
    # over-relaxed mixing, axpy, absmax
    mean, prev = rng.standard_normal(5000), rng.standard_normal(5000)
    dm, dp = dev(mean), dev(prev)
    ok(lib.fe_gpu_mix_means(dm.ptr, dp.ptr, 5000, 1.5), "mix")
    mixed = prev + 1.5 * (mean - prev)
    assert np.allclose(host(dm, np.float64, (5000,)), mixed, rtol=1e-15, atol=1e-15)
    assert np.array_equal(host(dm, np.float64, (5000,)), host(dp, np.float64, (5000,)))
    x = rng.standard_normal(5000)
    dx = dev(x)
    ok(lib.fe_gpu_axpy(5000, -0.25, dx.ptr, dp.ptr), "axpy")
    assert np.allclose(host(dp, np.float64, (5000,)), host(dm, np.float64, (5000,)) - 0.25 * x, rtol=1e-15,
                       atol=1e-15)
    out = C.c_double(0)
    ok(lib.fe_gpu_absmax(dx.ptr, 5000, C.byref(out)), "absmax")
    assert out.value == np.max(np.abs(x))


def test_cluster_scores_and_meat(built):
    lib = N.lib()
    rng = np.random.default_rng(3)
    n, k, G = 80_000, 4, 1200
    W = rng.standard_normal((n, k))
    r = rng.standard_normal(n)
    ids = rng.integers(1, G + 1, n).astype(np.int32)
    ids[:50] = 0
    dW, dr, dids = dev(W), dev(r), dev(ids)
    S0 = rng.standard_normal((G, k))
    dS = dev(S0)
    ok(lib.fe_gpu_cluster_scores(dr.ptr, dW.ptr, dids.ptr, n, k, n, G, dS.ptr), "scores")
    m = ids > 0
    ref = S0 + np.stack([np.bincount(ids[m] - 1, weights=r[m] * W[m, j], minlength=G) for j in range(k)], 1)
    S = host(dS, np.float64, (G, k))
    assert np.allclose(S, ref, rtol=1e-12, atol=1e-11)
    dM = DeviceBuffer(8 * k * k)
    ok(lib.fe_gpu_cluster_meat(G, k, dS.ptr, G, dM.ptr), "meat")
    M = host(dM, np.float64, (k, k))
    iu = np.triu_indices(k)
    assert np.allclose(M[iu], (S.T @ S)[iu], rtol=1e-12, atol=1e-10)


def test_copy_columns_and_cluster_ids(built):
    lib = N.lib()
    rng = np.random.default_rng(4)
    n = 10_000
    A = rng.standard_normal((n, 5))
    dA, dD = dev(A), DeviceBuffer(8 * n * 4)
    idx = np.array([5, 2], np.int32)
    ok(lib.fe_gpu_copy_columns(dA.ptr, n, idx.ctypes.data_as(C.POINTER(C.c_int)), 2, n, dD.ptr, n, 1), "copy")
    D = host(dD, np.float64, (n, 4))
    assert np.array_equal(D[:, 1], A[:, 4]) and np.array_equal(D[:, 2], A[:, 1])
    sizes = [300, 17, 9]
    fe = np.vstack([rng.integers(1, s + 1, n) for s in sizes]).astype(np.int32)
    dfe = [dev(fe[d]) for d in range(3)]
    for subset in ([1, 2], [1, 3], [2, 3], [1, 2, 3]):
        strides, acc = [], 1
        for d in subset:
            strides.append(acc)
            acc *= sizes[d - 1]
        ptrs = (C.c_void_p * len(subset))(*[C.c_void_p(dfe[d - 1].ptr) for d in subset])
        st = (C.c_ulonglong * len(subset))(*strides)
        dout = DeviceBuffer(4 * n)
        nc = C.c_int(0)
        ok(lib.fe_gpu_build_multi_cluster_ids(ptrs, st, len(subset), n, dout.ptr, C.byref(nc)), "multi ids")
        ids, ncl, _ = O.cluster_ids(fe, np.array(sizes), subset)
        assert nc.value == ncl
        assert np.array_equal(host(dout, np.int32, (n,)), ids)
        # the host-array builder (cluster_id_builder.c interface), on the device
        dims = np.array(subset, np.int32)
        szs = np.array([sizes[d - 1] for d in subset], np.int32)
        out = np.zeros(n, np.int32)
        nc2 = C.c_int(0)
        fef = np.asfortranarray(fe)
        code = lib.fe_build_cluster_ids(fef.ctypes.data, 3, n, dims.ctypes.data_as(C.POINTER(C.c_int)),
                                        szs.ctypes.data_as(C.POINTER(C.c_int)), len(subset), out.ctypes.data,
                                        C.byref(nc2))
        assert code == 0 and nc2.value == ncl and np.array_equal(out, ids)
