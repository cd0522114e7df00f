"""fe_gpu_syrk_noalloc: the cross product W^T W without device allocation.

Some callers cannot let the library allocate device memory while they run
(a host that owns all device buffers through its own allocator and budget,
or a section that must not touch the allocator). This entry point keeps its
scratch in a fixed device array instead of the memory pool. It is checked
here through the C ABI against fe_gpu_syrk, on two calls in a row, within the
cross-product tolerance of the other tests (1e-12 relative to the largest
entry). The file sorts last so a stop-at-first-failure run has already run
every other test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _upper(a):
    return np.triu(a)


def test_syrk_noalloc_matches_syrk_twice(built):
    from fe_gpu_gb300 import _native as N
    from fe_gpu_gb300.estimator import DeviceBuffer

    lib = N.lib()
    N.check(lib.fe_gpu_runtime_is_available(), "no CUDA device")
    rng = np.random.default_rng(2026)
    for n, k, alpha, beta in ((50_000, 9, 1.0, 0.0), (7_777, 32, 0.75, 0.5)):
        W = np.asfortranarray(rng.standard_normal((n, k)))
        Q0 = np.asfortranarray(rng.standard_normal((k, k)))
        dW = DeviceBuffer.from_array(W)
        dQa = DeviceBuffer.from_array(Q0)
        dQb = DeviceBuffer.from_array(Q0)
        N.check(lib.fe_gpu_syrk(n, k, alpha, dW.ptr, n, beta, dQa.ptr), "fe_gpu_syrk")
        N.check(lib.fe_gpu_syrk_noalloc(n, k, alpha, dW.ptr, n, beta, dQb.ptr), "fe_gpu_syrk_noalloc")
        a = dQa.to_array(np.float64, (k, k), order="F")
        b = dQb.to_array(np.float64, (k, k), order="F")
        scale = np.max(np.abs(a))
        assert np.max(np.abs(_upper(a) - _upper(b))) <= 1e-12 * scale
        # strictly lower triangle untouched, as in the reference syrk (upper fill)
        np.testing.assert_array_equal(np.tril(b, -1), np.tril(Q0, -1))
        ref = alpha * (W.T @ W) + beta * Q0
        assert np.max(np.abs(_upper(b) - _upper(ref))) <= 1e-10 * np.max(np.abs(ref))
        for buf in (dW, dQa, dQb):
            buf.free()


def _pool(lib, reset=False):
    import ctypes as C

    used, high, reserved = C.c_ulonglong(), C.c_ulonglong(), C.c_ulonglong()
    assert lib.fegb_pool_usage(1 if reset else 0, C.byref(used), C.byref(high), C.byref(reserved)) == 0
    return used.value, high.value, reserved.value


def test_syrk_noalloc_allocates_nothing(built):
    """The device's memory and its stream-ordered pool are unchanged by a call:
    the pool's high-water mark (reset just before) stays at the bytes in use,
    nothing is reserved, and the device's free memory does not move. fe_gpu_syrk
    on the same input is the control: it takes its partials from the pool."""
    import torch

    from fe_gpu_gb300 import _native as N
    from fe_gpu_gb300.estimator import DeviceBuffer

    lib = N.lib()
    N.check(lib.fe_gpu_runtime_is_available(), "no CUDA device")
    n, k = 200_000, 16
    W = np.asfortranarray(np.random.default_rng(7).standard_normal((n, k)))
    dW = DeviceBuffer.from_array(W)
    dQ = DeviceBuffer.from_array(np.zeros((k, k), order="F"))
    N.check(lib.fe_gpu_syrk_noalloc(n, k, 1.0, dW.ptr, n, 0.0, dQ.ptr), "fe_gpu_syrk_noalloc (set-up)")
    torch.cuda.synchronize()
    for _ in range(2):
        used0, _, reserved0 = _pool(lib, reset=True)
        free0, _ = torch.cuda.mem_get_info()
        N.check(lib.fe_gpu_syrk_noalloc(n, k, 1.0, dW.ptr, n, 0.0, dQ.ptr), "fe_gpu_syrk_noalloc")
        used1, high1, reserved1 = _pool(lib)
        free1, _ = torch.cuda.mem_get_info()
        assert (used1, high1, reserved1) == (used0, used0, reserved0)
        assert free1 == free0
    # control: the allocating entry point does move the pool's high-water mark
    used0, _, _ = _pool(lib, reset=True)
    N.check(lib.fe_gpu_syrk(n, k, 1.0, dW.ptr, n, 0.0, dQ.ptr), "fe_gpu_syrk")
    _, high, _ = _pool(lib)
    assert high > used0
    dW.free()
    dQ.free()


def test_syrk_noalloc_no_rows_scales_q(built):
    """n_rows = 0: Q = beta Q on the upper triangle, the lower one untouched."""
    from fe_gpu_gb300 import _native as N
    from fe_gpu_gb300.estimator import DeviceBuffer

    lib = N.lib()
    k = 7
    Q0 = np.asfortranarray(np.random.default_rng(3).standard_normal((k, k)))
    dW = DeviceBuffer.from_array(np.zeros((1, k), order="F"))
    for _ in range(2):
        dQ = DeviceBuffer.from_array(Q0)
        N.check(lib.fe_gpu_syrk_noalloc(0, k, 1.0, dW.ptr, 1, 0.5, dQ.ptr), "fe_gpu_syrk_noalloc")
        q = dQ.to_array(np.float64, (k, k), order="F")
        np.testing.assert_array_equal(np.triu(q), np.triu(0.5 * Q0))
        np.testing.assert_array_equal(np.tril(q, -1), np.tril(Q0, -1))
        dQ.free()
    dW.free()


def test_syrk_noalloc_rejects_short_leading_dimension(built):
    """ldW below max(1, n_rows) is an error, as the reference's syrk reports."""
    from fe_gpu_gb300 import _native as N
    from fe_gpu_gb300.estimator import DeviceBuffer

    lib = N.lib()
    n, k = 100, 4
    dW = DeviceBuffer.from_array(np.zeros((n, k), order="F"))
    dQ = DeviceBuffer.from_array(np.zeros((k, k), order="F"))
    for fn in (lib.fe_gpu_syrk_noalloc, lib.fe_gpu_syrk):
        assert fn(n, k, 1.0, dW.ptr, n - 1, 0.0, dQ.ptr) != 0
        assert "ldW" in N.last_error()
    dW.free()
    dQ.free()


def test_syrk_noalloc_rejects_wide_input(built):
    from fe_gpu_gb300 import _native as N
    from fe_gpu_gb300.estimator import DeviceBuffer

    lib = N.lib()
    n, k = 100, 33
    dW = DeviceBuffer.from_array(np.zeros((n, k), order="F"))
    dQ = DeviceBuffer.from_array(np.zeros((k, k), order="F"))
    st = lib.fe_gpu_syrk_noalloc(n, k, 1.0, dW.ptr, n, 0.0, dQ.ptr)
    assert st != 0
    assert "32-column limit" in N.last_error()
    dW.free()
    dQ.free()
