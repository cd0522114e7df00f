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
