"""The C-ABI library loads without a GPU and exports every symbol that the
public headers declare (include/fe_gpu_runtime.h, include/fegb.h)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADERS = sorted((ROOT / "include").glob("*.h"))
DECL = re.compile(r"^\s*(?:int|void|long long)\s+([A-Za-z_][A-Za-z0-9_]*)\s*\(", re.M)


def declared_symbols():
    names = []
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += DECL.findall(text)
    return sorted(set(names))


def test_headers_declare_reference_boundary():
    names = set(declared_symbols())
    # the 27 entry points of the reference kernel-level ABI plus the host cluster builder
    reference = {
        "fe_gpu_runtime_is_available", "fe_gpu_runtime_init", "fe_gpu_runtime_shutdown", "fe_gpu_runtime_malloc",
        "fe_gpu_runtime_free", "fe_gpu_runtime_memcpy_htod", "fe_gpu_runtime_memcpy_dtoh",
        "fe_gpu_runtime_memcpy_dtod", "fe_gpu_runtime_memset", "fe_gpu_runtime_get_last_error",
        "fe_gpu_runtime_clear_error", "fe_gpu_linalg_init", "fe_gpu_linalg_shutdown", "fe_gpu_syrk", "fe_gpu_gemv",
        "fe_gpu_residual", "fe_gpu_dot", "fe_gpu_gemm", "fe_gpu_cluster_scores", "fe_gpu_cluster_meat",
        "fe_gpu_fe_accumulate", "fe_gpu_fe_compute_means", "fe_gpu_fe_subtract", "fe_gpu_mix_means", "fe_gpu_axpy",
        "fe_gpu_absmax", "fe_gpu_copy_columns", "fe_gpu_build_multi_cluster_ids", "fe_build_cluster_ids",
    }
    assert reference <= names


def test_library_exports_every_declared_symbol(built):
    from fe_gpu_gb300 import _native

    lib = ctypes.CDLL(str(_native.library_path()))
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding table covers the same set
    assert set(declared_symbols()) == set(_native.SIGNATURES)


def test_last_error_roundtrip_without_gpu(built):
    from fe_gpu_gb300 import _native

    lib = _native.lib()
    assert lib.fe_gpu_runtime_clear_error() == 0
    assert _native.last_error() == "OK"
    # a host-side argument error sets the message and a nonzero status without touching a device
    st = lib.fe_gpu_copy_columns(None, 1, None, 1, 1, None, 1, 0)
    assert st != 0
    assert "Invalid buffers" in _native.last_error()


def test_missing_library_fails_loudly(tmp_path, monkeypatch):
    from fe_gpu_gb300 import _native

    monkeypatch.setattr(_native, "_lib", None)
    monkeypatch.setattr(_native, "_LIB_PATH", tmp_path / "nope.so")
    with pytest.raises(_native.FeGpuError):
        _native.lib()
