"""ctypes bindings to libfegb.so (the C ABI declared in include/fe_gpu_runtime.h
and include/fegb.h).

There is no fallback: if the shared library is missing or cannot be loaded,
every entry point raises FeGpuError. Build it with fe_gpu_gb300.build.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "_build" / "libfegb.so"
_lock = threading.Lock()
_lib = None


class FeGpuError(RuntimeError):
    """Nonzero status from the C ABI (message from fe_gpu_runtime_get_last_error)."""

    def __init__(self, status: int, message: str, where: str = ""):
        self.status = status
        self.message = message
        super().__init__(f"{where}: status {status}: {message}" if where else f"status {status}: {message}")


class FegbConfig(C.Structure):
    _fields_ = [
        ("fe_tol", C.c_double),
        ("fe_max_iter", C.c_int),
        ("precision", C.c_int),
        ("demean_method", C.c_int),
        ("se_convention", C.c_int),
        ("drop_singletons", C.c_int),
        ("n_cluster_dims", C.c_int),
        ("cluster_dims", C.POINTER(C.c_int)),
        ("n_iv_regressors", C.c_int),
        ("iv_regressors", C.POINTER(C.c_int)),
        ("n_iv_instruments", C.c_int),
        ("iv_instruments", C.POINTER(C.c_int)),
        ("verbose", C.c_int),
        ("stream", C.c_void_p),
        ("profile", C.c_int),
    ]


class FegbResult(C.Structure):
    _fields_ = [
        ("converged", C.c_int),
        ("fe_iterations", C.c_int),
        ("solver_info", C.c_int),
        ("rank", C.c_int),
        ("dof_model", C.c_int),
        ("dof_fes", C.c_int),
        ("dof_resid", C.c_longlong),
        ("is_iv", C.c_int),
        ("n_instruments", C.c_int),
        ("n_cluster_dims_used", C.c_int),
        ("psd_fix_applied", C.c_int),
        ("min_single_cluster", C.c_int),
        ("n_obs_used", C.c_longlong),
        ("n_singletons", C.c_longlong),
        ("max_update", C.c_double),
        ("rss", C.c_double),
        ("tss_total", C.c_double),
        ("tss_within", C.c_double),
        ("r2", C.c_double),
        ("r2_adj", C.c_double),
        ("r2_within", C.c_double),
        ("f_stat", C.c_double),
        ("projections", C.c_int),
        ("outer_iterations", C.c_int),
        ("demean_bytes", C.c_double),
        ("time_h2d", C.c_double),
        ("time_prep", C.c_double),
        ("time_demean", C.c_double),
        ("time_regression", C.c_double),
        ("time_se", C.c_double),
        ("time_total", C.c_double),
        ("prof_launches", C.c_int * 8),
        ("prof_seconds", C.c_double * 8),
        ("prof_bytes", C.c_double * 8),
    ]

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if name.startswith("prof_") else v
        return out


class FeGpuDeviceInfo(C.Structure):
    _fields_ = [
        ("device_id", C.c_int),
        ("total_global_mem", C.c_size_t),
        ("multiprocessor_count", C.c_int),
        ("major", C.c_int),
        ("minor", C.c_int),
        ("name", C.c_char * 256),
    ]


DESIGN_MAX_FACTORS = 8  # FEGB_DESIGN_MAX_FACTORS


class FegbDesignFactor(C.Structure):
    _fields_ = [("src", C.c_int), ("level", C.c_int), ("is_dummy", C.c_int)]


class FegbDesignColumn(C.Structure):
    _fields_ = [("n_factors", C.c_int), ("factors", FegbDesignFactor * DESIGN_MAX_FACTORS)]


class FegbSpec(C.Structure):
    _fields_ = [
        ("n", C.c_longlong),
        ("k", C.c_int),
        ("l", C.c_int),
        ("n_fe", C.c_int),
        ("y", C.c_void_p),
        ("W", C.c_void_p),
        ("Z", C.c_void_p),
        ("fe_ids", C.POINTER(C.c_void_p)),
        ("n_cluster_dims", C.c_int),
        ("cluster_dims", C.POINTER(C.c_int)),
        ("n_iv_regressors", C.c_int),
        ("iv_regressors", C.POINTER(C.c_int)),
        ("n_iv_instruments", C.c_int),
        ("iv_instruments", C.POINTER(C.c_int)),
    ]


class FegbDataset(C.Structure):
    _fields_ = [
        ("n", C.c_longlong),
        ("k", C.c_int),
        ("l", C.c_int),
        ("n_fe", C.c_int),
        ("has_cluster", C.c_int),
        ("has_weights", C.c_int),
        ("precision_flag", C.c_int),
        ("metadata_offset", C.c_longlong),
        ("y", C.c_void_p),
        ("W", C.c_void_p),
        ("Z", C.c_void_p),
        ("fe_ids", C.c_void_p),
        ("cluster", C.c_void_p),
        ("weights", C.c_void_p),
        ("seconds", C.c_double),
    ]


_P = C.c_void_p
_I = C.c_int
_LL = C.c_longlong
_D = C.c_double
_SZ = C.c_size_t
_IP = C.POINTER(C.c_int)
_DP = C.POINTER(C.c_double)

# name -> (restype, argtypes); mirrors include/fe_gpu_runtime.h and include/fegb.h
SIGNATURES = {
    "fe_gpu_runtime_is_available": (_I, []),
    "fe_gpu_runtime_init": (_I, [_I, C.POINTER(FeGpuDeviceInfo)]),
    "fe_gpu_runtime_shutdown": (_I, []),
    "fe_gpu_runtime_malloc": (_I, [C.POINTER(C.c_void_p), _SZ]),
    "fe_gpu_runtime_free": (_I, [_P]),
    "fe_gpu_runtime_memcpy_htod": (_I, [_P, _P, _SZ]),
    "fe_gpu_runtime_memcpy_dtoh": (_I, [_P, _P, _SZ]),
    "fe_gpu_runtime_memcpy_dtod": (_I, [_P, _P, _SZ]),
    "fe_gpu_runtime_memset": (_I, [_P, _I, _SZ]),
    "fe_gpu_runtime_get_last_error": (_I, [C.c_char_p, _SZ]),
    "fe_gpu_runtime_clear_error": (_I, []),
    "fe_gpu_linalg_init": (_I, []),
    "fe_gpu_linalg_shutdown": (_I, []),
    "fe_gpu_syrk": (_I, [_I, _I, _D, _P, _I, _D, _P]),
    "fe_gpu_syrk_noalloc": (_I, [_I, _I, _D, _P, _I, _D, _P]),
    "fe_gpu_gemv": (_I, [_I, _I, _D, _P, _I, _P, _D, _P]),
    "fe_gpu_residual": (_I, [_I, _I, _P, _I, _P, _P, _P]),
    "fe_gpu_dot": (_I, [_I, _P, _P, _DP]),
    "fe_gpu_gemm": (_I, [C.c_char, C.c_char, _I, _I, _I, _D, _P, _I, _P, _I, _D, _P, _I]),
    "fe_gpu_cluster_scores": (_I, [_P, _P, _P, _I, _I, _I, _I, _P]),
    "fe_gpu_cluster_meat": (_I, [_I, _I, _P, _I, _P]),
    "fe_gpu_fe_accumulate": (_I, [_P, _P, _P, _P, _SZ, _I, _I, _I, _SZ, _P, _P, _P, _P]),
    "fe_gpu_fe_compute_means": (_I, [_P, _P, _P, _P, _I, _I, _I]),
    "fe_gpu_fe_subtract": (_I, [_P, _P, _P, _P, _SZ, _I, _I, _SZ, _P, _P, _P, _D]),
    "fe_gpu_mix_means": (_I, [_P, _P, _SZ, _D]),
    "fe_gpu_axpy": (_I, [_I, _D, _P, _P]),
    "fe_gpu_absmax": (_I, [_P, _LL, _DP]),
    "fe_gpu_copy_columns": (_I, [_P, _I, _IP, _I, _I, _P, _I, _I]),
    "fe_gpu_build_multi_cluster_ids": (_I, [C.POINTER(C.c_void_p), C.POINTER(C.c_ulonglong), _I, _LL, _P, _IP]),
    "fe_build_cluster_ids": (_I, [_P, _I, _LL, _IP, _IP, _I, _P, _IP]),
    "fegb_config_init": (None, [C.POINTER(FegbConfig)]),
    "fegb_estimate_host": (_I, [C.POINTER(FegbConfig), _LL, _I, _I, _I, _P, _P, _P, _P, _IP, _DP, _DP,
                                C.POINTER(FegbResult)]),
    "fegb_estimate_device": (_I, [C.POINTER(FegbConfig), _LL, _I, _I, _I, _P, _P, _P, C.POINTER(C.c_void_p), _IP,
                                  _DP, _DP, C.POINTER(FegbResult)]),
    "fegb_within_transform": (_I, [C.POINTER(FegbConfig), _LL, _I, _I, _I, _P, _P, _P, C.POINTER(C.c_void_p), _IP,
                                   _IP, _IP, _DP]),
    "fegb_cluster_ids": (_I, [C.POINTER(C.c_void_p), _IP, _I, _LL, _P, _IP]),
    "fegb_compact_ids": (_I, [_P, _LL, _P, _IP]),
    "fegb_group_sizes": (_I, [C.POINTER(C.c_void_p), _I, _LL, _IP]),
    "fegb_drop_singletons": (_I, [C.POINTER(C.c_void_p), _IP, _I, _LL, _P, C.POINTER(C.c_longlong)]),
    "fegb_kernel_launches": (_LL, []),
    "fegb_set_tuning": (_I, [C.c_char_p, _I]),
    "fegb_get_tuning": (_I, [C.c_char_p, _IP]),
    "fegb_reset_tuning": (_I, []),
    "fegb_pool_usage": (_I, [_I, C.POINTER(C.c_ulonglong), C.POINTER(C.c_ulonglong), C.POINTER(C.c_ulonglong)]),
    "fegb_test_dense_pair": (_I, [_P, _LL, _I, _P, _P, _I, _I, _P, _P, _I, _I, _P, _P, _P]),
    "fegb_test_group_sums": (_I, [_P, _LL, _I, _P, _I, _I, _P]),
    "fegb_test_gram": (_I, [_P, _LL, _I, _I, _P]),
    "fegb_reconstruct_fe": (_I, [C.POINTER(FegbConfig), _LL, _I, _I, _P, _P, _DP, C.POINTER(C.c_void_p), _IP, _DP,
                                 C.POINTER(C.c_longlong), _IP, _DP]),
    "fegb_load_bin": (_I, [C.c_char_p, C.POINTER(FegbDataset)]),
    "fegb_free_dataset": (_I, [C.POINTER(FegbDataset)]),
    "fegb_estimate_batch": (_I, [C.POINTER(FegbConfig), _I, C.POINTER(FegbSpec), _DP, _DP, C.POINTER(FegbResult)]),
    "fegb_design_levels": (_I, [_P, _LL, _I, _IP, _IP, _P]),
    "fegb_build_design": (_I, [C.POINTER(C.c_void_p), _I, _LL, C.POINTER(FegbDesignColumn), _I, _P, _LL, _P]),
}


def library_path() -> Path:
    return _LIB_PATH


def lib():
    """Load libfegb.so (once). Raises FeGpuError when it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not _LIB_PATH.exists():
            raise FeGpuError(-1, f"{_LIB_PATH} not built; run python -m fe_gpu_gb300.build", "load")
        handle = C.CDLL(str(_LIB_PATH), mode=os.RTLD_NOW | getattr(os, "RTLD_GLOBAL", 0))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
        return _lib


def last_error() -> str:
    buf = C.create_string_buffer(512)
    lib().fe_gpu_runtime_get_last_error(buf, 512)
    return buf.value.decode(errors="replace")


def check(status: int, where: str = "") -> None:
    if status != 0:
        raise FeGpuError(status, last_error(), where)


def int_array(values) -> C.Array:
    vals = [int(v) for v in values]
    arr = (C.c_int * max(1, len(vals)))(*vals)
    return arr
