"""Host-side estimator interface, mirroring the reference's estimation driver
(src/core/fe_pipeline.f90) and its configuration/types
(src/core/fe_config.f90:16-46, src/core/fe_types.f90, fe_pipeline.f90:37-64).

All numerical work happens in libfegb.so through its C ABI; this module only
marshals arguments. Device memory, when needed, comes from the library's own
fe_gpu_runtime_malloc (no torch dependency).
"""
from __future__ import annotations

import copy
import ctypes as C
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

from . import _native as N
from .bin_io import fe_dataset_header, fe_host_arrays

PRECISIONS = {"fp64": 0, "mixed": 1}
SE_CONVENTIONS = {"gpu": 0, "cpu": 1}


@dataclass
class fe_runtime_config:  # src/core/fe_config.f90:16-46 (host-facing subset)
    data_path: str = "data.bin"
    fe_tolerance: float = 1.0e-6
    fe_max_iterations: int = 500
    use_gpu: bool = True
    force_cpu: bool = False
    verbose: bool = False
    cpu_threads: int = 0
    fast_mode: bool = False
    demean_cg: bool = False
    cluster_fe_dims: list = field(default_factory=list)
    iv_regressors: list = field(default_factory=list)
    iv_instrument_cols: list = field(default_factory=list)
    # additions of this library
    precision: str = "fp64"          # "fp64" (plain) or "mixed" (FP32 sweeps + FP64 refinement)
    se_convention: str = "gpu"       # "gpu" (reference GPU estimator) or "cpu" (reference CPU estimator)
    drop_singletons: bool = False
    # mixed precision: also fit the plain FP64 form (FP64 storage, the
    # reference's AP scheme) on the same inputs and attach every coefficient's
    # and SE's relative error against it to the result
    verify_fp64: bool = False


def init_default_config() -> fe_runtime_config:  # src/core/fe_config.f90:53-79
    return fe_runtime_config()


@dataclass
class fe_estimation_result:  # src/core/fe_pipeline.f90:37-64
    converged: bool = False
    fe_iterations: int = 0
    solver_info: int = 0
    rank: int = 0
    cluster_fe_dims: list = field(default_factory=list)
    time_demean: float = 0.0
    time_regression: float = 0.0
    time_se: float = 0.0
    rss: float = 0.0
    tss_total: float = 0.0
    tss_within: float = 0.0
    r2: float = 0.0
    r2_adj: float = 0.0
    r2_within: float = 0.0
    f_stat: float = 0.0
    dof_model: int = 0
    dof_fes: int = 0
    dof_resid: int = 0
    is_iv: bool = False
    n_instruments: int = 0
    beta: np.ndarray = field(default_factory=lambda: np.zeros(0))
    se: np.ndarray = field(default_factory=lambda: np.zeros(0))
    coef_names: list = field(default_factory=list)
    depvar_name: str = ""
    psd_fix_applied: bool = False
    max_update: float = 0.0
    n_obs_used: int = 0
    n_singletons: int = 0
    stats: dict = field(default_factory=dict)
    # with verify_fp64: |x - x_fp64| / |x_fp64| per coefficient and SE (0 where
    # both are 0, e.g. a column the filter dropped), and the FP64 fit's values
    beta_rel_err_vs_fp64: Optional[np.ndarray] = None
    se_rel_err_vs_fp64: Optional[np.ndarray] = None
    beta_fp64: Optional[np.ndarray] = None
    se_fp64: Optional[np.ndarray] = None


def _make_config(cfg: fe_runtime_config, stream: Optional[int] = None, profile: bool = False):
    c = N.FegbConfig()
    N.lib().fegb_config_init(C.byref(c))
    c.fe_tol = float(cfg.fe_tolerance)
    c.fe_max_iter = int(cfg.fe_max_iterations)
    if cfg.precision not in PRECISIONS:
        raise ValueError(f"precision must be one of {list(PRECISIONS)}")
    c.precision = PRECISIONS[cfg.precision]
    c.demean_method = 1 if cfg.demean_cg else 0
    if cfg.se_convention not in SE_CONVENTIONS:
        raise ValueError(f"se_convention must be one of {list(SE_CONVENTIONS)}")
    c.se_convention = SE_CONVENTIONS[cfg.se_convention]
    c.drop_singletons = 1 if cfg.drop_singletons else 0
    keep = []
    for name, field_n, field_p in (("cluster_fe_dims", "n_cluster_dims", "cluster_dims"),
                                   ("iv_regressors", "n_iv_regressors", "iv_regressors"),
                                   ("iv_instrument_cols", "n_iv_instruments", "iv_instruments")):
        vals = list(getattr(cfg, name))
        arr = N.int_array(vals)
        keep.append(arr)
        setattr(c, field_n, len(vals))
        setattr(c, field_p, C.cast(arr, C.POINTER(C.c_int)))
    c.verbose = 1 if cfg.verbose else 0
    c.stream = C.c_void_p(stream) if stream else None
    c.profile = 1 if profile else 0
    return c, keep


def _coef_names(header: Optional[fe_dataset_header], k: int) -> list:
    names = list(header.regressor_names) if header is not None else []
    if len(names) == k:
        return names
    return [f"beta_{i + 1}" for i in range(k)]


def _result_from(res: N.FegbResult, beta, se, cfg: fe_runtime_config, header) -> fe_estimation_result:
    r = fe_estimation_result()
    d = res.as_dict()
    r.converged = bool(d["converged"])
    r.fe_iterations = d["fe_iterations"]
    r.solver_info = d["solver_info"]
    r.rank = d["rank"]
    r.time_demean = d["time_demean"]
    r.time_regression = d["time_regression"]
    r.time_se = d["time_se"]
    for key in ("rss", "tss_total", "tss_within", "r2", "r2_adj", "r2_within", "f_stat", "dof_model", "dof_fes",
                "dof_resid", "n_instruments", "max_update", "n_obs_used"):
        setattr(r, key, d[key])
    r.n_singletons = d["n_singletons"]
    r.is_iv = bool(d["is_iv"])
    r.psd_fix_applied = bool(d["psd_fix_applied"])
    r.beta = beta
    r.se = se
    r.cluster_fe_dims = list(cfg.cluster_fe_dims)[:3] if d["n_cluster_dims_used"] else []
    r.coef_names = _coef_names(header, len(beta))
    r.depvar_name = header.depvar_name if header is not None else ""
    r.stats = d
    return r


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data if a is not None and a.size else None


def _rel_err(x: np.ndarray, ref: np.ndarray) -> np.ndarray:
    x, ref = np.asarray(x, dtype=np.float64), np.asarray(ref, dtype=np.float64)
    d = np.abs(x - ref)
    return np.where(d == 0.0, 0.0, d / np.maximum(np.abs(ref), np.finfo(np.float64).tiny))


def _attach_fp64_errors(res: fe_estimation_result, cfg: fe_runtime_config, refit) -> fe_estimation_result:
    """verify_fp64: refit in the plain FP64 form (AP) and attach the errors."""
    if not cfg.verify_fp64 or cfg.precision == "fp64":
        return res
    c64 = copy.copy(cfg)
    c64.precision = "fp64"
    c64.demean_cg = False
    c64.verify_fp64 = False
    ref = refit(c64)
    res.beta_fp64, res.se_fp64 = ref.beta, ref.se
    res.beta_rel_err_vs_fp64 = _rel_err(res.beta, ref.beta)
    res.se_rel_err_vs_fp64 = _rel_err(res.se, ref.se)
    return res


def _tune(rows: int, columns: int, tune: bool) -> None:
    if tune:
        from . import autotune

        autotune.apply_for_shape(int(rows), int(columns))


def fe_gpu_estimate(cfg: fe_runtime_config, header: Optional[fe_dataset_header], host: fe_host_arrays,
                    group_sizes: Optional[Sequence[int]] = None, stream: Optional[int] = None,
                    profile: bool = False, tune: bool = True) -> fe_estimation_result:
    """fe_gpu_estimate (src/core/fe_pipeline.f90:516) over host arrays: the
    upload, within-transform, normal equations and SEs all run in libfegb.so."""
    y = np.ascontiguousarray(host.y, dtype=np.float64)
    n = y.shape[0]
    W = np.asfortranarray(host.W, dtype=np.float64) if host.W is not None else np.zeros((n, 0), order="F")
    Z = np.asfortranarray(host.Z, dtype=np.float64) if host.Z is not None else np.zeros((n, 0), order="F")
    fe = np.asfortranarray(host.fe_ids, dtype=np.int32) if host.fe_ids is not None else np.zeros((0, n), np.int32,
                                                                                                   order="F")
    if fe.ndim != 2 or fe.shape[1] != n:
        raise ValueError("fe_ids must have shape (n_fe, n)")
    k, l, n_fe = W.shape[1], Z.shape[1], fe.shape[0]
    _tune(n, 1 + k + l, tune)
    c, keep = _make_config(cfg, stream, profile)
    beta = np.zeros(max(k, 1))
    se = np.zeros(max(k, 1))
    res = N.FegbResult()
    gs = N.int_array(group_sizes) if group_sizes is not None else None
    st = N.lib().fegb_estimate_host(C.byref(c), n, k, l, n_fe, _ptr(y), _ptr(W), _ptr(Z), _ptr(fe),
                                    C.cast(gs, C.POINTER(C.c_int)) if gs is not None else None,
                                    beta.ctypes.data_as(C.POINTER(C.c_double)),
                                    se.ctypes.data_as(C.POINTER(C.c_double)), C.byref(res))
    N.check(st, "fegb_estimate_host")
    del keep
    out = _result_from(res, beta[:k].copy(), se[:k].copy(), cfg, header)
    return _attach_fp64_errors(out, cfg, lambda c64: fe_gpu_estimate(c64, header, host, group_sizes, stream,
                                                                     tune=tune))


def fe_gpu_estimate_device(cfg: fe_runtime_config, n: int, k: int, l: int, d_y: int, d_W: Optional[int],
                           d_Z: Optional[int], d_fe_ids: Sequence[int], group_sizes: Optional[Sequence[int]] = None,
                           stream: Optional[int] = None, header: Optional[fe_dataset_header] = None,
                           profile: bool = False, tune: bool = True) -> fe_estimation_result:
    """Same fit over device arrays (raw device pointers), e.g. from the
    fe_gpu_dataset upload (src/gpu/fe_gpu_data.f90:41-120). tune: apply the
    autotuner's knobs for this shape first."""
    _tune(n, 1 + k + l, tune)
    c, keep = _make_config(cfg, stream, profile)
    n_fe = len(d_fe_ids)
    ptrs = (C.c_void_p * max(1, n_fe))(*[C.c_void_p(int(p)) for p in d_fe_ids])
    beta = np.zeros(max(k, 1))
    se = np.zeros(max(k, 1))
    res = N.FegbResult()
    gs = N.int_array(group_sizes) if group_sizes is not None else None
    st = N.lib().fegb_estimate_device(C.byref(c), n, k, l, n_fe, C.c_void_p(d_y), C.c_void_p(d_W or 0) if d_W else None,
                                      C.c_void_p(d_Z) if d_Z else None, ptrs,
                                      C.cast(gs, C.POINTER(C.c_int)) if gs is not None else None,
                                      beta.ctypes.data_as(C.POINTER(C.c_double)),
                                      se.ctypes.data_as(C.POINTER(C.c_double)), C.byref(res))
    N.check(st, "fegb_estimate_device")
    del keep
    out = _result_from(res, beta[:k].copy(), se[:k].copy(), cfg, header)
    return _attach_fp64_errors(out, cfg, lambda c64: fe_gpu_estimate_device(c64, n, k, l, d_y, d_W, d_Z, d_fe_ids,
                                                                            group_sizes, stream, header,
                                                                            tune=tune))


@dataclass
class fe_batch_spec:
    """One specification of a batch: device pointers in the fegb_estimate_device
    layout plus its own cluster dimensions and IV columns."""
    n: int
    k: int
    l: int
    d_y: int
    d_W: Optional[int]
    d_Z: Optional[int]
    d_fe_ids: Sequence[int]
    cluster_fe_dims: Sequence[int] = ()
    iv_regressors: Sequence[int] = ()
    iv_instrument_cols: Sequence[int] = ()


def fe_gpu_estimate_batch(cfg: fe_runtime_config, specs: Sequence[fe_batch_spec], stream: Optional[int] = None,
                          profile: bool = False) -> list:
    """fegb_estimate_batch: many independent fits sharing one within-transform
    per column-count class. cfg supplies tolerance, precision, method and SE
    convention; every spec its own clusters and IV columns."""
    c, keep = _make_config(cfg, stream, profile)
    m = len(specs)
    arr = (N.FegbSpec * max(1, m))()
    for i, sp in enumerate(specs):
        ids = (C.c_void_p * max(1, len(sp.d_fe_ids)))(*[C.c_void_p(int(p)) for p in sp.d_fe_ids])
        keep.append(ids)
        a = arr[i]
        a.n, a.k, a.l, a.n_fe = int(sp.n), int(sp.k), int(sp.l), len(sp.d_fe_ids)
        a.y = C.c_void_p(int(sp.d_y))
        a.W = C.c_void_p(int(sp.d_W)) if sp.d_W else None
        a.Z = C.c_void_p(int(sp.d_Z)) if sp.d_Z else None
        a.fe_ids = C.cast(ids, C.POINTER(C.c_void_p))
        for name, fn, fp in (("cluster_fe_dims", "n_cluster_dims", "cluster_dims"),
                             ("iv_regressors", "n_iv_regressors", "iv_regressors"),
                             ("iv_instrument_cols", "n_iv_instruments", "iv_instruments")):
            vals = N.int_array(list(getattr(sp, name)))
            keep.append(vals)
            setattr(a, fn, len(getattr(sp, name)))
            setattr(a, fp, C.cast(vals, C.POINTER(C.c_int)))
    ktot = sum(int(sp.k) for sp in specs)
    beta = np.zeros(max(ktot, 1))
    se = np.zeros(max(ktot, 1))
    res = (N.FegbResult * max(1, m))()
    st = N.lib().fegb_estimate_batch(C.byref(c), m, arr, beta.ctypes.data_as(C.POINTER(C.c_double)),
                                     se.ctypes.data_as(C.POINTER(C.c_double)), res)
    N.check(st, "fegb_estimate_batch")
    del keep
    out, off = [], 0
    for i, sp in enumerate(specs):
        cfg_i = copy.copy(cfg)
        cfg_i.cluster_fe_dims = list(sp.cluster_fe_dims)
        out.append(_result_from(res[i], beta[off:off + sp.k].copy(), se[off:off + sp.k].copy(), cfg_i, None))
        off += sp.k
    return out


def fe_gpu_within_transform_device(cfg: fe_runtime_config, n: int, k: int, l: int, d_y: int, d_W: Optional[int],
                                   d_Z: Optional[int], d_fe_ids: Sequence[int],
                                   group_sizes: Optional[Sequence[int]] = None) -> tuple:
    """fe_gpu_within_transform (src/gpu/fe_gpu_demean.f90:63) on device
    columns in place. Returns (converged, iterations, max_update)."""
    c, keep = _make_config(cfg)
    n_fe = len(d_fe_ids)
    ptrs = (C.c_void_p * max(1, n_fe))(*[C.c_void_p(int(p)) for p in d_fe_ids])
    conv = C.c_int(0)
    it = C.c_int(0)
    mu = C.c_double(0.0)
    gs = N.int_array(group_sizes) if group_sizes is not None else None
    st = N.lib().fegb_within_transform(C.byref(c), n, k, l, n_fe, C.c_void_p(d_y), C.c_void_p(d_W) if d_W else None,
                                       C.c_void_p(d_Z) if d_Z else None, ptrs,
                                       C.cast(gs, C.POINTER(C.c_int)) if gs is not None else None, C.byref(conv),
                                       C.byref(it), C.byref(mu))
    N.check(st, "fegb_within_transform")
    del keep
    return bool(conv.value), it.value, mu.value


class DeviceBuffer:
    """fe_device_buffer (src/gpu/fe_gpu_runtime.f90:36-39) over the library's
    own allocator."""

    def __init__(self, nbytes: int):
        self.size_bytes = int(nbytes)
        p = C.c_void_p()
        N.check(N.lib().fe_gpu_runtime_malloc(C.byref(p), self.size_bytes), "fe_gpu_runtime_malloc")
        self.ptr = p.value or 0

    @classmethod
    def from_array(cls, a: np.ndarray) -> "DeviceBuffer":
        a = np.ascontiguousarray(a) if not a.flags.f_contiguous else a
        b = cls(a.nbytes)
        if a.nbytes:
            N.check(N.lib().fe_gpu_runtime_memcpy_htod(b.ptr, a.ctypes.data, a.nbytes), "memcpy_htod")
        return b

    def to_array(self, dtype, shape, order="C") -> np.ndarray:
        out = np.empty(shape, dtype=dtype, order=order)
        if out.nbytes:
            N.check(N.lib().fe_gpu_runtime_memcpy_dtoh(out.ctypes.data, self.ptr, out.nbytes), "memcpy_dtoh")
        return out

    def free(self) -> None:
        if self.ptr:
            N.check(N.lib().fe_gpu_runtime_free(self.ptr), "fe_gpu_runtime_free")
            self.ptr = 0

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def fe_gpu_within_transform(cfg: fe_runtime_config, host: fe_host_arrays,
                            group_sizes: Optional[Sequence[int]] = None) -> tuple:
    """Upload, demean on the device, download (the test_gpu_demean.f90 flow).
    Returns (converged, iterations, max_update) and updates host.y/W/Z."""
    y = np.ascontiguousarray(host.y, dtype=np.float64)
    n = y.shape[0]
    W = np.asfortranarray(host.W, dtype=np.float64)
    Z = np.asfortranarray(host.Z, dtype=np.float64) if host.Z is not None else np.zeros((n, 0), order="F")
    fe = np.asarray(host.fe_ids, dtype=np.int32)
    k, l = W.shape[1], Z.shape[1]
    by, bW, bZ = DeviceBuffer.from_array(y), DeviceBuffer.from_array(W), DeviceBuffer.from_array(Z)
    bids = [DeviceBuffer.from_array(np.ascontiguousarray(fe[d])) for d in range(fe.shape[0])]
    out = fe_gpu_within_transform_device(cfg, n, k, l, by.ptr, bW.ptr if k else None, bZ.ptr if l else None,
                                         [b.ptr for b in bids], group_sizes)
    host.y = by.to_array(np.float64, (n,))
    host.W = bW.to_array(np.float64, (n, k), order="F") if k else W
    if l:
        host.Z = bZ.to_array(np.float64, (n, l), order="F")
    return out


def compute_fe_group_sizes(fe_ids: np.ndarray) -> np.ndarray:
    """compute_fe_group_sizes (src/core/fe_grouping.f90:11-37) on the device:
    G_d = max id; raises FeGpuError if any id < 1."""
    fe = np.asarray(fe_ids, dtype=np.int32)
    n_fe, n = fe.shape
    bufs = [DeviceBuffer.from_array(np.ascontiguousarray(fe[d])) for d in range(n_fe)]
    ptrs = (C.c_void_p * max(1, n_fe))(*[C.c_void_p(b.ptr) for b in bufs])
    sizes = (C.c_int * max(1, n_fe))()
    N.check(N.lib().fegb_group_sizes(ptrs, n_fe, n, sizes), "fegb_group_sizes")
    return np.array(sizes[:n_fe], dtype=np.int64)


def build_cluster_ids(fe_ids: np.ndarray, group_sizes: Sequence[int], subset_dims: Sequence[int]):
    """build_cluster_ids (src/core/fe_cluster_utils.f90:27-72) through
    fe_build_cluster_ids; returns (ids, n_clusters, status)."""
    fe = np.asfortranarray(fe_ids, dtype=np.int32)
    n_fe, n = fe.shape
    if len(subset_dims) <= 0:
        return np.zeros(n, np.int32), 0, -1
    dims = np.array(subset_dims, dtype=np.int32)
    sizes = np.array([group_sizes[d - 1] for d in subset_dims], dtype=np.int32)
    out = np.zeros(n, dtype=np.int32)
    nc = C.c_int(0)
    st = N.lib().fe_build_cluster_ids(fe.ctypes.data, n_fe, n, dims.ctypes.data_as(C.POINTER(C.c_int)),
                                      sizes.ctypes.data_as(C.POINTER(C.c_int)), len(dims), out.ctypes.data,
                                      C.byref(nc))
    return out, (nc.value if st == 0 else 0), st


def fe_gpu_reconstruct_fe(cfg: fe_runtime_config, host: fe_host_arrays, beta: np.ndarray,
                          group_sizes: Optional[Sequence[int]] = None) -> tuple:
    """FE values of --save-fe (reconstruct_and_save_fixed_effects,
    src/core/fe_pipeline.f90:1619-1733) on the device, from host arrays and the
    fitted beta. Returns ([values per dimension], [counts per dimension],
    iterations, max_update); values[d][g - 1] belongs to level g."""
    y = np.ascontiguousarray(host.y, dtype=np.float64)
    n = y.shape[0]
    W = np.asfortranarray(host.W, dtype=np.float64) if host.W is not None else np.zeros((n, 0), order="F")
    fe = np.asarray(host.fe_ids, dtype=np.int32)
    k, n_fe = W.shape[1], fe.shape[0]
    gs = [int(v) for v in (group_sizes if group_sizes is not None else fe.max(axis=1))]
    by, bW = DeviceBuffer.from_array(y), DeviceBuffer.from_array(W)
    bids = [DeviceBuffer.from_array(np.ascontiguousarray(fe[d])) for d in range(n_fe)]
    ptrs = (C.c_void_p * max(1, n_fe))(*[C.c_void_p(b.ptr) for b in bids])
    b = np.ascontiguousarray(beta[:k], dtype=np.float64)
    total = sum(gs)
    vals = np.zeros(max(1, total))
    cnts = np.zeros(max(1, total), dtype=np.int64)
    it = C.c_int(0)
    mu = C.c_double(0)
    c, keep = _make_config(cfg)
    gsa = N.int_array(gs)
    st = N.lib().fegb_reconstruct_fe(C.byref(c), n, k, n_fe, C.c_void_p(by.ptr), C.c_void_p(bW.ptr) if k else None,
                                     b.ctypes.data_as(C.POINTER(C.c_double)), ptrs, C.cast(gsa, C.POINTER(C.c_int)),
                                     vals.ctypes.data_as(C.POINTER(C.c_double)),
                                     cnts.ctypes.data_as(C.POINTER(C.c_longlong)), C.byref(it), C.byref(mu))
    N.check(st, "fegb_reconstruct_fe")
    del keep
    out_v, out_c, off = [], [], 0
    for g in gs:
        out_v.append(vals[off:off + g].copy())
        out_c.append(cnts[off:off + g].copy())
        off += g
    return out_v, out_c, it.value, mu.value


def format_es24_16(v: float) -> str:
    """Fortran ES24.16: one digit before the point, 16 after, exponent
    'E+dd' when it fits two digits and '+ddd' (no letter) otherwise,
    right-aligned in 24 characters."""
    m, e = f"{v:.16E}".split("E")
    ex = int(e)
    tail = f"E{ex:+03d}" if abs(ex) <= 99 else f"{ex:+04d}"
    return f"{m}{tail}".rjust(24)


def write_fe_outputs(prefix: str, values: Sequence[np.ndarray], counts: Sequence[np.ndarray]) -> list:
    """write_fe_outputs (src/core/fe_pipeline.f90:1735-1771): one
    <prefix>_fe<d>.csv per dimension, header 'level_id,fe_value', one line
    'g,value' (I0, ES24.16) per level with a nonzero count."""
    paths = []
    for d, (v, c) in enumerate(zip(values, counts), start=1):
        path = f"{prefix}_fe{d}.csv"
        with open(path, "w") as f:
            f.write("level_id,fe_value\n")
            for g in range(len(v)):
                if c[g] > 0:
                    f.write(f"{g + 1},{format_es24_16(float(v[g]))}\n")
        paths.append(path)
    return paths
