"""TEST INFRASTRUCTURE ONLY: ctypes wrapper over the CPU oracle
(oracle/fe_oracle.c, a C restatement of the reference estimation path) and,
where it was built, over the reference's own compiled cluster-id builder
(oracle/_ref/libref_cluster_ids.so, recipe oracle/build_ref.sh).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, and only as the checker. The product (fe_gpu_gb300) never does.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from dataclasses import dataclass
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libfe_oracle.so"
REF_LIB = HERE / "_ref" / "libref_cluster_ids.so"

_lib = None
_ref = None


class OrcConfig(C.Structure):
    _fields_ = [
        ("fe_tol", C.c_double),
        ("fe_max_iter", C.c_int),
        ("n_cluster_dims", C.c_int),
        ("cluster_dims", C.POINTER(C.c_int)),
        ("n_iv_regressors", C.c_int),
        ("iv_regressors", C.POINTER(C.c_int)),
        ("n_iv_instruments", C.c_int),
        ("iv_instruments", C.POINTER(C.c_int)),
        ("demean_scheme", C.c_int),
    ]


class OrcResult(C.Structure):
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
        ("max_update", C.c_double),
        ("rss", C.c_double),
        ("tss_total", C.c_double),
        ("tss_within", C.c_double),
        ("r2", C.c_double),
        ("r2_adj", C.c_double),
        ("r2_within", C.c_double),
        ("f_stat", C.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def build() -> Path:
    """Compile the oracle with gcc (idempotent)."""
    src = HERE / "fe_oracle.c"
    (HERE / "_build").mkdir(exist_ok=True)
    if not LIB.exists() or LIB.stat().st_mtime < max(src.stat().st_mtime, (HERE / "fe_oracle.h").stat().st_mtime):
        tmp = LIB.with_suffix(".so.tmp")
        subprocess.run(["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-o", str(tmp), str(src), "-lm"], check=True)
        tmp.replace(LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(str(LIB))
        P = C.c_void_p
        _lib.orc_cpu_estimate.argtypes = [C.POINTER(OrcConfig), C.c_longlong, C.c_int, C.c_int, P, P, P, P, P, P,
                                          C.POINTER(OrcResult)]
        _lib.orc_gpu_estimate.argtypes = [C.POINTER(OrcConfig), C.c_longlong, C.c_int, C.c_int, C.c_int, P, P, P, P,
                                          P, P, P, C.POINTER(OrcResult)]
        _lib.orc_cluster_ids.argtypes = [P, C.c_int, C.c_longlong, P, P, C.c_int, P, C.POINTER(C.c_int)]
        _lib.orc_group_sizes.argtypes = [P, C.c_int, C.c_longlong, P]
        _lib.orc_compact_ids.argtypes = [P, C.c_longlong, P, C.POINTER(C.c_int)]
        _lib.orc_drop_singletons.argtypes = [P, C.c_int, C.c_longlong, P, P]
        _lib.orc_drop_singletons.restype = C.c_longlong
        _lib.orc_demean_forward.argtypes = [P, P, C.c_int, C.c_longlong, C.c_int, P, P, C.c_double, C.c_int,
                                            C.POINTER(C.c_int), C.POINTER(C.c_double)]
        _lib.orc_demean_symmetric.argtypes = [P, P, C.c_int, P, C.c_int, C.c_longlong, C.c_int, P, P, C.c_double,
                                              C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double)]
        _lib.orc_chol_solve_invert.argtypes = [C.c_int, P, P, P, P]
        _lib.orc_reconstruct_fe.argtypes = [C.c_longlong, C.c_int, C.c_int, P, P, P, P, P, C.c_double, C.c_int, P, P,
                                            C.POINTER(C.c_int), C.POINTER(C.c_double)]
        _lib.orc_psd_fix.argtypes = [C.c_int, P]
    return _lib


def ref_lib():
    """The reference's compiled cluster-id builder, or None where the
    reference tree was not available to build it."""
    global _ref
    if _ref is None and REF_LIB.exists():
        _ref = C.CDLL(str(REF_LIB))
        P = C.c_void_p
        _ref.fe_build_cluster_ids.argtypes = [P, C.c_int, C.c_longlong, P, P, C.c_int, P, C.POINTER(C.c_int)]
    return _ref


def _iarr(v):
    v = list(v)
    return (C.c_int * max(1, len(v)))(*v), len(v)


@dataclass
class OracleFit:
    beta: np.ndarray
    se: np.ndarray
    stats: dict


def _config(tol, max_iter, cluster_dims, iv_regressors, iv_instruments, scheme):
    cd, ncd = _iarr(cluster_dims)
    ivr, nivr = _iarr(iv_regressors)
    ivi, nivi = _iarr(iv_instruments)
    cfg = OrcConfig(tol, max_iter, ncd, C.cast(cd, C.POINTER(C.c_int)), nivr, C.cast(ivr, C.POINTER(C.c_int)),
                    nivi, C.cast(ivi, C.POINTER(C.c_int)), scheme)
    return cfg, (cd, ivr, ivi)


def _prep(y, W, Z, fe_ids):
    y = np.ascontiguousarray(y, dtype=np.float64)
    n = y.shape[0]
    W = np.asfortranarray(W, dtype=np.float64) if W is not None else np.zeros((n, 0), order="F")
    Z = np.asfortranarray(Z, dtype=np.float64) if Z is not None else np.zeros((n, 0), order="F")
    fe = np.asfortranarray(fe_ids, dtype=np.int32)
    return y, W, Z, fe


def group_sizes(fe_ids) -> np.ndarray:
    fe = np.asfortranarray(fe_ids, dtype=np.int32)
    out = np.zeros(fe.shape[0], dtype=np.int32)
    st = lib().orc_group_sizes(fe.ctypes.data, fe.shape[0], fe.shape[1], out.ctypes.data)
    if st != 0:
        raise ValueError("FE indices must be positive")
    return out


def cpu_estimate(y, W, fe_ids, tol=1e-8, max_iter=100000, cluster_dims=(), sizes=None) -> OracleFit:
    """fe_cpu_estimate (src/core/fe_pipeline.f90:71-513)."""
    y, W, _, fe = _prep(y, W, None, fe_ids)
    sizes = np.asarray(group_sizes(fe) if sizes is None else sizes, dtype=np.int32)
    cfg, keep = _config(tol, max_iter, cluster_dims, (), (), 0)
    k = W.shape[1]
    beta = np.zeros(max(k, 1))
    se = np.zeros(max(k, 1))
    res = OrcResult()
    lib().orc_cpu_estimate(C.byref(cfg), y.shape[0], k, fe.shape[0], y.ctypes.data, W.ctypes.data, fe.ctypes.data,
                           sizes.ctypes.data, beta.ctypes.data, se.ctypes.data, C.byref(res))
    del keep
    return OracleFit(beta[:k].copy(), se[:k].copy(), res.as_dict())


def gpu_estimate(y, W, fe_ids, Z=None, tol=1e-8, max_iter=100000, cluster_dims=(), iv_regressors=(),
                 iv_instruments=(), sizes=None) -> OracleFit:
    """GPU-path conventions of fe_gpu_estimate (src/core/fe_pipeline.f90:516-1896) on the CPU."""
    y, W, Z, fe = _prep(y, W, Z, fe_ids)
    sizes = np.asarray(group_sizes(fe) if sizes is None else sizes, dtype=np.int32)
    cfg, keep = _config(tol, max_iter, cluster_dims, iv_regressors, iv_instruments, 1)
    k, l = W.shape[1], Z.shape[1]
    beta = np.zeros(max(k, 1))
    se = np.zeros(max(k, 1))
    res = OrcResult()
    lib().orc_gpu_estimate(C.byref(cfg), y.shape[0], k, l, fe.shape[0], y.ctypes.data, W.ctypes.data,
                           Z.ctypes.data, fe.ctypes.data, sizes.ctypes.data, beta.ctypes.data, se.ctypes.data,
                           C.byref(res))
    del keep
    return OracleFit(beta[:k].copy(), se[:k].copy(), res.as_dict())


def demean_forward(y, W, fe_ids, tol, max_iter, sizes=None):
    y, W, _, fe = _prep(y, W, None, fe_ids)
    y, W = y.copy(), W.copy(order="F")
    sizes = np.asarray(group_sizes(fe) if sizes is None else sizes, dtype=np.int32)
    conv = C.c_int(0)
    mu = C.c_double(0)
    it = lib().orc_demean_forward(y.ctypes.data, W.ctypes.data, W.shape[1], y.shape[0], fe.shape[0], fe.ctypes.data,
                                  sizes.ctypes.data, tol, max_iter, C.byref(conv), C.byref(mu))
    return y, W, it, bool(conv.value), mu.value


def demean_symmetric(y, W, fe_ids, tol, max_iter, Z=None, sizes=None):
    y, W, Z, fe = _prep(y, W, Z, fe_ids)
    y, W, Z = y.copy(), W.copy(order="F"), Z.copy(order="F")
    sizes = np.asarray(group_sizes(fe) if sizes is None else sizes, dtype=np.int32)
    conv = C.c_int(0)
    mu = C.c_double(0)
    it = lib().orc_demean_symmetric(y.ctypes.data, W.ctypes.data, W.shape[1], Z.ctypes.data, Z.shape[1], y.shape[0],
                                    fe.shape[0], fe.ctypes.data, sizes.ctypes.data, tol, max_iter, C.byref(conv),
                                    C.byref(mu))
    return y, W, Z, it, bool(conv.value), mu.value


def cluster_ids(fe_ids, sizes, subset_dims, use_reference: bool = False):
    """Intersection ids (1-based) for the 1-based subset_dims; restated
    builder by default, the reference's compiled builder with use_reference."""
    fe = np.asfortranarray(fe_ids, dtype=np.int32)
    n_fe, n = fe.shape
    dims = np.array(subset_dims, dtype=np.int32)
    ss = np.array([sizes[d - 1] for d in subset_dims], dtype=np.int32)
    out = np.zeros(n, dtype=np.int32)
    nc = C.c_int(0)
    L = ref_lib() if use_reference else lib()
    if L is None:
        raise RuntimeError("reference cluster builder not built")
    fn = L.fe_build_cluster_ids if use_reference else L.orc_cluster_ids
    st = fn(fe.ctypes.data, n_fe, n, dims.ctypes.data, ss.ctypes.data, len(dims), out.ctypes.data, C.byref(nc))
    return out, nc.value, st


def compact_ids(raw):
    raw = np.ascontiguousarray(raw, dtype=np.int32)
    out = np.zeros_like(raw)
    lv = C.c_int(0)
    lib().orc_compact_ids(raw.ctypes.data, raw.size, out.ctypes.data, C.byref(lv))
    return out, lv.value


def drop_singletons(fe_ids, sizes=None):
    fe = np.asfortranarray(fe_ids, dtype=np.int32)
    sizes = np.asarray(group_sizes(fe) if sizes is None else sizes, dtype=np.int32)
    keep = np.zeros(fe.shape[1], dtype=np.uint8)
    dropped = lib().orc_drop_singletons(fe.ctypes.data, fe.shape[0], fe.shape[1], sizes.ctypes.data, keep.ctypes.data)
    return keep.astype(bool), int(dropped)


def chol_solve_invert(Q, b):
    n = Q.shape[0]
    Qc = np.asfortranarray(Q, dtype=np.float64).copy(order="F")
    b = np.ascontiguousarray(b, dtype=np.float64)
    beta = np.zeros(n)
    Qi = np.zeros((n, n), order="F")
    info = lib().orc_chol_solve_invert(n, Qc.ctypes.data, b.ctypes.data, beta.ctypes.data, Qi.ctypes.data)
    return beta, Qi, info


def psd_fix(A):
    A = np.asfortranarray(A, dtype=np.float64).copy(order="F")
    applied = lib().orc_psd_fix(A.shape[0], A.ctypes.data)
    return A, bool(applied)


def reconstruct_fe(y, W, fe_ids, beta, tol=1e-8, max_iter=100000, sizes=None):
    """FE values of --save-fe, restated loop for loop
    (src/core/fe_pipeline.f90:1619-1733). Returns ([values per dimension],
    [counts per dimension], iterations, max_update)."""
    y, W, _, fe = _prep(y, W, None, fe_ids)
    n_fe, n = fe.shape
    k = W.shape[1]
    sizes = np.asarray(group_sizes(fe) if sizes is None else sizes, dtype=np.int32)
    b = np.ascontiguousarray(np.asarray(beta, dtype=np.float64)[:k])
    total = int(sizes.sum())
    vals = np.zeros(max(1, total))
    cnts = np.zeros(max(1, total), dtype=np.int64)
    it = C.c_int(0)
    mu = C.c_double(0)
    st = lib().orc_reconstruct_fe(C.c_longlong(n), k, n_fe, y.ctypes.data, W.ctypes.data, b.ctypes.data,
                                  fe.ctypes.data, sizes.ctypes.data, C.c_double(tol), max_iter, vals.ctypes.data,
                                  cnts.ctypes.data, C.byref(it), C.byref(mu))
    if st != 0:
        raise RuntimeError("orc_reconstruct_fe failed")
    out_v, out_c, off = [], [], 0
    for g in sizes:
        out_v.append(vals[off:off + g].copy())
        out_c.append(cnts[off:off + g].copy())
        off += g
    return out_v, out_c, it.value, mu.value
