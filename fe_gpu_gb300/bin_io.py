"""The fe_gpu ``.bin`` dataset format: reader and writer.

Reader restates load_dataset_from_file (src/io/fe_data_io.f90:23-66,
78-202, 243-299, 360-389): a new (28-byte) or old (24-byte) header detected
from the file size, FP32 or FP64 values (always returned as FP64), an
optional trailing precision flag and an optional ``META`` v1 names block.
Writer restates write_binary (tools/generate_synthetic_data.py:180-210).
"""
from __future__ import annotations

import os
import struct
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

PRECISION_FLOAT64 = 0
PRECISION_FLOAT32 = 1

HEADER_BASE_BYTES_NEW = 8 + 5 * 4
HEADER_BASE_BYTES_OLD = 8 + 4 * 4


class FeDataError(ValueError):
    pass


@dataclass
class fe_dataset_header:  # src/core/fe_types.f90:9-26
    n_obs: int = 0
    n_regressors: int = 0
    n_instruments: int = 0
    n_fe: int = 0
    has_cluster: bool = False
    has_weights: bool = False
    precision_flag: int = PRECISION_FLOAT64
    metadata_bytes: int = 0
    depvar_name: str = ""
    regressor_names: list = field(default_factory=list)
    instrument_names: list = field(default_factory=list)
    fe_names: list = field(default_factory=list)
    cluster_name: str = ""
    weight_name: str = ""

    def summary(self) -> str:
        return (f"N={self.n_obs}, K={self.n_regressors}, L={self.n_instruments}, FE dims={self.n_fe}, "
                f"clusters={'T' if self.has_cluster else 'F'}, weights={'T' if self.has_weights else 'F'}, "
                f"precision_flag={self.precision_flag}")


@dataclass
class fe_host_arrays:  # src/core/fe_types.f90:28-36
    y: np.ndarray
    W: np.ndarray            # (n, k), column-major
    Z: np.ndarray            # (n, l), column-major
    fe_ids: np.ndarray       # (n_fe, n), dimension index fastest in memory
    cluster: Optional[np.ndarray] = None
    weights: Optional[np.ndarray] = None


def _data_bytes(n, k, l, n_fe, has_cluster, has_weights, vb) -> int:
    # compute_data_bytes, src/io/fe_data_io.f90:331-349
    total = n * (1 + k) * vb
    if l > 0:
        total += n * l * vb
    if has_weights:
        total += n * vb
    total += n_fe * n * 4
    if has_cluster:
        total += n * 4
    return total


def read_header(buf: bytes, file_size: int) -> tuple[fe_dataset_header, int]:
    """Header parsing of src/io/fe_data_io.f90:78-202; returns the header and
    the byte offset where the data starts."""
    if file_size < HEADER_BASE_BYTES_OLD:
        raise FeDataError("File too small to contain required header")
    n_obs, k = struct.unpack_from("<qi", buf, 0)
    if n_obs <= 0:
        raise FeDataError("N must be positive")
    if k < 0:
        raise FeDataError("K must be non-negative")
    t = struct.unpack_from("<4i", buf, 12)
    new = dict(n_instruments=t[0], n_fe=t[1], has_cluster=t[2] != 0, has_weights=t[3] != 0)
    old = dict(n_instruments=0, n_fe=t[0], has_cluster=t[1] != 0, has_weights=t[2] != 0)

    def totals(base, h):
        if h["n_instruments"] < 0 or h["n_fe"] < 0:
            return (-1, -1)
        return (base + _data_bytes(n_obs, k, h["n_instruments"], h["n_fe"], h["has_cluster"], h["has_weights"], 8),
                base + _data_bytes(n_obs, k, h["n_instruments"], h["n_fe"], h["has_cluster"], h["has_weights"], 4))

    n64, n32 = totals(HEADER_BASE_BYTES_NEW, new)
    o64, o32 = totals(HEADER_BASE_BYTES_OLD, old)
    match_new = file_size in (n64, n32, n64 + 4, n32 + 4)
    match_old = file_size in (o64, o32, o64 + 4, o32 + 4)
    if not match_new and not match_old:
        match_new = True
    if match_new:
        base = HEADER_BASE_BYTES_NEW
        l, n_fe, hc, hw = struct.unpack_from("<4i", buf, 12)
        hdr = fe_dataset_header(n_obs=n_obs, n_regressors=k, n_instruments=l, n_fe=n_fe, has_cluster=hc != 0,
                                has_weights=hw != 0)
        if l < 0:
            raise FeDataError("L must be non-negative")
    else:
        base = HEADER_BASE_BYTES_OLD
        n_fe, hc, hw = struct.unpack_from("<3i", buf, 12)
        hdr = fe_dataset_header(n_obs=n_obs, n_regressors=k, n_instruments=0, n_fe=n_fe, has_cluster=hc != 0,
                                has_weights=hw != 0)
    if hdr.n_fe < 0:
        raise FeDataError("n_fe must be non-negative")
    t64 = base + _data_bytes(n_obs, k, hdr.n_instruments, hdr.n_fe, hdr.has_cluster, hdr.has_weights, 8)
    t32 = base + _data_bytes(n_obs, k, hdr.n_instruments, hdr.n_fe, hdr.has_cluster, hdr.has_weights, 4)
    if file_size == t64:
        hdr.precision_flag = PRECISION_FLOAT64
        return hdr, base
    if file_size == t32:
        hdr.precision_flag = PRECISION_FLOAT32
        return hdr, base
    (flag,) = struct.unpack_from("<i", buf, base)
    hdr.precision_flag = flag
    if flag == PRECISION_FLOAT64:
        expected = base + 4 + _data_bytes(n_obs, k, hdr.n_instruments, hdr.n_fe, hdr.has_cluster, hdr.has_weights, 8)
    elif flag == PRECISION_FLOAT32:
        expected = base + 4 + _data_bytes(n_obs, k, hdr.n_instruments, hdr.n_fe, hdr.has_cluster, hdr.has_weights, 4)
    else:
        raise FeDataError(f"Unsupported precision flag value: {flag}")
    if file_size < expected:
        raise FeDataError("File size does not match header metadata for declared precision")
    hdr.metadata_bytes = file_size - expected
    return hdr, base + 4


def _read_text(mv: memoryview, pos: int) -> tuple[str, int]:
    (nch,) = struct.unpack_from("<i", mv, pos)
    pos += 4
    if nch < 0:
        raise FeDataError("Negative string length found in metadata block")
    s = bytes(mv[pos:pos + nch]).decode("utf-8", errors="replace")
    return s, pos + nch


def _read_text_list(mv: memoryview, pos: int) -> tuple[list, int]:
    (cnt,) = struct.unpack_from("<i", mv, pos)
    pos += 4
    if cnt < 0:
        raise FeDataError("Negative metadata string count")
    out = []
    for _ in range(cnt):
        s, pos = _read_text(mv, pos)
        out.append(s)
    return out, pos


def load_dataset_from_file(path: str) -> tuple[fe_dataset_header, fe_host_arrays]:
    if not os.path.exists(path):
        raise FeDataError(f"Dataset file not found: {path}")
    size = os.path.getsize(path)
    with open(path, "rb") as f:
        raw = f.read()
    hdr, pos = read_header(raw, size)
    n, k, l = hdr.n_obs, hdr.n_regressors, hdr.n_instruments
    vdt = np.float32 if hdr.precision_flag == PRECISION_FLOAT32 else np.float64
    vb = np.dtype(vdt).itemsize

    def take(count, dtype):
        nonlocal pos
        nb = count * np.dtype(dtype).itemsize
        if pos + nb > len(raw):
            raise FeDataError("IO error while reading data block")
        a = np.frombuffer(raw, dtype=np.dtype(dtype).newbyteorder("<"), count=count, offset=pos)
        pos += nb
        return a

    y = take(n, vdt).astype(np.float64)
    W = take(n * k, vdt).astype(np.float64).reshape((n, k), order="F") if k > 0 else np.zeros((n, 0), order="F")
    Z = take(n * l, vdt).astype(np.float64).reshape((n, l), order="F") if l > 0 else np.zeros((n, 0), order="F")
    fe = np.empty((hdr.n_fe, n), dtype=np.int32, order="F")
    for d in range(hdr.n_fe):
        fe[d, :] = take(n, np.int32)
    cluster = take(n, np.int32).copy() if hdr.has_cluster else None
    weights = take(n, vdt).astype(np.float64) if hdr.has_weights else None
    if hdr.metadata_bytes > 0:
        mv = memoryview(raw)
        if bytes(mv[pos:pos + 4]) != b"META":
            raise FeDataError("Unexpected metadata marker in dataset file")
        (version,) = struct.unpack_from("<i", mv, pos + 4)
        p = pos + 8
        if version != 1:
            raise FeDataError("Unsupported metadata version in dataset file")
        hdr.depvar_name, p = _read_text(mv, p)
        hdr.regressor_names, p = _read_text_list(mv, p)
        hdr.instrument_names, p = _read_text_list(mv, p)
        hdr.fe_names, p = _read_text_list(mv, p)
        hdr.cluster_name, p = _read_text(mv, p)
        hdr.weight_name, p = _read_text(mv, p)
    del vb
    host = fe_host_arrays(y=np.ascontiguousarray(y), W=np.asfortranarray(W), Z=np.asfortranarray(Z), fe_ids=fe,
                          cluster=cluster, weights=weights)
    return hdr, host


def _write_text(f, s: str) -> None:
    b = s.encode("utf-8")
    f.write(struct.pack("<i", len(b)))
    f.write(b)


def write_dataset(path: str, y, W, fe_ids, Z=None, cluster=None, weights=None, precision_flag: int = 0,
                  metadata: Optional[dict] = None, header: str = "new", write_flag: bool = True) -> None:
    """Write a ``.bin`` file. header='new' writes the 28-byte header (with L),
    'old' the 24-byte one; write_flag controls the trailing precision flag."""
    y = np.asarray(y)
    n = y.shape[0]
    W = np.zeros((n, 0)) if W is None else np.asarray(W)
    Z = np.zeros((n, 0)) if Z is None else np.asarray(Z)
    fe_ids = np.asarray(fe_ids).reshape(-1, n)
    dt = np.float32 if precision_flag == PRECISION_FLOAT32 else np.float64
    with open(path, "wb") as f:
        f.write(struct.pack("<q", n))
        f.write(struct.pack("<i", W.shape[1]))
        if header == "new":
            f.write(struct.pack("<i", Z.shape[1]))
        f.write(struct.pack("<i", fe_ids.shape[0]))
        f.write(struct.pack("<i", 1 if cluster is not None else 0))
        f.write(struct.pack("<i", 1 if weights is not None else 0))
        if write_flag:
            f.write(struct.pack("<i", precision_flag))
        f.write(y.astype(dt).tobytes())
        f.write(np.asarray(W, dtype=dt).tobytes(order="F"))
        if header == "new" and Z.shape[1] > 0:
            f.write(np.asarray(Z, dtype=dt).tobytes(order="F"))
        for d in range(fe_ids.shape[0]):
            f.write(fe_ids[d].astype("<i4").tobytes())
        if cluster is not None:
            f.write(np.asarray(cluster, dtype="<i4").tobytes())
        if weights is not None:
            f.write(np.asarray(weights, dtype=dt).tobytes())
        if metadata:
            f.write(b"META")
            f.write(struct.pack("<i", 1))
            _write_text(f, metadata.get("y", ""))
            for key in ("x", "iv", "fe"):
                items = metadata.get(key, [])
                f.write(struct.pack("<i", len(items)))
                for s in items:
                    _write_text(f, s)
            _write_text(f, metadata.get("cluster", ""))
            _write_text(f, metadata.get("weights", ""))


def read_metadata(path: str, offset: int, hdr: fe_dataset_header) -> fe_dataset_header:
    """Reads the META names block at byte offset into hdr (the tail parsed by
    load_dataset_from_file, src/io/fe_data_io.f90:360-389)."""
    if offset <= 0:
        return hdr
    with open(path, "rb") as f:
        f.seek(offset)
        raw = f.read()
    mv = memoryview(raw)
    if bytes(mv[0:4]) != b"META":
        raise FeDataError("Unexpected metadata marker in dataset file")
    (version,) = struct.unpack_from("<i", mv, 4)
    if version != 1:
        raise FeDataError("Unsupported metadata version in dataset file")
    p = 8
    hdr.depvar_name, p = _read_text(mv, p)
    hdr.regressor_names, p = _read_text_list(mv, p)
    hdr.instrument_names, p = _read_text_list(mv, p)
    hdr.fe_names, p = _read_text_list(mv, p)
    hdr.cluster_name, p = _read_text(mv, p)
    hdr.weight_name, p = _read_text(mv, p)
    return hdr


class DeviceDataset:
    """A .bin dataset loaded straight into device memory (fegb_load_bin).
    Device pointers: y, W, Z (column-major, ld n), fe_ids[d]; freed on close()."""

    def __init__(self, path: str):
        import ctypes as C

        from . import _native as N

        self._ds = N.FegbDataset()
        N.check(N.lib().fegb_load_bin(str(path).encode(), C.byref(self._ds)), "fegb_load_bin")
        d = self._ds
        self.n, self.k, self.l, self.n_fe = d.n, d.k, d.l, d.n_fe
        self.seconds = d.seconds
        self.header = fe_dataset_header(n_obs=d.n, n_regressors=d.k, n_instruments=d.l, n_fe=d.n_fe,
                                        has_cluster=bool(d.has_cluster), has_weights=bool(d.has_weights),
                                        precision_flag=d.precision_flag)
        read_metadata(path, d.metadata_offset, self.header)
        self.y = d.y or 0
        self.W = d.W or 0
        self.Z = d.Z or 0
        self.fe_ids = [(d.fe_ids or 0) + 4 * self.n * j for j in range(self.n_fe)]
        self.cluster = d.cluster or 0
        self.weights = d.weights or 0

    def close(self) -> None:
        import ctypes as C

        from . import _native as N

        if self._ds is not None:
            N.check(N.lib().fegb_free_dataset(C.byref(self._ds)), "fegb_free_dataset")
            self._ds = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
