"""Build the CUDA library libfegb.so for sm_103a and the CPU oracle library.

The CUDA sources under csrc/ are compiled in parallel with nvcc (one
-gencode, no cmake) and linked into fe_gpu_gb300/_build/libfegb.so.
The oracle (test infrastructure, oracle/fe_oracle.c) is compiled with gcc into
oracle/_build/libfe_oracle.so; it is never linked into libfegb.so.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"
ORACLE = ROOT / "oracle"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-diag-suppress", "177"]
SOURCES = ["prep.cu", "sweep.cu", "dense_umma.cu", "batch_est.cu", "linalg.cu", "fit.cu", "runtime.cu", "design.cu", "loader.cu"]
LIB_NAME = "libfegb.so"


def nvcc_path() -> str:
    cand = shutil.which("nvcc")
    if cand:
        return cand
    for p in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(p):
            return p
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfegb.so")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + proc.stdout + proc.stderr)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_cuda(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    nvcc = nvcc_path()
    headers = list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    objs = []
    jobs = []
    for src in SOURCES:
        s = CSRC / src
        o = BUILD / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-I", str(INCLUDE), "-I", str(CSRC), "-c", str(s), "-o", str(o)])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for _ in ex.map(_run, jobs):
                pass
    lib = BUILD / LIB_NAME
    if force or jobs or _stale(lib, objs):
        tmp = BUILD / (LIB_NAME + ".tmp")
        _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"])
        os.replace(tmp, lib)
    if verbose:
        print("built", lib)
    return lib


def build_oracle(force: bool = False) -> Path:
    out_dir = ORACLE / "_build"
    out_dir.mkdir(parents=True, exist_ok=True)
    lib = out_dir / "libfe_oracle.so"
    srcs = [ORACLE / "fe_oracle.c", ORACLE / "fe_oracle.h"]
    if force or _stale(lib, srcs):
        cc = shutil.which("gcc") or shutil.which("cc")
        if not cc:
            raise RuntimeError("a C compiler is required to build the oracle")
        tmp = out_dir / "libfe_oracle.so.tmp"
        _run([cc, "-O2", "-fopenmp", "-fPIC", "-shared", "-o", str(tmp), str(ORACLE / "fe_oracle.c"), "-lm"])
        os.replace(tmp, lib)
    return lib


def build_reference_cluster_builder() -> Path | None:
    """Compile the reference's own C cluster-id builder into oracle/_ref when
    the reference tree is present (recipe: oracle/build_ref.sh)."""
    script = ORACLE / "build_ref.sh"
    if not script.exists():
        return None
    proc = subprocess.run(["bash", str(script)], capture_output=True, text=True)
    lib = ORACLE / "_ref" / "libref_cluster_ids.so"
    if proc.returncode != 0 or not lib.exists():
        return None
    return lib


def main() -> int:
    force = "--force" in sys.argv
    build_cuda(force=force, verbose=True)
    build_oracle(force=force)
    build_reference_cluster_builder()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
