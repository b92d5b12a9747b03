"""Builds the in-tree CUDA library ``libtokura_zgeev_gb300.so`` for sm_103a.

The library is the C-ABI product (``include/tokura_blas.h``); Python reaches
it through ctypes (:mod:`tokura_zgeev_batched_gb300.api`). Translation units
compile in parallel with ``nvcc -gencode arch=compute_103a,code=sm_103a`` and
link with ``nvcc -shared``. A rebuild happens when any source is newer than
the library or the recorded build flags changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(REPO_DIR, "include")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_NAME = "libtokura_zgeev_gb300.so"
LIB_PATH = os.path.join(PKG_DIR, LIB_NAME)

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden", "--expt-relaxed-constexpr"]
SOURCES = [
    "zgeev_plain.cu",
    "peak_probe.cu",
    "zgeev_noalloc.cu",
    "zgeev_strided.cu",
    "zgeev_pointer.cu",
    "cgeev_batched.cu",
    "dgeev_batched.cu",
    "zgeev_ragged.cu",
    "zgeev_ragged_split.cu",
    "tokura_tuner.cu",
    "zgeev_backward.cu",
    "zgeev_vectors.cu",
    "tokura_capi.cpp",
    "compat_cxx.cpp",
    "tokura_host_pipeline.cpp",
    "tokura_host_alloc.cpp",
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the library")


def _flags_digest(extra: list[str]) -> str:
    return hashlib.sha1(" ".join(ARCH_FLAGS + NVCC_FLAGS + extra + SOURCES).encode()).hexdigest()


def _all_inputs() -> list[str]:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    files.append(os.path.abspath(__file__))
    return files


def needs_build(extra: list[str] | None = None) -> bool:
    extra = extra or []
    stamp = os.path.join(BUILD_DIR, "flags.sha1")
    if not os.path.exists(LIB_PATH) or not os.path.exists(stamp):
        return True
    with open(stamp) as f:
        if f.read().strip() != _flags_digest(extra):
            return True
    lib_mtime = os.path.getmtime(LIB_PATH)
    return any(os.path.getmtime(p) > lib_mtime for p in _all_inputs())


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
    cmd = [_nvcc(), "-c", os.path.join(CSRC, src), "-o", obj, "-I", INCLUDE, "-I", CSRC] + ARCH_FLAGS + NVCC_FLAGS + extra
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return obj


def build(force: bool = False, extra: list[str] | None = None, verbose: bool = False) -> str:
    """Compiles the library if needed and returns its path."""
    extra = list(extra or [])
    if not force and not needs_build(extra):
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, len(SOURCES))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    tmp = LIB_PATH + ".tmp"
    cmd = [_nvcc(), "-shared", "-o", tmp] + objs + ARCH_FLAGS + ["-Xcompiler", "-fPIC"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    with open(os.path.join(BUILD_DIR, "flags.sha1"), "w") as f:
        f.write(_flags_digest(extra))
    if verbose:
        print(f"built {LIB_PATH}", file=sys.stderr)
    return LIB_PATH


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
