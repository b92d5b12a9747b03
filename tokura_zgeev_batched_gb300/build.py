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
# Bounds-checked build (-DTOKURA_DEBUG_BOUNDS, csrc/zgeev_debug.cuh): a separate library.
DEBUG_BUILD_DIR = os.path.join(PKG_DIR, "_build_debug")
DEBUG_LIB_PATH = os.path.join(PKG_DIR, "libtokura_zgeev_gb300_debug.so")
DEBUG_FLAGS = ["-DTOKURA_DEBUG_BOUNDS"]

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
    "zgeev_ragged_bwd.cu",
    "tokura_tuner.cu",
    "zgeev_backward.cu",
    "zgeev_vectors.cu",
    "zgeev_debug.cu",
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


def _paths(debug: bool) -> tuple[str, str]:
    return (DEBUG_BUILD_DIR, DEBUG_LIB_PATH) if debug else (BUILD_DIR, LIB_PATH)


def needs_build(extra: list[str] | None = None, debug: bool = False) -> bool:
    extra = list(extra or []) + (DEBUG_FLAGS if debug else [])
    build_dir, lib_path = _paths(debug)
    stamp = os.path.join(build_dir, "flags.sha1")
    if not os.path.exists(lib_path) or not os.path.exists(stamp):
        return True
    with open(stamp) as f:
        if f.read().strip() != _flags_digest(extra):
            return True
    lib_mtime = os.path.getmtime(lib_path)
    return any(os.path.getmtime(p) > lib_mtime for p in _all_inputs())


def _compile(src: str, extra: list[str], build_dir: str = BUILD_DIR) -> str:
    obj = os.path.join(build_dir, os.path.basename(src) + ".o")
    cmd = [_nvcc(), "-c", os.path.join(CSRC, src), "-o", obj, "-I", INCLUDE, "-I", CSRC] + ARCH_FLAGS + NVCC_FLAGS + extra
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return obj


def build(force: bool = False, extra: list[str] | None = None, verbose: bool = False, debug: bool = False) -> str:
    """Compiles the library if needed and returns its path (``debug``: the bounds-checked
    library, a separate file)."""
    if not force and not needs_build(extra, debug):
        return _paths(debug)[1]
    extra = list(extra or []) + (DEBUG_FLAGS if debug else [])
    build_dir, lib_path = _paths(debug)
    os.makedirs(build_dir, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(max(os.cpu_count() or 8, 8), len(SOURCES))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, build_dir), SOURCES))
    tmp = lib_path + ".tmp"
    cmd = [_nvcc(), "-shared", "-o", tmp] + objs + ARCH_FLAGS + ["-Xcompiler", "-fPIC"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, lib_path)
    with open(os.path.join(build_dir, "flags.sha1"), "w") as f:
        f.write(_flags_digest(extra))
    if verbose:
        print(f"built {lib_path}", file=sys.stderr)
    return lib_path


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, debug="--debug" in sys.argv)
