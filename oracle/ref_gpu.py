"""TEST INFRASTRUCTURE — the reference library built for sm_103a, for a GPU comparison.

Only ``tests/``, ``__graft_entry__.build()`` and ``bench.py``'s baseline legs use this module;
the product never does.

Recipe (nothing of the reference is committed):
  * :func:`stage` copies the reference library's own sources
    (``tokura_zgeev_batched_library/src/*`` and ``include/*``) from the reference checkout
    (``TOKURA_REFERENCE_ROOT``, default ``/root/reference``) into ``oracle/_ref/src`` and
    ``oracle/_ref/include`` — git-ignored, so they travel with the working tree to a GPU
    machine without entering the history;
  * :func:`build` compiles them unmodified — ``tokura_zgeev_batched.cu``,
    ``tokura_zhseqr_helper.cu`` and ``tokura_zhseqr_MWB_helper.cu``, the files its own
    compile.sh builds into ``libtokurablas.so`` minus the tuner's ``main`` and ``set_mat.cu`` —
    together with ``oracle/ref_gpu_glue.cu`` (the three host functions the reference declares
    but never defines) into ``oracle/_ref/libtokurablas_ref.so`` for sm_103a.

Running the reference's kernels safely. Its kernels exit threads before block barriers
(``tokura_zgehrd_MWB_kernel.cuh:186-192``, ``tokura_zhseqr_MWB_kernel.cuh:639-652``) and let
the 32 matrices that share a warp leave the QR sweep loop at different passes while the
others keep executing ``__syncthreads`` (``tokura_zhseqr_MWB_kernel.cuh:725-727, 777``):
barriers in divergent control flow, which CUDA leaves undefined (they can hang). Its sweep
cap is n^4 passes (16.7 M at n = 64, ``:655``). :func:`solve_uniform` therefore only runs
batches whose size is a multiple of 32 in which every group of 32 consecutive matrices (one
thread block) holds 32 copies of one matrix, so every thread of a block follows the same
control flow, and only matrices that the CPU restatement of the reference's algorithm
(``oracle/ref_algorithm.c``) converges within a stated number of passes.
"""
from __future__ import annotations

import ctypes
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
SRC_DIR = os.path.join(REF_DIR, "src")
INC_DIR = os.path.join(REF_DIR, "include")
LIB_PATH = os.path.join(REF_DIR, "libtokurablas_ref.so")
GLUE = os.path.join(HERE, "ref_gpu_glue.cu")
LIBRARY_SOURCES = ("tokura_zgeev_batched.cu", "tokura_zhseqr_helper.cu", "tokura_zhseqr_MWB_helper.cu")

# C++-mangled names the reference library exports (its header has no extern "C").
SYM_CREATE = "_Z12tokuraCreatePP12tokurablas_t"
SYM_DESTROY = "_Z13tokuraDestroyP12tokurablas_t"
SYM_WORKSPACE = "_Z42tokura_get_zgeeveigenvaluesgetworspacesizeii"
SYM_SOLVE = "_Z24tokura_zgeev_batched_gpuP12tokurablas_tiiP7double2S2_S2_PcP11CUstream_st"

_lib = None


def reference_root() -> str:
    return os.environ.get("TOKURA_REFERENCE_ROOT", "/root/reference")


def stage() -> bool:
    """Copies the reference library's sources into oracle/_ref when the reference checkout is
    present; returns whether staged sources exist afterwards."""
    lib_root = os.path.join(reference_root(), "tokura_zgeev_batched_library")
    if os.path.isdir(lib_root):
        os.makedirs(SRC_DIR, exist_ok=True)
        os.makedirs(INC_DIR, exist_ok=True)
        for pat, dst in (("src/*.cu", SRC_DIR), ("src/*.cuh", SRC_DIR), ("src/*.h", SRC_DIR),
                         ("include/*.h", INC_DIR)):
            for f in glob.glob(os.path.join(lib_root, pat)):
                shutil.copyfile(f, os.path.join(dst, os.path.basename(f)))
    return staged()


def staged() -> bool:
    return all(os.path.exists(os.path.join(SRC_DIR, f)) for f in LIBRARY_SOURCES) and os.path.exists(
        os.path.join(INC_DIR, "tokura_blas.h"))


def _nvcc() -> str | None:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return None


def build(force: bool = False) -> str | None:
    """Builds oracle/_ref/libtokurablas_ref.so from the staged sources (returns its path, or
    None when no sources are staged or nvcc is missing)."""
    if not staged():
        return None
    nvcc = _nvcc()
    if nvcc is None:
        return None
    inputs = [os.path.join(SRC_DIR, f) for f in LIBRARY_SOURCES] + [GLUE]
    deps = inputs + glob.glob(os.path.join(SRC_DIR, "*")) + glob.glob(os.path.join(INC_DIR, "*"))
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(p) for p in deps):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc, "-shared", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "-Xcompiler", "-fPIC",
           "-I", INC_DIR, "-I", SRC_DIR, "-o", tmp] + inputs
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"reference build failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def undefined_symbols(path: str = LIB_PATH) -> list[str]:
    """Undefined tokura_* symbols of the built library (empty: every called helper is defined)."""
    out = subprocess.run(["nm", "-D", "-u", "-C", path], capture_output=True, text=True, check=True).stdout
    return [ln.split()[-1] for ln in out.splitlines() if "tokura" in ln]


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("reference library not built (oracle/_ref/libtokurablas_ref.so)")
        lib = ctypes.CDLL(LIB_PATH)
        getattr(lib, SYM_CREATE).argtypes = [ctypes.POINTER(ctypes.c_void_p)]
        getattr(lib, SYM_DESTROY).argtypes = [ctypes.c_void_p]
        getattr(lib, SYM_WORKSPACE).argtypes = [ctypes.c_int, ctypes.c_int]
        getattr(lib, SYM_WORKSPACE).restype = ctypes.c_size_t
        getattr(lib, SYM_SOLVE).argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 5
        _lib = lib
    return _lib


def safe_matrices(mats, max_passes_per_n: int = 20):
    """Indices of the matrices that the CPU restatement of the reference's algorithm converges
    within max_passes_per_n * n passes of its sweep loop, and the passes of all."""
    import numpy as np

    from oracle import lapack_oracle as lo

    mats = np.ascontiguousarray(mats)
    n = mats.shape[-1]
    _, flag, passes = lo.reference_algorithm(mats, return_sweeps=True)
    ok = np.nonzero((flag == 0) & (passes <= max_passes_per_n * n))[0]
    return ok, passes


def solve_uniform(distinct, stream=None, copies: int = 32, reps: int = 1):
    """Runs the reference's tokura_zgeev_batched_gpu on a device batch in which each of the
    ``distinct`` matrices (numpy ``[d, n, n]``, each read as a column-major buffer) fills one
    thread block as ``copies`` (= 32) consecutive copies. Returns ``(eigenvalues [d*32, n],
    flag [d*32], ms)`` with ``ms`` the CUDA-event time of one call (average of ``reps`` calls;
    A is re-copied before each, since the reference overwrites it)."""
    import numpy as np
    import torch

    if copies != 32:
        raise ValueError("one thread block of the reference's kernels holds 32 matrices")
    lib = load()
    d, n, _ = distinct.shape
    batch = d * copies
    dev = torch.device("cuda", torch.cuda.current_device())
    src = torch.from_numpy(np.ascontiguousarray(distinct)).to(dev).repeat_interleave(copies, dim=0)
    A = torch.empty_like(src)
    eig = torch.empty(batch, n, dtype=torch.complex128, device=dev)
    flag = torch.empty(batch, dtype=torch.int8, device=dev)
    work = torch.empty(int(getattr(lib, SYM_WORKSPACE)(n, batch)), dtype=torch.uint8, device=dev)
    h = ctypes.c_void_p()
    st = getattr(lib, SYM_CREATE)(ctypes.byref(h))
    if st != 0:
        raise RuntimeError(f"reference tokuraCreate returned {st}")
    s = stream if stream is not None else torch.cuda.current_stream(dev)
    total = 0.0
    try:
        for _ in range(reps):
            A.copy_(src)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(s)
            st = getattr(lib, SYM_SOLVE)(h, n, batch, A.data_ptr(), eig.data_ptr(), work.data_ptr(), flag.data_ptr(),
                                         s.cuda_stream)
            e1.record(s)
            torch.cuda.synchronize()
            if st != 0:
                raise RuntimeError(f"reference tokura_zgeev_batched_gpu returned {st}")
            total += e0.elapsed_time(e1)
    finally:
        getattr(lib, SYM_DESTROY)(h)
    return eig, flag, total / reps


if __name__ == "__main__":
    print("staged:", stage(), file=sys.stderr)
    print("built:", build(force="--force" in sys.argv), file=sys.stderr)
