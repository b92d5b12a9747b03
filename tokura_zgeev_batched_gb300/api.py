"""Host-side mirror of the reference's C API, over the in-tree C-ABI library.

The functions below keep the reference's names, argument order, argument
meaning and integer return codes (tokura_zgeev_batched_library/include/
tokura_blas.h:129-151, README.md:26-74); pointers are passed as integers
(device addresses) and streams as ``cudaStream_t`` integers, exactly what a
ctypes binding of the reference would pass. On top of that,
:func:`zgeev_batched` is a torch-tensor convenience wrapper.

The library must be built (``tokura_zgeev_batched_gb300.build.build()``);
loading fails loudly otherwise — there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

_LIB = None

MAX_MATRIX_SIZE = 64

# Exported C symbols declared in include/tokura_blas.h, with ctypes signatures.
_SIGNATURES = {
    "tokuraCreate": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p)]),
    "tokuraDestroy": (ctypes.c_int, [ctypes.c_void_p]),
    "tokura_get_zgeeveigenvaluesgetworspacesize": (ctypes.c_size_t, [ctypes.c_int, ctypes.c_int]),
    "tokura_zgeev_batched_gpu": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_void_p],
    ),
    "tokuraSetSweepCap": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "tokuraSetPlainConfig": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "tokuraSetPlainQrLanes": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "tokuraGetPlainConfig": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)],
    ),
    "tokura_probe_fp64_peak": (
        ctypes.c_int, [ctypes.POINTER(ctypes.c_double), ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "tokura_zgeev_batched_gpu_noalloc": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_void_p],
    ),
    "tokura_zgeev_noalloc_max_bytes": (ctypes.c_size_t, []),
    "tokura_zgeev_ragged_gpu": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
    ),
    "tokura_get_zgeev_ragged_workspacesize": (ctypes.c_size_t, [ctypes.c_int, ctypes.c_longlong]),
    "tokuraSetRaggedLanes": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "tokuraSetHostLinkRate": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    "tokuraSetRaggedHintMinOrder": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "tokuraHostAlloc": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]),
    "tokuraHostFree": (ctypes.c_int, [ctypes.c_void_p]),
    "tokuraAutotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]),
    "tokuraAutotuneRagged": (ctypes.c_int,
                             [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]),
    "tokuraSaveTuning": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "tokuraSetBalancing": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "tokuraSetShiftHints": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "tokuraSetScaledRotations": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "tokuraDebugAttach": (ctypes.c_int, [ctypes.c_void_p]),
    "tokura_zgeev_vectors_batched_gpu": (
        ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 7),
    "tokura_get_zgeev_vectors_workspacesize": (ctypes.c_size_t, [ctypes.c_int, ctypes.c_int]),
    "tokura_zgeev_batched_host": (
        ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 3 + [ctypes.c_int]),
    "tokura_zgeev_backward_gpu": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 7,
    ),
    "tokura_get_zgeev_backward_workspacesize": (ctypes.c_size_t, [ctypes.c_int, ctypes.c_int]),
    "tokura_zgeev_ragged_backward_gpu": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong]
        + [ctypes.c_void_p] * 7,
    ),
    "tokura_get_zgeev_ragged_backward_workspacesize": (ctypes.c_size_t, [ctypes.c_int, ctypes.c_longlong]),
    "tokuraLoadTuning": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "tokura_zgeev_strided_batched_gpu": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong,
         ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
    ),
    "tokura_zgeev_pointer_batched_gpu": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
    ),
    "tokura_get_dgeev_workspacesize": (ctypes.c_size_t, [ctypes.c_int, ctypes.c_int]),
    "tokura_dgeev_batched_gpu": (
        ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 6),
    "tokura_sgeev_batched_gpu": (
        ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 6),
    "tokuraSetRealConfig": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "tokura_cgeev_batched_gpu": (
        ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 5),
}


def exported_symbols() -> list[str]:
    return list(_SIGNATURES)


def debug_bounds_requested() -> bool:
    """TOKURA_ZGEEV_DEBUG_BOUNDS=1 selects the bounds-checked library (csrc/zgeev_debug.cuh) for
    this process; it must be set before the first call into the library."""
    return os.environ.get("TOKURA_ZGEEV_DEBUG_BOUNDS", "0") not in ("", "0")


def lib(autobuild: bool = True) -> ctypes.CDLL:
    """Loads (building first if allowed and needed) the C-ABI library."""
    global _LIB
    if _LIB is not None:
        return _LIB
    debug = debug_bounds_requested()
    path = _build.DEBUG_LIB_PATH if debug else _build.LIB_PATH
    if autobuild and _build.needs_build(debug=debug):
        _build.build(debug=debug)
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with tokura_zgeev_batched_gb300.build.build()")
    handle = ctypes.CDLL(path)
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(handle, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = handle
    return handle


class Handle:
    """Owns a ``tokurablas_t*`` (tokuraCreate/tokuraDestroy)."""

    def __init__(self):
        ptr = ctypes.c_void_p()
        status = lib().tokuraCreate(ctypes.byref(ptr))
        if status != 0:
            raise RuntimeError(f"tokuraCreate failed with status {status}")
        self.ptr = ptr

    @property
    def value(self) -> int:
        return self.ptr.value

    def set_sweep_cap(self, cap: int) -> int:
        return int(lib().tokuraSetSweepCap(self.ptr, int(cap)))

    def set_plain_config(self, n: int, lanes: int, threads: int) -> int:
        return int(lib().tokuraSetPlainConfig(self.ptr, int(n), int(lanes), int(threads)))

    def set_plain_qr_lanes(self, n: int, lanes: int) -> int:
        """Lanes per matrix of the hinted QR phase for order n (0: as the first launch)."""
        return int(lib().tokuraSetPlainQrLanes(self.ptr, int(n), int(lanes)))

    def plain_config(self, n: int, batch: int) -> tuple[int, int]:
        lanes, threads = ctypes.c_int(), ctypes.c_int()
        st = lib().tokuraGetPlainConfig(self.ptr, int(n), int(batch), ctypes.byref(lanes), ctypes.byref(threads))
        if st != 0:
            raise ValueError(f"tokuraGetPlainConfig returned {st}")
        return lanes.value, threads.value

    def autotune(self, n_min: int, n_max: int, batch_count: int, stream: int = 0) -> int:
        """Times all plain-kernel shapes for orders n_min..n_max and keeps the fastest (synchronizes)."""
        return int(lib().tokuraAutotune(self.ptr, int(n_min), int(n_max), int(batch_count), stream))

    def autotune_ragged(self, batch_count: int, n_min: int = 1, n_max: int = 64, stream: int = 0) -> int:
        return int(lib().tokuraAutotuneRagged(self.ptr, int(batch_count), int(n_min), int(n_max), stream))

    def save_tuning(self, path: str) -> int:
        return int(lib().tokuraSaveTuning(self.ptr, os.fsencode(path)))

    def load_tuning(self, path: str) -> int:
        return int(lib().tokuraLoadTuning(self.ptr, os.fsencode(path)))

    def set_balancing(self, mode: int) -> int:
        """0 none, 1 permute, 2 scale, 3 both (LAPACK zgeev's default)."""
        return int(lib().tokuraSetBalancing(self.ptr, int(mode)))

    def set_shift_hints(self, mode: int) -> int:
        """FP32 eigenvalue estimates as first shifts: 1 (default) uniform batches with n >= 12,
        2 every entry point and order (ragged too), 0 off (Wilkinson shifts only)."""
        return int(lib().tokuraSetShiftHints(self.ptr, int(mode)))

    def set_scaled_rotations(self, min_order: int) -> int:
        """QR with scaled rotations from order max(7, lanes * min_order) on (1..64; 65 = never)."""
        return int(lib().tokuraSetScaledRotations(self.ptr, int(min_order)))

    def set_real_config(self, n: int, lanes: int, threads: int) -> int:
        return int(lib().tokuraSetRealConfig(self.ptr, int(n), int(lanes), int(threads)))

    def set_ragged_lanes(self, lanes: int) -> int:
        return int(lib().tokuraSetRaggedLanes(self.ptr, int(lanes)))

    def set_ragged_hint_min_order(self, n: int) -> int:
        """Ragged calls under shift-hint mode 1 estimate orders >= n (65: none)."""
        return int(lib().tokuraSetRaggedHintMinOrder(self.ptr, int(n)))

    def set_host_link_rate(self, gbs: float) -> int:
        """Host-to-device GB/s the host-buffer call plans for (0 = the rate its last call measured)."""
        return int(lib().tokuraSetHostLinkRate(self.ptr, float(gbs)))

    def close(self):
        if self.ptr is not None and self.ptr.value:
            lib().tokuraDestroy(self.ptr)
        self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def tokuraCreate() -> tuple[int, Handle | None]:
    try:
        return 0, Handle()
    except RuntimeError:
        return 1, None


def tokuraDestroy(handle: Handle | None) -> int:
    if handle is not None:
        handle.close()
    return 0


def tokura_get_zgeeveigenvaluesgetworspacesize(n: int, batch_count: int) -> int:
    return int(lib().tokura_get_zgeeveigenvaluesgetworspacesize(int(n), int(batch_count)))


def _ptr(h) -> int | None:
    if h is None:
        return None
    if isinstance(h, Handle):
        return h.value
    if isinstance(h, ctypes.c_void_p):
        return h.value
    return int(h)


def tokura_zgeev_batched_gpu(handle, n: int, batch_count: int, A: int, eigenvalues: int, work: int, flag: int,
                             cudastream: int = 0) -> int:
    """Raw entry point: device addresses as integers, returns the C status."""
    return int(lib().tokura_zgeev_batched_gpu(_ptr(handle), int(n), int(batch_count), A, eigenvalues, work, flag,
                                              cudastream))


def tokura_zgeev_batched_gpu_noalloc(handle, n: int, batch_count: int, A: int, eigenvalues: int, flag: int,
                                     cudastream: int = 0) -> int:
    """Workspace-free entry point (static device staging array; see include/tokura_blas_ext.h)."""
    return int(lib().tokura_zgeev_batched_gpu_noalloc(_ptr(handle), int(n), int(batch_count), A, eigenvalues, flag,
                                                      cudastream))


def noalloc_max_bytes() -> int:
    return int(lib().tokura_zgeev_noalloc_max_bytes())


_DEFAULT_HANDLE = None


def default_handle() -> Handle:
    global _DEFAULT_HANDLE
    if _DEFAULT_HANDLE is None:
        _DEFAULT_HANDLE = Handle()
    return _DEFAULT_HANDLE


def zgeev_batched(A, handle: Handle | None = None, work=None, stream=None):
    """Eigenvalues of a batch of square complex128 CUDA matrices ``A[..., n, n]``.

    Returns ``(eigenvalues[..., n], flag[...])`` (flag int8: 0 converged,
    1 iteration cap hit, 2 non-finite input). A is not modified. Runs on the
    current torch stream unless ``stream`` (a torch.cuda.Stream) is given.
    """
    import torch

    if not A.is_cuda or A.dtype != torch.complex128:
        raise TypeError("A must be a complex128 CUDA tensor")
    n = A.shape[-1]
    if A.shape[-2] != n:
        raise ValueError("matrices must be square")
    batch_shape = A.shape[:-2]
    Ab = A.reshape(-1, n, n)
    # eig(M^T) = eig(M): the row-major buffer of M is the column-major buffer of M^T.
    Ab = Ab.contiguous()
    batch = Ab.shape[0]
    eig = torch.empty(batch, n, dtype=torch.complex128, device=A.device)
    flag = torch.empty(batch, dtype=torch.int8, device=A.device)
    if batch == 0:
        return eig.reshape(*batch_shape, n), flag.reshape(batch_shape)
    need = tokura_get_zgeeveigenvaluesgetworspacesize(n, batch)
    if work is None or work.numel() * work.element_size() < need:
        work = torch.empty(need, dtype=torch.uint8, device=A.device)
    s = stream if stream is not None else torch.cuda.current_stream(A.device)
    h = handle if handle is not None else default_handle()
    status = tokura_zgeev_batched_gpu(h, n, batch, Ab.data_ptr(), eig.data_ptr(), work.data_ptr(), flag.data_ptr(),
                                      s.cuda_stream)
    if status != 0:
        raise RuntimeError(f"tokura_zgeev_batched_gpu returned {status}")
    return eig.reshape(*batch_shape, n), flag.reshape(batch_shape)


def tokura_zgeev_strided_batched_gpu(handle, n: int, batch_count: int, A: int, lda: int, strideA: int,
                                     eigenvalues: int, strideW: int, work: int, flag: int, stream: int = 0) -> int:
    return int(lib().tokura_zgeev_strided_batched_gpu(_ptr(handle), int(n), int(batch_count), A, int(lda),
                                                      int(strideA), eigenvalues, int(strideW), work, flag, stream))


def tokura_zgeev_pointer_batched_gpu(handle, n: int, batch_count: int, Aarray: int, lda: int, eigenvalues: int,
                                     work: int, flag: int, stream: int = 0) -> int:
    return int(lib().tokura_zgeev_pointer_batched_gpu(_ptr(handle), int(n), int(batch_count), Aarray, int(lda),
                                                      eigenvalues, work, flag, stream))


def tokura_cgeev_batched_gpu(handle, n: int, batch_count: int, A: int, eigenvalues: int, work: int, flag: int,
                             stream: int = 0) -> int:
    return int(lib().tokura_cgeev_batched_gpu(_ptr(handle), int(n), int(batch_count), A, eigenvalues, work, flag,
                                              stream))


def _column_major_view(M):
    """(leading dimension, transposed?) for a CUDA matrix view whose rows or
    columns are unit-stride, or None. eig(M^T) = eig(M), so a row-major view
    is read as the column-major view of M^T."""
    r, c = M.stride(-2), M.stride(-1)
    n = M.shape[-1]
    if n == 1:
        return 1, False
    if r == 1 and c >= n:
        return c, False
    if c == 1 and r >= n:
        return r, True
    return None


def zgeev_strided(A, handle: Handle | None = None, work=None, stream=None):
    """Eigenvalues of a 3-D complex128 CUDA tensor ``A[b, n, n]`` read in place
    through its strides (e.g. ``big[:, :n, :n]`` sub-blocks or an expanded
    single matrix), via tokura_zgeev_strided_batched_gpu. Falls back to a
    contiguous copy only when neither matrix dimension is unit-stride.
    Returns ``(eigenvalues[b, n], flag[b])``.
    """
    import torch

    if not A.is_cuda or A.dtype != torch.complex128 or A.dim() != 3 or A.shape[-1] != A.shape[-2]:
        raise TypeError("A must be a 3-D complex128 CUDA tensor of square matrices")
    batch, n = A.shape[0], A.shape[-1]
    view = _column_major_view(A)
    if view is None or A.stride(0) < 0:
        A = A.contiguous()
        view = _column_major_view(A)
    lda = view[0]
    eig = torch.empty(batch, n, dtype=torch.complex128, device=A.device)
    flag = torch.empty(batch, dtype=torch.int8, device=A.device)
    if batch == 0:
        return eig, flag
    need = tokura_get_zgeeveigenvaluesgetworspacesize(n, batch)
    if work is None or work.numel() * work.element_size() < need:
        work = torch.empty(need, dtype=torch.uint8, device=A.device)
    s = stream if stream is not None else torch.cuda.current_stream(A.device)
    h = handle if handle is not None else default_handle()
    st = tokura_zgeev_strided_batched_gpu(h, n, batch, A.data_ptr(), lda, A.stride(0) if batch > 1 else 0,
                                          eig.data_ptr(), n, work.data_ptr(), flag.data_ptr(), s.cuda_stream)
    if st != 0:
        raise RuntimeError(f"tokura_zgeev_strided_batched_gpu returned {st}")
    return eig, flag


def zgeev_pointers(mats, handle: Handle | None = None, work=None, stream=None):
    """Eigenvalues of a list of complex128 CUDA matrices (each ``[n, n]``, any
    addresses, one common leading dimension) via the pointer-array entry point.
    ``None`` entries are passed as NULL pointers (flag 3, NaN eigenvalues).
    Returns ``(eigenvalues[len, n], flag[len])``.
    """
    import torch

    present = [m for m in mats if m is not None]
    if not present:
        raise ValueError("need at least one matrix")
    dev = present[0].device
    n = present[0].shape[-1]
    views = {_column_major_view(m) for m in present}
    if len(views) != 1 or None in views or any(m.shape != (n, n) or m.dtype != torch.complex128 for m in present):
        raise ValueError("matrices must be complex128 [n, n] views sharing one leading dimension")
    lda = views.pop()[0]
    batch = len(mats)
    ptrs = torch.tensor([m.data_ptr() if m is not None else 0 for m in mats], dtype=torch.int64).to(dev)
    eig = torch.empty(batch, n, dtype=torch.complex128, device=dev)
    flag = torch.empty(batch, dtype=torch.int8, device=dev)
    need = tokura_get_zgeeveigenvaluesgetworspacesize(n, batch)
    if work is None or work.numel() * work.element_size() < need:
        work = torch.empty(need, dtype=torch.uint8, device=dev)
    s = stream if stream is not None else torch.cuda.current_stream(dev)
    h = handle if handle is not None else default_handle()
    st = tokura_zgeev_pointer_batched_gpu(h, n, batch, ptrs.data_ptr(), lda, eig.data_ptr(), work.data_ptr(),
                                          flag.data_ptr(), s.cuda_stream)
    if st != 0:
        raise RuntimeError(f"tokura_zgeev_pointer_batched_gpu returned {st}")
    return eig, flag


def cgeev_batched(A, handle: Handle | None = None, work=None, stream=None):
    """Eigenvalues of complex64 CUDA matrices ``A[..., n, n]``, computed in FP64
    and returned as complex64 (tokura_cgeev_batched_gpu). Returns
    ``(eigenvalues[..., n], flag[...])``."""
    import torch

    if not A.is_cuda or A.dtype != torch.complex64:
        raise TypeError("A must be a complex64 CUDA tensor")
    n = A.shape[-1]
    if A.shape[-2] != n:
        raise ValueError("matrices must be square")
    batch_shape = A.shape[:-2]
    Ab = A.reshape(-1, n, n).contiguous()
    batch = Ab.shape[0]
    eig = torch.empty(batch, n, dtype=torch.complex64, device=A.device)
    flag = torch.empty(batch, dtype=torch.int8, device=A.device)
    if batch == 0:
        return eig.reshape(*batch_shape, n), flag.reshape(batch_shape)
    need = tokura_get_zgeeveigenvaluesgetworspacesize(n, batch)
    if work is None or work.numel() * work.element_size() < need:
        work = torch.empty(need, dtype=torch.uint8, device=A.device)
    s = stream if stream is not None else torch.cuda.current_stream(A.device)
    h = handle if handle is not None else default_handle()
    st = tokura_cgeev_batched_gpu(h, n, batch, Ab.data_ptr(), eig.data_ptr(), work.data_ptr(), flag.data_ptr(),
                                  s.cuda_stream)
    if st != 0:
        raise RuntimeError(f"tokura_cgeev_batched_gpu returned {st}")
    return eig.reshape(*batch_shape, n), flag.reshape(batch_shape)


def tokura_get_dgeev_workspacesize(n: int, batch_count: int) -> int:
    return int(lib().tokura_get_dgeev_workspacesize(int(n), int(batch_count)))


def tokura_dgeev_batched_gpu(handle, n: int, batch_count: int, A: int, wr: int, wi: int, work: int, flag: int,
                             stream: int = 0) -> int:
    return int(lib().tokura_dgeev_batched_gpu(_ptr(handle), int(n), int(batch_count), A, wr, wi, work, flag, stream))


def tokura_sgeev_batched_gpu(handle, n: int, batch_count: int, A: int, wr: int, wi: int, work: int, flag: int,
                             stream: int = 0) -> int:
    return int(lib().tokura_sgeev_batched_gpu(_ptr(handle), int(n), int(batch_count), A, wr, wi, work, flag, stream))


def dgeev_batched(A, handle: Handle | None = None, work=None, stream=None):
    """Eigenvalues of real CUDA matrices ``A[..., n, n]`` (float64 -> dgeev
    path, float32 -> sgeev path, FP64 inside). Returns ``(wr, wi, flag)`` in
    LAPACK's convention (conjugate pairs adjacent, positive imaginary part
    first). Matrices are taken as stored by torch (row-major); eig(M^T) =
    eig(M), so the spectrum is that of A.
    """
    import torch

    if not A.is_cuda or A.dtype not in (torch.float64, torch.float32):
        raise TypeError("A must be a float64 or float32 CUDA tensor")
    n = A.shape[-1]
    if A.shape[-2] != n:
        raise ValueError("matrices must be square")
    batch_shape = A.shape[:-2]
    Ab = A.reshape(-1, n, n).contiguous()
    batch = Ab.shape[0]
    wr = torch.empty(batch, n, dtype=A.dtype, device=A.device)
    wi = torch.empty(batch, n, dtype=A.dtype, device=A.device)
    flag = torch.empty(batch, dtype=torch.int8, device=A.device)
    if batch > 0:
        need = tokura_get_dgeev_workspacesize(n, batch)
        if work is None or work.numel() * work.element_size() < need:
            work = torch.empty(need, dtype=torch.uint8, device=A.device)
        s = stream if stream is not None else torch.cuda.current_stream(A.device)
        h = handle if handle is not None else default_handle()
        fn = tokura_dgeev_batched_gpu if A.dtype == torch.float64 else tokura_sgeev_batched_gpu
        st = fn(h, n, batch, Ab.data_ptr(), wr.data_ptr(), wi.data_ptr(), work.data_ptr(), flag.data_ptr(),
                s.cuda_stream)
        if st != 0:
            raise RuntimeError(f"{fn.__name__} returned {st}")
    return wr.reshape(*batch_shape, n), wi.reshape(*batch_shape, n), flag.reshape(batch_shape)


def probe_fp64_peak(device=None) -> float:
    """Measured FP64 FMA throughput of the device in FLOP/s (synchronizes)."""
    import torch

    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    scratch = torch.empty(512 * sms, dtype=torch.float64, device=dev)
    out = ctypes.c_double()
    st = lib().tokura_probe_fp64_peak(ctypes.byref(out), scratch.data_ptr(), scratch.numel(),
                                      torch.cuda.current_stream(dev).cuda_stream)
    if st != 0:
        raise RuntimeError(f"tokura_probe_fp64_peak returned {st}")
    return out.value


def tokura_get_zgeev_ragged_workspacesize(batch_count: int, total_elements: int) -> int:
    return int(lib().tokura_get_zgeev_ragged_workspacesize(int(batch_count), int(total_elements)))


def tokura_zgeev_ragged_gpu(handle, batch_count: int, n: int, offsets: int, eig_offsets: int | None,
                            total_elements: int, A: int, eigenvalues: int, work: int, flag: int,
                            stream: int = 0) -> int:
    """Raw ragged entry point (device addresses as integers)."""
    return int(lib().tokura_zgeev_ragged_gpu(_ptr(handle), int(batch_count), n, offsets, eig_offsets,
                                             int(total_elements), A, eigenvalues, work, flag, stream))


def zgeev_ragged(A_packed, n, offsets=None, eig_offsets=None, handle: Handle | None = None, work=None,
                 stream=None, total_eigenvalues: int | None = None):
    """Eigenvalues of a ragged batch on the GPU.

    ``A_packed``: 1-D complex128 CUDA tensor with the matrices one after another
    (column-major each); ``n``: int32 CUDA tensor of orders; ``offsets``: int64
    element offsets (default: packed, exclusive prefix sum of n^2). Returns
    ``(eigenvalues, flag)`` with eigenvalues packed by the prefix sum of n
    unless ``eig_offsets`` is given (then the output holds ``max(eig_offsets + n)`` entries).
    Pass ``offsets`` and ``total_eigenvalues`` to avoid host synchronisation.
    """
    import torch

    if not A_packed.is_cuda or A_packed.dtype != torch.complex128 or A_packed.dim() != 1:
        raise TypeError("A_packed must be a 1-D complex128 CUDA tensor")
    dev = A_packed.device
    n = n.to(device=dev, dtype=torch.int32).contiguous()
    batch = n.numel()
    n64 = n.to(torch.int64)
    if offsets is None:
        offsets = torch.cumsum(n64 * n64, 0) - n64 * n64
    offsets = offsets.to(device=dev, dtype=torch.int64).contiguous()
    if eig_offsets is None:
        # total_eigenvalues avoids a host synchronisation (e.g. under CUDA-graph capture)
        total_eig = total_eigenvalues if total_eigenvalues is not None else (int(n64.sum().item()) if batch else 0)
        eptr = None
    else:
        eig_offsets = eig_offsets.to(device=dev, dtype=torch.int64).contiguous()
        total_eig = int((eig_offsets + n64).max().item()) if batch else 0
        eptr = eig_offsets.data_ptr()
    eig = torch.empty(max(total_eig, 1), dtype=torch.complex128, device=dev)
    flag = torch.empty(batch, dtype=torch.int8, device=dev)
    if batch == 0:
        return eig[:0], flag
    total = A_packed.numel()
    need = tokura_get_zgeev_ragged_workspacesize(batch, total)
    if work is None or work.numel() * work.element_size() < need:
        work = torch.empty(need, dtype=torch.uint8, device=dev)
    s = stream if stream is not None else torch.cuda.current_stream(dev)
    h = handle if handle is not None else default_handle()
    st = tokura_zgeev_ragged_gpu(h, batch, n.data_ptr(), offsets.data_ptr(), eptr, total, A_packed.data_ptr(),
                                 eig.data_ptr(), work.data_ptr(), flag.data_ptr(), s.cuda_stream)
    if st != 0:
        raise RuntimeError(f"tokura_zgeev_ragged_gpu returned {st}")
    return eig[:total_eig], flag


def tokura_zgeev_backward_gpu(handle, n: int, batch_count: int, A: int, eigenvalues: int, grad_eigenvalues: int,
                              grad_A: int, work: int, flag: int, stream: int = 0) -> int:
    return int(lib().tokura_zgeev_backward_gpu(_ptr(handle), int(n), int(batch_count), A, eigenvalues,
                                               grad_eigenvalues, grad_A, work, flag, stream))


def tokura_get_zgeev_backward_workspacesize(n: int, batch_count: int) -> int:
    return int(lib().tokura_get_zgeev_backward_workspacesize(int(n), int(batch_count)))


def tokura_zgeev_ragged_backward_gpu(handle, batch_count: int, n: int, offsets: int, eig_offsets: int | None,
                                     total_elements: int, A: int, eigenvalues: int, grad_eigenvalues: int,
                                     grad_A: int, work: int, flag: int, stream: int = 0) -> int:
    return int(lib().tokura_zgeev_ragged_backward_gpu(_ptr(handle), int(batch_count), n, offsets, eig_offsets,
                                                      int(total_elements), A, eigenvalues, grad_eigenvalues, grad_A,
                                                      work, flag, stream))


def tokura_get_zgeev_ragged_backward_workspacesize(batch_count: int, total_elements: int) -> int:
    return int(lib().tokura_get_zgeev_ragged_backward_workspacesize(int(batch_count), int(total_elements)))


def zgeev_backward(A, eigenvalues, grad_eigenvalues, handle: Handle | None = None, work=None, stream=None):
    """grad_A for a batch ``A[..., n, n]`` (torch's complex-gradient convention). Returns (grad_A, flag)."""
    import torch

    n = A.shape[-1]
    Ab = A.reshape(-1, n, n).contiguous()
    batch = Ab.shape[0]
    lam = eigenvalues.reshape(batch, n).contiguous()
    g = grad_eigenvalues.reshape(batch, n).to(torch.complex128).contiguous()
    gA = torch.empty_like(Ab)
    flag = torch.empty(batch, dtype=torch.int8, device=A.device)
    if batch == 0:
        return gA.reshape(A.shape), flag
    need = tokura_get_zgeev_backward_workspacesize(n, batch)
    if work is None or work.numel() * work.element_size() < need:
        work = torch.empty(need, dtype=torch.uint8, device=A.device)
    s = stream if stream is not None else torch.cuda.current_stream(A.device)
    h = handle if handle is not None else default_handle()
    st = tokura_zgeev_backward_gpu(h, n, batch, Ab.data_ptr(), lam.data_ptr(), g.data_ptr(), gA.data_ptr(),
                                   work.data_ptr(), flag.data_ptr(), s.cuda_stream)
    if st != 0:
        raise RuntimeError(f"tokura_zgeev_backward_gpu returned {st}")
    return gA.reshape(A.shape), flag


def tokura_zgeev_batched_host(handle, n: int, batch_count: int, A: int, eigenvalues: int, flag: int,
                              chunk_matrices: int = 0) -> int:
    """Host-buffer entry point (host addresses as integers); blocks until the results are on the host."""
    return int(lib().tokura_zgeev_batched_host(_ptr(handle), int(n), int(batch_count), A, eigenvalues, flag,
                                               int(chunk_matrices)))


class HostBlock:
    """Owns memory from tokuraHostAlloc (pinned, on huge pages); freed when the last reference goes."""

    def __init__(self, nbytes: int):
        p = ctypes.c_void_p()
        st = lib().tokuraHostAlloc(ctypes.byref(p), int(nbytes))
        if st != 0:
            raise RuntimeError(f"tokuraHostAlloc returned {st}")
        self.ptr = p.value
        self.nbytes = int(nbytes)

    def __del__(self):
        if getattr(self, "ptr", None):
            try:
                lib().tokuraHostFree(ctypes.c_void_p(self.ptr))
            except Exception:  # noqa: BLE001 - interpreter shutdown: the process unmaps it anyway
                pass
            self.ptr = None


def host_empty(shape, dtype):
    """Uninitialised CPU torch tensor in tokuraHostAlloc memory (pinned, huge pages): the host
    buffers for :func:`zgeev_batched_host` / ``tokura_zgeev_batched_host``."""
    import math

    import numpy as np
    import torch

    shape = tuple(int(s) for s in shape)
    itemsize = torch.empty((), dtype=dtype).element_size()
    nbytes = max(1, math.prod(shape)) * itemsize
    block = HostBlock(nbytes)
    raw = (ctypes.c_uint8 * nbytes).from_address(block.ptr)
    raw.block = block  # tensor -> numpy array -> raw -> block: freed with the last view
    t = torch.from_numpy(np.ctypeslib.as_array(raw)).view(dtype)
    return t[: math.prod(shape)].view(shape)


def zgeev_batched_host(A, handle: Handle | None = None, chunk_matrices: int = 0):
    """Eigenvalues of host-resident matrices (numpy complex128 ``[..., n, n]`` or a CPU torch tensor).

    Pinned (page-locked) torch tensors let the copies overlap the solves; :func:`host_empty`
    gives pinned memory on huge pages, which keeps the host link at full rate.
    Returns numpy ``(eigenvalues[..., n], flag[...])``.
    """
    import numpy as np

    if hasattr(A, "numpy"):
        arr = A.contiguous()
        ptr = arr.data_ptr()
        shape = tuple(arr.shape)
        keep = arr
    else:
        keep = np.ascontiguousarray(A, dtype=np.complex128)
        ptr = keep.ctypes.data
        shape = keep.shape
    n = shape[-1]
    batch = int(np.prod(shape[:-2])) if len(shape) > 2 else 1
    eig = np.empty((batch, n), np.complex128)
    flag = np.empty(batch, np.int8)
    h = handle if handle is not None else default_handle()
    st = tokura_zgeev_batched_host(h, n, batch, ptr, eig.ctypes.data, flag.ctypes.data, chunk_matrices)
    del keep
    if st != 0:
        raise RuntimeError(f"tokura_zgeev_batched_host returned {st}")
    return eig.reshape(*shape[:-2], n), flag.reshape(shape[:-2])


def tokura_get_zgeev_vectors_workspacesize(n: int, batch_count: int) -> int:
    return int(lib().tokura_get_zgeev_vectors_workspacesize(int(n), int(batch_count)))


def zgeev_vectors(A, left: bool = True, right: bool = True, handle: Handle | None = None, stream=None):
    """Eigenvalues and eigenvectors of complex128 CUDA matrices ``A[..., n, n]`` (ZGEEV with 'V').

    The matrices are taken as stored by torch (row-major). Returns
    ``(w[..., n], VL, VR, flag)`` with ``VR[..., :, i]`` the right eigenvector of
    ``w[..., i]`` (``A @ VR = VR @ diag(w)``) and ``VL[..., :, i]`` the left one
    (``VL^H @ A = diag(w) @ VL^H``), each unit-norm with its largest component
    real; VL / VR are None when not requested.
    """
    import torch

    n = A.shape[-1]
    batch_shape = A.shape[:-2]
    # The library reads column-major buffers: pass A^T (row-major A read as column-major is A^T).
    At = A.reshape(-1, n, n).transpose(-1, -2).contiguous()
    batch = At.shape[0]
    w = torch.empty(batch, n, dtype=torch.complex128, device=A.device)
    flag = torch.empty(batch, dtype=torch.int8, device=A.device)
    VLc = torch.empty(batch, n, n, dtype=torch.complex128, device=A.device) if left else None
    VRc = torch.empty(batch, n, n, dtype=torch.complex128, device=A.device) if right else None
    work = torch.empty(int(lib().tokura_get_zgeev_vectors_workspacesize(n, batch)), dtype=torch.uint8,
                       device=A.device)
    s = stream if stream is not None else torch.cuda.current_stream(A.device)
    h = handle if handle is not None else default_handle()
    st = int(lib().tokura_zgeev_vectors_batched_gpu(_ptr(h), n, batch, At.data_ptr(), w.data_ptr(),
                                                    VLc.data_ptr() if left else None,
                                                    VRc.data_ptr() if right else None, work.data_ptr(),
                                                    flag.data_ptr(), s.cuda_stream))
    if st != 0:
        raise RuntimeError(f"tokura_zgeev_vectors_batched_gpu returned {st}")
    # Column-major results read back row-major are transposed: undo.
    VL = VLc.transpose(-1, -2).reshape(*batch_shape, n, n) if left else None
    VR = VRc.transpose(-1, -2).reshape(*batch_shape, n, n) if right else None
    return w.reshape(*batch_shape, n), VL, VR, flag.reshape(batch_shape)
