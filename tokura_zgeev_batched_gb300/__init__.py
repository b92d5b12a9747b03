"""GB300-native batched eigenvalue-only ZGEEV (drop-in for tokura_zgeev_batched).

The product is the C-ABI library built from ``csrc/`` (see ``include/
tokura_blas.h``); :mod:`.api` mirrors the reference's C API from Python and
adds torch-tensor wrappers.
"""
from .api import (  # noqa: F401
    MAX_MATRIX_SIZE,
    Handle,
    cgeev_batched,
    dgeev_batched,
    default_handle,
    exported_symbols,
    host_empty,
    lib,
    tokura_get_zgeeveigenvaluesgetworspacesize,
    tokura_zgeev_batched_gpu,
    tokuraCreate,
    tokuraDestroy,
    zgeev_batched,
    zgeev_batched_host,
    zgeev_pointers,
    zgeev_ragged,
    zgeev_strided,
    zgeev_vectors,
)
