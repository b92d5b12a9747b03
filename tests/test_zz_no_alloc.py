"""The workspace-free entry point tokura_zgeev_batched_gpu_noalloc, through the C ABI.

Some callers cannot allocate device memory when they need eigenvalues (for
example inside a host application that owns all device memory); this entry point stages matrices in a static
32 MiB device array instead of a caller workspace. Its results must match the
regular entry point's on the same inputs, on consecutive calls that reuse the
array. This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from oracle import lapack_oracle as lo
from tokura_zgeev_batched_gb300 import api
from tokura_zgeev_batched_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def regular(h, A, n, batch, stream):
    import torch

    eig = torch.empty(batch, n, dtype=torch.complex128, device="cuda")
    flag = torch.empty(batch, dtype=torch.int8, device="cuda")
    work = torch.empty(api.tokura_get_zgeeveigenvaluesgetworspacesize(n, batch), dtype=torch.uint8, device="cuda")
    st = api.lib().tokura_zgeev_batched_gpu(h.value, n, batch, A.data_ptr(), eig.data_ptr(), work.data_ptr(),
                                            flag.data_ptr(), stream)
    assert st == 0
    return eig, flag


def noalloc(h, A, n, batch, stream):
    import torch

    eig = torch.full((batch, n), complex(np.nan, np.nan), dtype=torch.complex128, device="cuda")
    flag = torch.full((batch,), 9, dtype=torch.int8, device="cuda")
    st = api.lib().tokura_zgeev_batched_gpu_noalloc(h.value, n, batch, A.data_ptr(), eig.data_ptr(), flag.data_ptr(),
                                                    stream)
    assert st == 0
    return eig, flag


def test_noalloc_matches_regular_on_two_consecutive_calls(cuda):
    import torch

    h = api.Handle()
    stream = torch.cuda.current_stream().cuda_stream
    cases = [(64, 512, 31), (17, 1000, 32)]  # second call reuses the array left by the first
    for n, batch, seed in cases:
        A_np = wl.gaussian(batch, n, seed=seed)
        A = torch.from_numpy(A_np).cuda()
        A0 = A.clone()
        e_ref, f_ref = regular(h, A, n, batch, stream)
        e_na, f_na = noalloc(h, A, n, batch, stream)
        torch.cuda.synchronize()
        assert torch.equal(A, A0)
        assert torch.equal(f_na, f_ref) and int((f_na != 0).sum()) == 0
        fro = np.sqrt(np.sum(np.abs(A_np) ** 2, axis=(1, 2)))
        err = lo.matched_abs_errors(e_na.cpu().numpy(), e_ref.cpu().numpy()).max(axis=1) / fro
        assert err.max() <= lo.TOL_REL_FRO, err.max()


def test_noalloc_rejects_batches_beyond_the_static_array(cuda):
    import torch

    h = api.Handle()
    limit = api.noalloc_max_bytes()
    assert limit == 32 << 20
    n = 64
    batch = limit // (16 * n * n) + 1
    A = torch.zeros(1, dtype=torch.complex128, device="cuda")
    st = api.lib().tokura_zgeev_batched_gpu_noalloc(h.value, n, batch, A.data_ptr(), A.data_ptr(), A.data_ptr(),
                                                    ctypes.c_void_p(0))
    assert st == -8
    assert api.lib().tokura_zgeev_batched_gpu_noalloc(None, n, 1, A.data_ptr(), A.data_ptr(), A.data_ptr(), None) == -1


def test_noalloc_with_and_without_room_for_shift_hints(cuda):
    """At n = 64, 500 matrices leave room for the FP32 hints behind the staging
    area and 512 do not: both calls succeed and match LAPACK."""
    import torch

    h = api.Handle()
    stream = torch.cuda.current_stream().cuda_stream
    for batch in (500, 512):
        A_np = wl.gaussian(batch, 64, seed=batch)
        A = torch.from_numpy(A_np).cuda()
        e, f = noalloc(h, A, 64, batch, stream)
        torch.cuda.synchronize()
        rep = lo.parity_report(A_np, e.cpu().numpy(), f.cpu().numpy(), with_cond=False)
        assert rep["flag_mismatch"] == 0 and rep["max_rel_err"] <= lo.TOL_REL_FRO
