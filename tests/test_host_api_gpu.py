"""Host-buffer entry point: chunked, stream-pipelined copies + solves, same results as the device call."""
import numpy as np
import pytest

from oracle import lapack_oracle as lo
from tokura_zgeev_batched_gb300 import api
from tokura_zgeev_batched_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("chunk", [0, 7, 100, 5000])
def test_host_entry_matches_lapack(cuda, chunk):
    import torch

    A = wl.gaussian(1000, 12, seed=50)
    pinned = torch.from_numpy(A).pin_memory()
    h = api.Handle()
    w, f = api.zgeev_batched_host(pinned, handle=h, chunk_matrices=chunk)
    rep = lo.parity_report(A, w, f, with_cond=False)
    assert rep["flag_mismatch"] == 0 and rep["max_rel_err"] <= 1e-11
    # pageable numpy input, second call on the same handle (cached buffers are reused/grown)
    B = wl.gaussian(3000, 20, seed=51)
    w2, f2 = api.zgeev_batched_host(B, handle=h, chunk_matrices=chunk)
    rep = lo.parity_report(B, w2, f2, with_cond=False)
    assert rep["flag_mismatch"] == 0 and rep["max_rel_err"] <= 1e-11


def test_host_entry_argument_codes(cuda):
    import ctypes

    h = api.Handle()
    buf = (ctypes.c_char * 64)()
    p = ctypes.addressof(buf)
    f = api.tokura_zgeev_batched_host
    assert f(None, 2, 1, p, p, p) == -1
    assert f(h, 0, 1, p, p, p) == -2
    assert f(h, 2, 1, None, p, p) == -3
    assert f(h, 2, 1, p, None, p) == -4
    assert f(h, 2, 0, p, p, p) == -6
    assert f(h, 2, 1, p, p, None) == -7
    assert f(h, 2, 1, p, p, p, -1) == -8


@pytest.mark.parametrize("batch", [3000, 10000, 40000])
def test_host_entry_growing_chunks_bitwise_equal_device_call(cuda, batch):
    """The default chunk plan (1/16, 1/16, 1/8, 1/4, 1/2 of the batch, each at
    least 1,024 matrices) cuts the batch differently from the device call, but
    every matrix is solved by the same arithmetic: bitwise the same results."""
    import torch

    n = 16
    A = wl.torch_gaussian(batch, n, seed=batch)
    w_dev, f_dev = api.zgeev_batched(A)
    torch.cuda.synchronize()
    # zgeev_batched reads the row-major tensor as column-major A^T; pass the same buffer.
    A_host = A.cpu().pin_memory()
    w_host, f_host = api.zgeev_batched_host(A_host)
    assert np.array_equal(w_host.view(np.uint64), w_dev.cpu().numpy().view(np.uint64))
    assert np.array_equal(f_host, f_dev.cpu().numpy())
