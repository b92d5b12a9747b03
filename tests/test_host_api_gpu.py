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


@pytest.mark.parametrize("link_gbs", [0.0, 10.0, 1000.0])
@pytest.mark.parametrize("batch", [3000, 10000, 40000])
def test_host_entry_default_plans_bitwise_equal_device_call(cuda, batch, link_gbs):
    """Both default chunk plans (slow link: 1/16, 1/16, 1/8, 1/4, 1/2 of the
    batch; fast link: 2 equal chunks; each at least 1,024 matrices) cut the
    batch differently from the device call, but every matrix is solved by the
    same arithmetic: bitwise the same results. 0 = the measured rate: the
    second call plans with the rate the first one saw."""
    import torch

    n = 16
    A = wl.torch_gaussian(batch, n, seed=batch)
    w_dev, f_dev = api.zgeev_batched(A)
    torch.cuda.synchronize()
    h = api.Handle()
    assert h.set_host_link_rate(link_gbs) == 0
    # zgeev_batched reads the row-major tensor as column-major A^T; pass the same buffer.
    A_host = A.cpu().pin_memory()
    for _ in range(2):
        w_host, f_host = api.zgeev_batched_host(A_host, handle=h)
        assert np.array_equal(w_host.view(np.uint64), w_dev.cpu().numpy().view(np.uint64))
        assert np.array_equal(f_host, f_dev.cpu().numpy())


def test_set_host_link_rate_validation(cuda):
    h = api.Handle()
    assert h.set_host_link_rate(0.0) == 0 and h.set_host_link_rate(25.5) == 0
    assert h.set_host_link_rate(-1.0) == -2 and h.set_host_link_rate(float("nan")) == -2
    assert h.set_host_link_rate(float("inf")) == -2


def test_host_alloc_buffers_feed_the_host_entry(cuda):
    """tokuraHostAlloc memory (pinned, huge pages past one huge page) through the
    host entry point: bitwise the device call's results; explicit alloc/free codes."""
    import ctypes
    import gc

    import torch

    n, batch = 32, 80000  # 1.3 GB of input: spans more than one huge page
    A = wl.torch_gaussian(batch, n, seed=5)
    A_h = api.host_empty(A.shape, A.dtype)
    assert A_h.is_pinned() and A_h.shape == A.shape and A_h.dtype == A.dtype
    A_h.copy_(A)
    w_dev, f_dev = api.zgeev_batched(A)
    torch.cuda.synchronize()
    w_h, f_h = api.zgeev_batched_host(A_h)
    assert np.array_equal(w_h.view(np.uint64), w_dev.cpu().numpy().view(np.uint64))
    assert np.array_equal(f_h, f_dev.cpu().numpy())
    del A_h
    gc.collect()
    p = ctypes.c_void_p()
    assert api.lib().tokuraHostAlloc(ctypes.byref(p), 1000) == 0 and p.value
    ctypes.memset(p, 7, 1000)
    assert api.lib().tokuraHostFree(p) == 0
    assert api.lib().tokuraHostFree(p) == -1
