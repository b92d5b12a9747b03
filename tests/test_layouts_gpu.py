"""Strided, pointer-array and single-precision entry points.

Each must give bitwise the eigenvalues and flags of the contiguous entry
point on the same matrix entries (same solver, different loads/stores), and
parity with LAPACK follows from that; the FP32 path is checked against the
FP64 result of the widened matrix, rounded to nearest.
"""
import numpy as np
import pytest

from oracle import lapack_oracle as lo
from tokura_zgeev_batched_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def bits(t):
    return t.cpu().numpy().view(np.uint64 if t.element_size() == 16 else np.uint32)


def contiguous_solve(A):
    import torch
    from tokura_zgeev_batched_gb300 import api

    w, f = api.zgeev_batched(A.contiguous())
    torch.cuda.synchronize()
    return w, f


@pytest.mark.parametrize("n,big", [(1, 3), (7, 9), (16, 64), (33, 40), (64, 80)])
def test_subblocks_row_major(cuda, n, big):
    import torch
    from tokura_zgeev_batched_gb300 import api

    B = wl.torch_gaussian(200, big, seed=n)
    A = B[:, 1:n + 1, 2:n + 2] if big >= n + 2 else B[:, :n, :n]
    assert A.stride(-1) == 1 and A.stride(-2) == big
    w, f = api.zgeev_strided(A)
    w0, f0 = contiguous_solve(A)
    assert np.array_equal(bits(w), bits(w0))
    assert torch.equal(f, f0)


@pytest.mark.parametrize("n", [5, 32, 64])
def test_subblocks_column_major_and_parity(cuda, n):
    import torch
    from tokura_zgeev_batched_gb300 import api

    big = n + 11
    B = wl.torch_gaussian(150, big, seed=3 * n)
    A = B.transpose(-1, -2)[:, 3:n + 3, 4:n + 4]  # column-major with lda = big
    assert A.stride(-2) == 1 and A.stride(-1) == big
    w, f = api.zgeev_strided(A)
    # the kernel read A itself; the row-major copy of A^T has A as its column-major buffer
    w0, f0 = contiguous_solve(A.transpose(-1, -2))
    assert np.array_equal(bits(w), bits(w0))
    # LAPACK on the same matrices (column-major buffers of A^T have A's spectrum)
    An = A.contiguous().cpu().numpy()
    rep = lo.parity_report(An, w.cpu().numpy(), f.cpu().numpy())
    assert rep["flag_mismatch"] == 0
    assert rep["max_rel_err_well"] <= lo.TOL_REL_FRO, rep["max_rel_err_well"]


def test_broadcast_stride_zero_and_output_stride(cuda):
    import torch
    from tokura_zgeev_batched_gb300 import api

    n, batch, sw = 12, 100, 20
    one = wl.torch_gaussian(1, n, seed=11)
    A = one.expand(batch, n, n)
    assert A.stride(0) == 0
    w, f = api.zgeev_strided(A)
    assert (bits(w) == bits(w)[0]).all()
    # explicit output stride: gaps stay untouched
    At = one[0].transpose(0, 1).contiguous()  # its buffer is one[0] column-major
    out = torch.full((batch * sw,), complex(7.0, -7.0), dtype=torch.complex128, device="cuda")
    work = torch.empty(api.tokura_get_zgeeveigenvaluesgetworspacesize(n, batch), dtype=torch.uint8, device="cuda")
    flag = torch.empty(batch, dtype=torch.int8, device="cuda")
    h = api.default_handle()
    st = api.tokura_zgeev_strided_batched_gpu(h, n, batch, At.data_ptr(), n, 0, out.data_ptr(), sw, work.data_ptr(),
                                              flag.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert st == 0
    torch.cuda.synchronize()
    o = out.view(batch, sw)
    assert (o[:, n:] == complex(7.0, -7.0)).all()
    w1, _ = contiguous_solve(At[None])  # same buffer through the contiguous entry point
    assert (bits(o[:, :n]) == bits(w1)).all()  # (batch, 2n) against (1, 2n)
    assert (flag == 0).all()


def test_pointer_array_scattered(cuda):
    import torch
    from tokura_zgeev_batched_gb300 import api

    n = 24
    A = wl.torch_gaussian(300, n, seed=21)
    perm = torch.randperm(300, generator=torch.Generator().manual_seed(0))
    pool = A[perm].clone()  # matrices stored in a shuffled order
    inv = torch.argsort(perm)
    mats = [pool[int(inv[k])] for k in range(300)]
    w, f = api.zgeev_pointers(mats)
    w0, f0 = contiguous_solve(A)
    assert np.array_equal(bits(w), bits(w0))
    assert torch.equal(f, f0)


def test_pointer_array_lda_and_null(cuda):
    import torch
    from tokura_zgeev_batched_gb300 import api

    n, big = 10, 16
    B = wl.torch_gaussian(40, big, seed=5)
    mats = [B[k, :n, :n] for k in range(40)]
    mats[7] = None
    mats[39] = None
    w, f = api.zgeev_pointers(mats)
    fc = f.cpu().numpy()
    assert fc[7] == 3 and fc[39] == 3
    assert torch.isnan(w[7].real).all() and torch.isnan(w[39].imag).all()
    keep = [k for k in range(40) if mats[k] is not None]
    w0, f0 = contiguous_solve(torch.stack([mats[k] for k in keep]))
    assert np.array_equal(bits(w[keep]), bits(w0))
    assert (fc[keep] == 0).all()


@pytest.mark.parametrize("n", [1, 2, 9, 32, 64])
def test_complex64_is_rounded_fp64(cuda, n):
    import torch
    from tokura_zgeev_batched_gb300 import api

    A32 = wl.torch_gaussian(256, n, seed=40 + n).to(torch.complex64)
    w, f = api.cgeev_batched(A32)
    assert w.dtype == torch.complex64
    w64, f64 = contiguous_solve(A32.to(torch.complex128))
    assert np.array_equal(bits(w), bits(w64.to(torch.complex64)))
    assert torch.equal(f, f64)


def test_complex64_nonfinite(cuda):
    import torch
    from tokura_zgeev_batched_gb300 import api

    A32 = wl.torch_gaussian(8, 6, seed=1).to(torch.complex64)
    A32[3, 2, 1] = complex(float("inf"), 0.0)
    w, f = api.cgeev_batched(A32)
    fc = f.cpu().numpy()
    assert fc[3] == 2 and (np.delete(fc, 3) == 0).all()
    assert torch.isnan(w[3].real).all()


def test_strided_balanced_matches_contiguous(cuda):
    import torch
    from tokura_zgeev_batched_gb300 import api

    h = api.Handle()
    assert h.set_balancing(3) == 0
    B = wl.torch_gaussian(64, 40, seed=2)
    A = B[:, :33, :33]
    w, f = api.zgeev_strided(A, handle=h)
    w0, f0 = api.zgeev_batched(A.contiguous(), handle=h)
    torch.cuda.synchronize()
    assert np.array_equal(bits(w), bits(w0))
    assert torch.equal(f, f0)
