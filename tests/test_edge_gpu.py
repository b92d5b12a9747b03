"""Edge cases of the plain entry point on the GPU: flags, non-finite input, sizes, streams, graphs."""
import numpy as np
import pytest

from oracle import lapack_oracle as lo
from tokura_zgeev_batched_gb300 import api
from tokura_zgeev_batched_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def test_nonfinite_inputs_flagged(cuda):
    import torch

    A = wl.gaussian(40, 9, seed=1)
    A[3, 2, 5] = np.nan
    A[17, 0, 0] = np.inf
    A[33, 8, 8] = complex(1.0, -np.inf)
    At = torch.from_numpy(A).cuda()
    w, f = api.zgeev_batched(At)
    f = f.cpu().numpy()
    w = w.cpu().numpy()
    assert f[3] == 2 and f[17] == 2 and f[33] == 2
    assert np.isnan(w[3]).all() and np.isnan(w[17]).all()
    ok = np.ones(40, bool)
    ok[[3, 17, 33]] = False
    assert (f[ok] == 0).all()
    rep = lo.parity_report(A[ok], w[ok], f[ok])
    assert rep["max_rel_err"] <= lo.TOL_REL_FRO


def test_sweep_cap_sets_flag_and_returns(cuda):
    import torch

    h = api.Handle()
    assert h.set_sweep_cap(1) == 0
    A = torch.from_numpy(wl.gaussian(64, 20, seed=2)).cuda()
    w, f = api.zgeev_batched(A, handle=h)
    torch.cuda.synchronize()
    assert (f.cpu().numpy() == 1).all()
    assert h.set_sweep_cap(0) == 0
    w, f = api.zgeev_batched(A, handle=h)
    assert (f.cpu().numpy() == 0).all()


@pytest.mark.parametrize("batch", [1, 2, 31, 33, 97, 1000])
def test_ragged_tail_batches(cuda, batch):
    import torch

    for n in (3, 17, 64):
        A = wl.gaussian(batch, n, seed=batch * 100 + n)
        w, f = api.zgeev_batched(torch.from_numpy(A).cuda())
        rep = lo.parity_report(A, w.cpu().numpy(), f.cpu().numpy(), with_cond=False)
        assert rep["flag_mismatch"] == 0 and rep["max_rel_err"] <= 1e-11


def test_raw_entry_point_and_workspace_bound(cuda):
    """Raw C call on a user stream; the call must not write past the documented workspace."""
    import torch

    n, batch = 13, 77
    A = torch.from_numpy(wl.gaussian(batch, n, seed=4)).cuda()
    eig = torch.empty(batch, n, dtype=torch.complex128, device="cuda")
    flag = torch.full((batch + 64,), 7, dtype=torch.int8, device="cuda")
    need = api.tokura_get_zgeeveigenvaluesgetworspacesize(n, batch)
    guard = 4096
    work = torch.full((need + guard,), 0xAB, dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        st = api.tokura_zgeev_batched_gpu(api.default_handle(), n, batch, A.data_ptr(), eig.data_ptr(),
                                          work.data_ptr(), flag.data_ptr(), s.cuda_stream)
    assert st == 0
    s.synchronize()
    assert (work[need:] == 0xAB).all()
    assert (flag[batch:] == 7).all() and (flag[:batch] == 0).all()
    rep = lo.parity_report(A.cpu().numpy(), eig.cpu().numpy(), flag[:batch].cpu().numpy(), with_cond=False)
    assert rep["max_rel_err"] <= 1e-11


def test_cuda_graph_capture(cuda):
    import torch

    n, batch = 24, 300
    A = torch.from_numpy(wl.gaussian(batch, n, seed=8)).cuda()
    eig = torch.empty(batch, n, dtype=torch.complex128, device="cuda")
    flag = torch.empty(batch, dtype=torch.int8, device="cuda")
    work = torch.empty(api.tokura_get_zgeeveigenvaluesgetworspacesize(n, batch), dtype=torch.uint8, device="cuda")
    h = api.default_handle()
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        st = api.tokura_zgeev_batched_gpu(h, n, batch, A.data_ptr(), eig.data_ptr(), work.data_ptr(),
                                          flag.data_ptr(), torch.cuda.current_stream().cuda_stream)
        assert st == 0
    eig.zero_()
    g.replay()
    torch.cuda.synchronize()
    rep = lo.parity_report(A.cpu().numpy(), eig.cpu().numpy(), flag.cpu().numpy(), with_cond=False)
    assert rep["max_rel_err"] <= 1e-11 and rep["flag_mismatch"] == 0


def test_two_handles_and_concurrent_streams(cuda):
    import torch

    h1, h2 = api.Handle(), api.Handle()
    A1 = torch.from_numpy(wl.gaussian(500, 16, seed=10)).cuda()
    A2 = torch.from_numpy(wl.gaussian(500, 40, seed=11)).cuda()
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    w1, f1 = api.zgeev_batched(A1, handle=h1, stream=s1)
    w2, f2 = api.zgeev_batched(A2, handle=h2, stream=s2)
    torch.cuda.synchronize()
    for A, w, f in ((A1, w1, f1), (A2, w2, f2)):
        rep = lo.parity_report(A.cpu().numpy(), w.cpu().numpy(), f.cpu().numpy(), with_cond=False)
        assert rep["max_rel_err"] <= 1e-11


def test_lane_configs_agree(cuda):
    import torch

    A = torch.from_numpy(wl.gaussian(200, 33, seed=12)).cuda()
    outs = []
    for lanes in (1, 2, 4):
        h = api.Handle()
        assert h.set_plain_config(33, lanes, 64 * lanes) == 0
        assert h.plain_config(33, 200) == (lanes, 64 * lanes)
        w, f = api.zgeev_batched(A, handle=h)
        outs.append(w.cpu().numpy())
    for w in outs[1:]:
        assert lo.matched_abs_errors(w, outs[0]).max() < 1e-11 * 33


def test_purely_imaginary_subdiagonal(cuda):
    """A case the reference's real-part-only deflation test gets wrong (see tests/test_oracle.py)."""
    import torch

    H = np.array([[1, 2, 3], [2j, 4, 5], [0, 3j, 6]], np.complex128)
    A = np.stack([H, H.T.copy()])
    w, f = api.zgeev_batched(torch.from_numpy(A).cuda())
    rep = lo.parity_report(A, w.cpu().numpy(), f.cpu().numpy())
    assert rep["flag_mismatch"] == 0 and rep["max_rel_err"] <= lo.TOL_REL_FRO
