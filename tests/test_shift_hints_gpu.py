"""FP32 shift hints (tokuraSetShiftHints): estimator accuracy, parity with
hints on and off, the estimator's second stream under graph capture and
concurrent callers."""
import numpy as np
import pytest

from oracle import lapack_oracle as lo
from tokura_zgeev_batched_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def solve(A_np, mode, work=None):
    import torch
    from tokura_zgeev_batched_gb300 import api

    h = api.Handle()
    assert h.set_shift_hints(mode) == 0
    A = torch.from_numpy(np.ascontiguousarray(A_np)).cuda()
    w, f = api.zgeev_batched(A, handle=h, work=work)
    torch.cuda.synchronize()
    return w.cpu().numpy(), f.cpu().numpy()


def test_set_shift_hints_validation(cuda):
    from tokura_zgeev_batched_gb300 import api

    h = api.Handle()
    assert h.set_shift_hints(0) == 0 and h.set_shift_hints(1) == 0 and h.set_shift_hints(2) == 0
    assert h.set_shift_hints(3) == -2 and h.set_shift_hints(-1) == -2


@pytest.mark.parametrize("cls", ["gaussian", "vdv", "companion"])
@pytest.mark.parametrize("n", [8, 16, 33, 64])
def test_parity_hints_on_and_off(cuda, cls, n):
    A = wl.GENERATORS[cls](160, n, seed=900 + n)
    for mode in (0, 1):
        w, f = solve(A, mode)
        rep = lo.parity_report(A, w, f)
        assert rep["flag_mismatch"] == 0, (mode, rep)
        if rep["well_conditioned"]:
            assert rep["max_rel_err_well"] <= lo.TOL_REL_FRO, (mode, rep["max_rel_err_well"])


@pytest.mark.parametrize("n", [12, 32, 64])
def test_estimates_are_single_precision_eigenvalues(cuda, n):
    """The workspace holds the FP32 estimates after a hinted call (n >= 12; 8n
    bytes per matrix after the 16n^2 staging bytes); they match LAPACK to FP32
    accuracy."""
    import torch
    from tokura_zgeev_batched_gb300 import api

    batch = 128
    A = wl.gaussian(batch, n, seed=77 + n)
    need = api.tokura_get_zgeeveigenvaluesgetworspacesize(n, batch)
    work = torch.zeros(need, dtype=torch.uint8, device="cuda")
    solve(A, 1, work=work)
    est = work[16 * n * n * batch: 16 * n * n * batch + 8 * n * batch].view(torch.float32).view(batch, n, 2)
    est = (est[..., 0].double() + 1j * est[..., 1].double()).cpu().numpy()
    w_ref = lo.zgeev(A)[0]
    fro = np.linalg.norm(A, axis=(1, 2))
    err = np.array([lo.matched_abs_errors(est[k], w_ref[k]).max() / fro[k] for k in range(batch)])
    assert np.median(err) < 1e-6 and err.max() < 1e-4, (np.median(err), err.max())


def test_hinted_call_in_cuda_graph(cuda):
    """The fork to the estimator's stream and the join back are captured."""
    import torch
    from tokura_zgeev_batched_gb300 import api

    n, batch = 40, 500
    A = torch.from_numpy(wl.gaussian(batch, n, seed=12)).cuda()
    eig = torch.empty(batch, n, dtype=torch.complex128, device="cuda")
    flag = torch.empty(batch, dtype=torch.int8, device="cuda")
    work = torch.empty(api.tokura_get_zgeeveigenvaluesgetworspacesize(n, batch), dtype=torch.uint8, device="cuda")
    h = api.Handle()
    assert h.set_shift_hints(1) == 0
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):  # warm-up outside capture
        assert api.tokura_zgeev_batched_gpu(h, n, batch, A.data_ptr(), eig.data_ptr(), work.data_ptr(),
                                            flag.data_ptr(), s.cuda_stream) == 0
    s.synchronize()
    ref = eig.clone()
    eig.zero_()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        st = api.tokura_zgeev_batched_gpu(h, n, batch, A.data_ptr(), eig.data_ptr(), work.data_ptr(),
                                          flag.data_ptr(), s.cuda_stream)
    assert st == 0
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(eig, ref) and (flag == 0).all()


def test_concurrent_streams_share_one_handle(cuda):
    import torch
    from tokura_zgeev_batched_gb300 import api

    h = api.Handle()
    assert h.set_shift_hints(1) == 0
    streams = [torch.cuda.Stream() for _ in range(3)]
    outs, refs = [], []
    for k, s in enumerate(streams):
        n = 24 + 8 * k
        A_np = wl.gaussian(300, n, seed=40 + k)
        A = torch.from_numpy(A_np).cuda()
        torch.cuda.synchronize()
        with torch.cuda.stream(s):
            w, f = api.zgeev_batched(A, handle=h, stream=s)
        outs.append((A_np, w, f))
    torch.cuda.synchronize()
    for A_np, w, f in outs:
        rep = lo.parity_report(A_np, w.cpu().numpy(), f.cpu().numpy(), with_cond=False)
        assert rep["flag_mismatch"] == 0 and rep["max_rel_err"] <= lo.TOL_REL_FRO


def test_hints_on_every_layout_match_contiguous(cuda):
    """Strided, pointer and complex64 calls run the same split solver: bitwise equal."""
    import torch
    from tokura_zgeev_batched_gb300 import api

    n = 48
    B = wl.torch_gaussian(96, 56, seed=3)
    A = B[:, :n, :n]
    w_s, f_s = api.zgeev_strided(A)
    w_c, f_c = api.zgeev_batched(A.contiguous())
    w_p, f_p = api.zgeev_pointers([A[k] for k in range(96)])
    torch.cuda.synchronize()
    assert torch.equal(w_s, w_c) and torch.equal(w_p, w_c)
    assert torch.equal(f_s, f_c) and torch.equal(f_p, f_c)


@pytest.mark.parametrize("lanes", [0, 1, 4])
def test_ragged_with_hints(cuda, lanes):
    """Modes 1 (orders >= 20 here) and 2 (every order) run the ragged forward
    in two phases with the estimator beside the first; parity with LAPACK and
    identical flags to mode 0."""
    import torch
    from tokura_zgeev_batched_gb300 import api

    rng = np.random.default_rng(31)
    mats = [wl.gaussian(1, int(n), seed=500 + k)[0] for k, n in enumerate(rng.integers(1, 65, size=240))]
    mats[17] = np.zeros_like(mats[17])
    mats[40] = mats[40].copy()
    mats[40][0, 0] = np.inf
    buf, ns, offs, eoffs = wl.pack_ragged([np.ascontiguousarray(m.T) for m in mats])
    out = {}
    for mode in (0, 1, 2):
        h = api.Handle()
        assert h.set_shift_hints(mode) == 0 and h.set_ragged_lanes(lanes) == 0
        assert h.set_ragged_hint_min_order(20) == 0
        eig, flag = api.zgeev_ragged(torch.from_numpy(buf).cuda(), torch.from_numpy(ns).cuda(), handle=h)
        torch.cuda.synchronize()
        out[mode] = (eig.cpu().numpy(), flag.cpu().numpy())
    for mode in (1, 2):
        assert np.array_equal(out[0][1], out[mode][1])
        eig, flag = out[mode]
        assert flag[40] == 2 and flag[17] == 0 and (np.delete(flag, 40) == 0).all()
        for k, m in enumerate(mats):
            if k == 40:
                continue
            n = m.shape[0]
            got = eig[eoffs[k]: eoffs[k] + n]
            if k == 17:
                assert (got == 0).all()
                continue
            w_ref = lo.zgeev(np.ascontiguousarray(m.T)[None])[0][0]
            assert lo.matched_abs_errors(got, w_ref).max() <= lo.TOL_REL_FRO * np.linalg.norm(m), (mode, k)


def test_set_ragged_hint_min_order_validation(cuda):
    from tokura_zgeev_batched_gb300 import api

    h = api.Handle()
    assert h.set_ragged_hint_min_order(1) == 0 and h.set_ragged_hint_min_order(65) == 0
    assert h.set_ragged_hint_min_order(0) == -2 and h.set_ragged_hint_min_order(66) == -2
