"""The hinted plain call's QR phase at its own lane width (tokuraSetPlainQrLanes).

With shift hints the plain call is two launches (staging + Hessenberg, then the
QR); the QR launch may use fewer or more lanes per matrix than the first one,
reading the matrices from the first launch's staging tiles. Every width must
agree with LAPACK zgeev (the oracle) with identical flags; the library's own
choice (0) must be bitwise one of the explicit widths; without hints (one
launch) the setting must have no effect at all.
"""
import numpy as np
import pytest

from oracle import lapack_oracle as lo
from tokura_zgeev_batched_gb300 import api
from tokura_zgeev_batched_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def solve(A, n, qr_lanes, hints=1, lanes=4):
    h = api.Handle()
    assert h.set_plain_config(n, lanes, 32) == 0
    assert h.set_plain_qr_lanes(n, qr_lanes) == 0
    assert h.set_shift_hints(hints) == 0
    w, f = api.zgeev_batched(A, handle=h)
    return w, f


@pytest.mark.parametrize("n", [16, 20, 33, 64])
def test_every_qr_width_matches_lapack(cuda, n):
    import torch

    A_np = wl.gaussian(999, n, seed=900 + n)  # 999: the last staging tile is partial at every width
    A = torch.from_numpy(A_np).cuda()
    results = {}
    for lq in (1, 2, 4, 8):
        w, f = solve(A, n, lq)
        results[lq] = (w, f)
        rep = lo.parity_report(A_np, w.cpu().numpy(), f.cpu().numpy())
        assert rep["flag_mismatch"] == 0 and (f.cpu().numpy() == 0).all(), (lq, rep["flag_mismatch"])
        assert rep["max_rel_err_well"] <= lo.TOL_REL_FRO, (lq, rep["max_rel_err_well"])
    w0, f0 = solve(A, n, 0)
    chosen = 2 if n <= 24 else 4  # the library's choice after a four-lane first launch
    assert torch.equal(w0, results[chosen][0]) and torch.equal(f0, results[chosen][1])


def test_qr_width_is_ignored_without_hints(cuda):
    import torch

    n = 20
    A = torch.from_numpy(wl.gaussian(500, n, seed=77)).cuda()
    w1, f1 = solve(A, n, 1, hints=0)
    w8, f8 = solve(A, n, 8, hints=0)
    assert torch.equal(w1, w8) and torch.equal(f1, f8)


def test_setter_validates(cuda):
    h = api.Handle()
    assert h.set_plain_qr_lanes(0, 2) == -2
    assert h.set_plain_qr_lanes(65, 2) == -2
    assert h.set_plain_qr_lanes(16, 3) == -3
    assert h.set_plain_qr_lanes(16, 64) == -3
    assert h.set_plain_qr_lanes(16, 32) == 0
    assert h.set_plain_qr_lanes(16, 0) == 0
