"""Eigenvectors (ZGEEV with JOBVL/JOBVR = 'V') against LAPACK zgeev('V','V') and residual checks."""
import numpy as np
import pytest

from oracle import lapack_oracle as lo
from tokura_zgeev_batched_gb300 import api
from tokura_zgeev_batched_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def run(M, left=True, right=True, lanes=0):
    import torch

    h = api.Handle()
    if lanes:
        assert h.set_plain_config(M.shape[-1], lanes, 128) == 0
    w, VL, VR, f = api.zgeev_vectors(torch.from_numpy(M).cuda(), left=left, right=right, handle=h)
    torch.cuda.synchronize()
    return (w.cpu().numpy(), None if VL is None else VL.cpu().numpy(), None if VR is None else VR.cpu().numpy(),
            f.cpu().numpy())


@pytest.mark.parametrize("n", [1, 2, 5, 16, 33, 64])
@pytest.mark.parametrize("cls", ["gaussian", "vdv"])
def test_vectors_match_lapack(cuda, n, cls):
    M = wl.GENERATORS[cls](12, n, seed=600 + n)
    w, VL, VR, f = run(M)
    assert (f == 0).all()
    # LAPACK on the same logical matrices (buffers are read column-major, so pass M^T)
    wr, VLr, VRr, info = lo.zgeev_vectors(np.ascontiguousarray(M.transpose(0, 2, 1)))
    assert (info == 0).all()
    fro = np.sqrt(np.sum(np.abs(M) ** 2, axis=(1, 2)))
    _, rc, _ = lo.zgeevx_rconde(np.ascontiguousarray(M.transpose(0, 2, 1)))
    for k in range(M.shape[0]):
        # residuals and normalization
        assert np.abs(M[k] @ VR[k] - VR[k] * w[k][None, :]).max() <= 1e-12 * n * fro[k]
        assert np.abs(VL[k].conj().T @ M[k] - w[k][:, None] * VL[k].conj().T).max() <= 1e-12 * n * fro[k]
        for V in (VL[k], VR[k]):
            assert np.allclose(np.linalg.norm(V, axis=0), 1.0, atol=1e-13)
            top = V[np.argmax(np.abs(V), axis=0), np.arange(n)]
            assert np.all(top.real > 0) and np.all(np.abs(top.imag) <= 1e-15)
        # same vectors as LAPACK, up to the phase convention, for well-separated eigenvalues
        err = lo.matched_abs_errors(w[k][None], wr[k][None])[0]
        assert err.max() <= lo.TOL_REL_FRO * fro[k]
        order = [int(np.argmin(np.abs(w[k] - x))) for x in wr[k]]
        cond = 1.0 / rc[k]
        for i_ref, i in enumerate(order):
            if cond[i_ref] > 1e3:
                continue
            for ours, ref in ((VR[k][:, i], VRr[k][:, i_ref]), (VL[k][:, i], VLr[k][:, i_ref])):
                overlap = abs(np.vdot(ref, ours))
                assert overlap >= 1 - 1e-9, (k, i, overlap)


@pytest.mark.parametrize("lanes", [1, 2, 4, 8])
def test_vectors_lane_widths_and_optional_outputs(cuda, lanes):
    M = wl.gaussian(40, 20, seed=9)
    w, VL, VR, f = run(M, left=False, right=True, lanes=lanes)
    assert VL is None and (f == 0).all()
    for k in range(40):
        assert np.abs(M[k] @ VR[k] - VR[k] * w[k][None, :]).max() <= 1e-11
    w2, VL2, VR2, f2 = run(M, left=True, right=False, lanes=lanes)
    assert VR2 is None and np.abs(w2 - w).max() == 0.0


def test_vectors_nonfinite_flag(cuda):
    M = wl.gaussian(3, 6, seed=2)
    M[1, 0, 0] = np.nan
    w, VL, VR, f = run(M)
    assert list(f) == [0, 2, 0]
    assert np.isnan(VR[1]).all() and np.isfinite(VR[0]).all()
