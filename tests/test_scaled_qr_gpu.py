"""QR with scaled rotations (tokuraSetScaledRotations): parity with LAPACK at every lane width,
with shift hints on and off, on the golden fixtures (structured matrices: zeros, Jordan blocks,
circulants, huge and tiny scalings), against the plain rotations, and the sweep cap."""
import os

import numpy as np
import pytest

from oracle import lapack_oracle as lo
from tokura_zgeev_batched_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "zgeev_golden.npz")


def solve(A_np, min_order=1, hints=1, lanes=0, cap=0):
    import torch
    from tokura_zgeev_batched_gb300 import api

    h = api.Handle()
    assert h.set_scaled_rotations(min_order) == 0
    assert h.set_shift_hints(hints) == 0
    n = A_np.shape[-1]
    if lanes:
        assert h.set_plain_config(n, lanes, 64) == 0
    if cap:
        assert h.set_sweep_cap(cap) == 0
    A = torch.from_numpy(np.ascontiguousarray(A_np)).cuda()
    w, f = api.zgeev_batched(A, handle=h)
    torch.cuda.synchronize()
    return w.cpu().numpy(), f.cpu().numpy()


def test_setter_validation(cuda):
    from tokura_zgeev_batched_gb300 import api

    h = api.Handle()
    assert h.set_scaled_rotations(1) == 0 and h.set_scaled_rotations(64) == 0 and h.set_scaled_rotations(65) == 0
    assert h.set_scaled_rotations(0) == -2 and h.set_scaled_rotations(66) == -2


@pytest.mark.parametrize("lanes", [1, 2, 4, 8, 16, 32])
@pytest.mark.parametrize("n", [7, 8, 13, 24, 32, 47, 64])
def test_gaussian_every_lane_width(cuda, n, lanes):
    A = wl.gaussian(256, n, seed=3100 + n + lanes)
    for hints in (0, 1):
        w, f = solve(A, hints=hints, lanes=lanes)
        rep = lo.parity_report(A, w, f)
        assert rep["flag_mismatch"] == 0 and (f == 0).all(), (hints, rep)
        assert rep["max_rel_err_well"] <= lo.TOL_REL_FRO, (hints, rep["max_rel_err_well"])


@pytest.mark.parametrize("cls", ["vdv", "companion", "uniform"])
@pytest.mark.parametrize("n", [16, 32, 64])
def test_classes(cuda, cls, n):
    A = wl.GENERATORS[cls](400, n, seed=3300 + n)
    w, f = solve(A)
    rep = lo.parity_report(A, w, f)
    assert rep["flag_mismatch"] == 0, rep
    if rep["well_conditioned"]:
        assert rep["max_rel_err_well"] <= lo.TOL_REL_FRO, rep["max_rel_err_well"]


@pytest.mark.parametrize("lanes", [1, 4])
def test_golden_fixtures(cuda, lanes):
    golden = np.load(GOLDEN)
    for name in [str(x) for x in golden["names"]]:
        A = golden[f"{name}/A"]
        if A.shape[-1] < 7:
            continue
        w, f = solve(A, lanes=lanes)
        info = golden[f"{name}/info"]
        assert np.array_equal(f != 0, info != 0), name
        fro = np.sqrt(np.sum(np.abs(A) ** 2, axis=(1, 2)))
        fro = np.where(fro == 0, 1.0, fro)
        cond = 1.0 / np.maximum(golden[f"{name}/rconde"], 1e-300)
        err = lo.matched_abs_errors(w, golden[f"{name}/w"]).max(axis=1) / fro
        well = cond.max(axis=1) <= lo.COND_MAX
        assert np.all(err[well] <= lo.TOL_REL_FRO), (name, err)


def test_matches_plain_rotations(cuda):
    """Same eigenvalues as the plain rotations to the parity tolerance (not bitwise)."""
    A = wl.gaussian(500, 48, seed=3400)
    w_s, f_s = solve(A, min_order=1)
    w_p, f_p = solve(A, min_order=65)
    assert (f_s == 0).all() and (f_p == 0).all()
    fro = np.linalg.norm(A, axis=(1, 2))
    err = lo.matched_abs_errors(w_s, w_p).max(axis=1) / fro
    assert err.max() <= lo.TOL_REL_FRO, err.max()


def test_badly_scaled_entries(cuda):
    """Entries spread over many binades (D B D^-1, D = 2^U{-20..20}): scale factors and the
    rescaling keep full accuracy with balancing."""
    import torch
    from tokura_zgeev_batched_gb300 import api

    rng = np.random.default_rng(3500)
    n, batch = 40, 200
    B = wl.gaussian(batch, n, seed=3501)
    d = 2.0 ** rng.integers(-20, 21, size=(batch, n))
    A = d[:, :, None] * B / d[:, None, :]
    h = api.Handle()
    assert h.set_scaled_rotations(1) == 0 and h.set_balancing(3) == 0
    w, f = api.zgeev_batched(torch.from_numpy(A).cuda(), handle=h)
    w, f = w.cpu().numpy(), f.cpu().numpy()
    w_ref = lo.zgeev(B)[0]
    err = lo.matched_abs_errors(w, w_ref).max(axis=1) / np.linalg.norm(B, axis=(1, 2))
    assert (f == 0).all() and err.max() <= lo.TOL_REL_FRO, err.max()


def test_sweep_cap_sets_flag(cuda):
    A = wl.gaussian(64, 32, seed=3600)
    w, f = solve(A, cap=1)
    assert (f == 1).all()
    assert np.all(np.isfinite(w))


@pytest.mark.parametrize("lanes", [1, 4])
@pytest.mark.parametrize("n", [7, 24, 48])
def test_gradient_schur_scaled_and_plain(cuda, n, lanes):
    """The backward's Schur recomputation with scaled rotations gives torch's gradient, as
    the plain rotations do."""
    import torch

    from tokura_zgeev_batched_gb300 import api
    from tokura_zgeev_batched_gb300.autograd import eigvals

    A_np = wl.vdv(24, n, seed=3700 + n, min_sep=0.05)
    Ac = torch.from_numpy(A_np).clone().requires_grad_(True)
    lam = torch.linalg.eigvals(Ac)
    torch.sum(torch.exp(lam.real) + lam.real ** 2 + lam.imag ** 2).backward()
    ref = Ac.grad.numpy()
    for min_order in (1, 65):
        h = api.Handle()
        assert h.set_scaled_rotations(min_order) == 0 and h.set_plain_config(n, lanes, 64) == 0
        A = torch.from_numpy(A_np).cuda().requires_grad_(True)
        lam_g, flag = eigvals(A, handle=h, return_flag=True)
        torch.sum(torch.exp(lam_g.real) + lam_g.real ** 2 + lam_g.imag ** 2).backward()
        g = A.grad.cpu().numpy()
        assert (flag.cpu().numpy() == 0).all()
        err = np.linalg.norm(g - ref, axis=(1, 2)) / np.linalg.norm(ref, axis=(1, 2))
        assert err.max() < 1e-9, (min_order, err.max())


@pytest.mark.parametrize("n", [9, 33, 64])
def test_eigenvectors_scaled_and_plain(cuda, n):
    import torch

    from tokura_zgeev_batched_gb300 import api

    M = wl.gaussian(24, n, seed=3800 + n)
    fro = np.linalg.norm(M, axis=(1, 2))
    for min_order in (1, 65):
        h = api.Handle()
        assert h.set_scaled_rotations(min_order) == 0
        w, VL, VR, f = api.zgeev_vectors(torch.from_numpy(M).cuda(), handle=h)
        w, VL, VR, f = w.cpu().numpy(), VL.cpu().numpy(), VR.cpu().numpy(), f.cpu().numpy()
        assert (f == 0).all()
        for k in range(M.shape[0]):
            assert np.abs(M[k] @ VR[k] - VR[k] * w[k][None, :]).max() <= 1e-12 * n * fro[k]
            assert np.abs(VL[k].conj().T @ M[k] - w[k][:, None] * VL[k].conj().T).max() <= 1e-12 * n * fro[k]
            assert np.allclose(np.linalg.norm(VR[k], axis=0), 1.0, atol=1e-13)
