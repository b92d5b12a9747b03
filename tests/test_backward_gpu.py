"""Differentiable mode: backward kernel vs torch.linalg.eigvals backward (CPU, FP64) and central differences."""
import numpy as np
import pytest

from tokura_zgeev_batched_gb300 import api
from tokura_zgeev_batched_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def loss_fn(lam):
    import torch

    return torch.sum(torch.exp(lam.real) + lam.real ** 2 + lam.imag ** 2)


def torch_cpu_grad(A_np):
    import torch

    A = torch.from_numpy(A_np).clone().requires_grad_(True)
    L = loss_fn(torch.linalg.eigvals(A))
    L.backward()
    return A.grad.numpy()


def our_grad(A_np, lanes=0):
    import torch

    from tokura_zgeev_batched_gb300.autograd import eigvals

    h = api.Handle()
    if lanes:
        assert h.set_plain_config(A_np.shape[-1], lanes, 128) == 0
    A = torch.from_numpy(A_np).cuda().requires_grad_(True)
    lam, flag = eigvals(A, handle=h, return_flag=True)
    L = loss_fn(lam)
    L.backward()
    return A.grad.cpu().numpy(), flag.cpu().numpy()


@pytest.mark.parametrize("n", [1, 2, 5, 16, 48])
@pytest.mark.parametrize("lanes", [1, 2, 4, 8])
def test_matches_torch_eigvals_backward(cuda, n, lanes):
    A = wl.vdv(24, n, seed=300 + n, min_sep=0.05)
    g_ref = torch_cpu_grad(A)
    g, flag = our_grad(A, lanes)
    assert (flag == 0).all()
    err = np.linalg.norm(g - g_ref, axis=(1, 2)) / np.maximum(np.linalg.norm(g_ref, axis=(1, 2)), 1e-300)
    assert err.max() < 1e-9, err.max()


def test_central_differences(cuda):
    import torch

    rng = np.random.default_rng(5)
    for n in (16, 48):
        A = wl.vdv(2, n, seed=77 + n, min_sep=0.05)
        g, flag = our_grad(A)
        assert (flag == 0).all()
        h = 1e-6
        for k in range(2):
            for _ in range(16):  # 16 entries x (Re, Im) x 2 matrices x 2 sizes = 64 entries per part
                i, j = rng.integers(0, n, 2)
                for part, unit in (("re", 1.0), ("im", 1j)):
                    Ap = A[k].copy()
                    Am = A[k].copy()
                    Ap[i, j] += h * unit
                    Am[i, j] -= h * unit
                    Lp = float(loss_fn(torch.linalg.eigvals(torch.from_numpy(Ap))))
                    Lm = float(loss_fn(torch.linalg.eigvals(torch.from_numpy(Am))))
                    fd = (Lp - Lm) / (2 * h)
                    ours = g[k, i, j].real if part == "re" else g[k, i, j].imag
                    assert abs(fd - ours) <= 1e-6 * max(1.0, abs(fd)), (n, k, i, j, part, fd, ours)


def test_backward_flags(cuda):
    import torch

    A = wl.vdv(6, 8, seed=9, min_sep=0.05)
    A[1, 2, 3] = np.nan
    A[2] = 0.0
    A[3] = np.diag(np.array([1, 1, 2, 3, 4, 5, 6, 7], np.complex128))  # repeated eigenvalue
    At = torch.from_numpy(A).cuda()
    lam, f = api.zgeev_batched(At)
    g = torch.ones_like(lam)
    gA, flag = api.zgeev_backward(At, lam, g)
    flag = flag.cpu().numpy()
    gA = gA.cpu().numpy()
    assert flag[1] == 2 and np.isnan(gA[1]).all()
    assert flag[2] == 4 and flag[3] == 4
    assert flag[0] == 0 and flag[4] == 0 and flag[5] == 0
    assert np.isfinite(gA[3]).all()


def test_ragged_backward_matches_torch(cuda):
    import torch

    from tokura_zgeev_batched_gb300.autograd import eigvals_ragged

    rng = np.random.default_rng(4)
    ns = rng.integers(1, 40, 60).astype(np.int32)
    mats = [wl.vdv(1, int(k), seed=1000 + j, min_sep=0.05)[0] for j, k in enumerate(ns)]
    buf, ns, offs, eoffs = wl.pack_ragged(mats)
    A = torch.from_numpy(buf).cuda().requires_grad_(True)
    lam = eigvals_ragged(A, torch.from_numpy(ns).cuda())
    L = loss_fn(lam)
    L.backward()
    g = A.grad.cpu().numpy()
    for j, m in enumerate(mats):
        k = m.shape[0]
        g_ref = torch_cpu_grad(m[None])[0]
        gj = g[offs[j]:offs[j] + k * k].reshape(k, k)
        assert np.linalg.norm(gj - g_ref) <= 1e-9 * max(np.linalg.norm(g_ref), 1.0), (j, k)


@pytest.mark.parametrize("lanes", [0, 1, 2, 4, 8])
def test_ragged_backward_large_shifted(cuda, lanes):
    """n up to 64, spectra shifted by +0.5 (the optimisation-loop construction), each lane width."""
    import torch

    from tokura_zgeev_batched_gb300.autograd import eigvals_ragged

    rng = np.random.default_rng(40 + lanes)
    ns = rng.integers(8, 65, 24).astype(np.int32)
    mats = [wl.vdv(1, int(k), seed=2000 + j, min_sep=0.05, shift=0.5)[0] for j, k in enumerate(ns)]
    buf, ns, offs, eoffs = wl.pack_ragged(mats)
    h = api.Handle()
    assert h.set_ragged_lanes(lanes) == 0
    A = torch.from_numpy(buf).cuda().requires_grad_(True)
    lam = eigvals_ragged(A, torch.from_numpy(ns).cuda(), handle=h)
    seg = torch.repeat_interleave(torch.arange(len(ns), device="cuda"), torch.from_numpy(ns).cuda().long())
    tau = 0.05
    x = lam.real / tau
    m = torch.full((len(ns),), -float("inf"), dtype=torch.float64, device="cuda").scatter_reduce(
        0, seg, x.detach(), reduce="amax")
    ssum = torch.zeros(len(ns), dtype=torch.float64, device="cuda").index_add(0, seg, torch.exp(x - m[seg]))
    loss = (tau * (torch.log(ssum) + m)).sum()
    (g,) = torch.autograd.grad(loss, A)
    g = g.cpu().numpy()
    for j, mtx in enumerate(mats):
        k = mtx.shape[0]
        At = torch.from_numpy(mtx).clone().requires_grad_(True)
        lt = torch.linalg.eigvals(At)
        (tau * torch.logsumexp(lt.real / tau, 0)).backward()
        ref = At.grad.numpy()
        gj = g[offs[j]:offs[j] + k * k].reshape(k, k)
        assert np.linalg.norm(gj - ref) <= 1e-8 * max(np.linalg.norm(ref), 1.0), (j, k, lanes)


def test_gradient_descent_loop_matches_torch_cpu(cuda):
    """Ten steps of the smoothed-abscissa descent: GPU ragged fwd+bwd loop vs the same loop in torch on the CPU."""
    import torch

    from tokura_zgeev_batched_gb300.autograd import eigvals_ragged

    rng = np.random.default_rng(8)
    ns = rng.integers(8, 30, 12).astype(np.int32)
    mats = [wl.vdv(1, int(k), seed=3000 + j, min_sep=0.05, shift=0.5)[0] for j, k in enumerate(ns)]
    buf, ns, offs, eoffs = wl.pack_ragged(mats)
    tau, lr, steps = 0.05, 1e-2, 10
    n_d = torch.from_numpy(ns).cuda()
    seg = torch.repeat_interleave(torch.arange(len(ns), device="cuda"), n_d.long())
    A = torch.from_numpy(buf).cuda().requires_grad_(True)
    for _ in range(steps):
        lam = eigvals_ragged(A, n_d)
        x = lam.real / tau
        m = torch.full((len(ns),), -float("inf"), dtype=torch.float64, device="cuda").scatter_reduce(
            0, seg, x.detach(), reduce="amax")
        s = torch.zeros(len(ns), dtype=torch.float64, device="cuda").index_add(0, seg, torch.exp(x - m[seg]))
        (g,) = torch.autograd.grad((tau * (torch.log(s) + m)).sum(), A)
        with torch.no_grad():
            A.sub_(lr * g)
    gpu = A.detach().cpu().numpy()
    for j, mtx in enumerate(mats):
        k = mtx.shape[0]
        # The library sees the buffer column-major, i.e. the matrix mtx^T; eigenvalues agree and the
        # gradient of the buffer is the gradient w.r.t. mtx in row-major order.
        X = torch.from_numpy(mtx.copy()).requires_grad_(True)
        for _ in range(steps):
            lt = torch.linalg.eigvals(X)
            (gx,) = torch.autograd.grad(tau * torch.logsumexp(lt.real / tau, 0), X)
            with torch.no_grad():
                X.sub_(lr * gx)
        got = gpu[offs[j]:offs[j] + k * k].reshape(k, k)
        assert np.abs(got - X.detach().numpy()).max() <= 1e-9 * max(1.0, np.abs(mtx).max()), (j, k)
