"""Balancing (tokuraSetBalancing): permutation isolation and power-of-two scaling.

The reference never balances (README.md:79); LAPACK zgeev does (zgebal,
JOB='B'). Checks: badly scaled similarity transforms D B D^-1 are solved to
the accuracy of B only with scaling on; eigenvalues isolated by the
permutation come back bit-exact; mode 0 is bit-identical to a fresh handle;
every mode keeps LAPACK parity on ordinary matrices and on the ragged,
host-buffer and workspace-free entry points.
"""
import numpy as np
import pytest

from oracle import lapack_oracle as lo
from tokura_zgeev_batched_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def scaled_similar(batch, n, spread, seed):
    """A_k = D_k B_k D_k^-1 with D_k = diag(2^e), e uniform in [-spread, spread]; returns (A, B)."""
    rng = np.random.default_rng(seed)
    B = wl.gaussian(batch, n, seed=seed + 1)
    e = rng.integers(-spread, spread + 1, size=(batch, n)).astype(np.float64)
    d = np.exp2(e)
    A = B * d[:, :, None] / d[:, None, :]
    return np.ascontiguousarray(A), B


def isolated_blocks(batch, n, top, bottom, seed):
    """P^T [[T1 X Y], [0 B Z], [0 0 T2]] P with upper-triangular T1 (top x top)
    and T2 (bottom x bottom); returns (A, planted diagonal eigenvalues)."""
    rng = np.random.default_rng(seed)
    A = np.empty((batch, n, n), np.complex128)
    planted = []
    for k in range(batch):
        M = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        M[top:, :top] = 0.0
        M[n - bottom:, : n - bottom] = 0.0
        M[:top, :top] = np.triu(M[:top, :top])
        M[n - bottom:, n - bottom:] = np.triu(M[n - bottom:, n - bottom:])
        p = rng.permutation(n)
        A[k] = M[np.ix_(p, p)]
        planted.append(np.concatenate([np.diag(M)[:top], np.diag(M)[n - bottom:]]))
    return A, planted


def solve(A_np, mode, handle=None):
    import torch
    from tokura_zgeev_batched_gb300 import api

    h = handle if handle is not None else api.Handle()
    assert h.set_balancing(mode) == 0
    # torch tensors are row-major: pass the column-major buffer of A (= A^T
    # row-major), so the kernel sees exactly A.
    At = torch.from_numpy(np.ascontiguousarray(np.swapaxes(A_np, -1, -2))).cuda()
    w, f = api.zgeev_batched(At, handle=h)
    torch.cuda.synchronize()
    return w.cpu().numpy(), f.cpu().numpy()


def max_matched_err(w, w_ref):
    return max(float(lo.matched_abs_errors(w[k], w_ref[k]).max()) for k in range(len(w)))


def test_set_balancing_validation(cuda):
    from tokura_zgeev_batched_gb300 import api

    h = api.Handle()
    for m in range(4):
        assert h.set_balancing(m) == 0
    assert h.set_balancing(-1) == -2
    assert h.set_balancing(4) == -2


@pytest.mark.parametrize("n", [8, 16, 32, 64])
def test_scaling_recovers_badly_scaled(cuda, n):
    A, B = scaled_similar(64, n, spread=20, seed=300 + n)
    w_ref, info, _ = lo.zgeev(B)  # eigenvalues of B, computed on the well-scaled matrix
    assert (info == 0).all()
    nb = np.linalg.norm(B, axis=(1, 2)).max()
    w3, f3 = solve(A, 3)
    w2, f2 = solve(A, 2)
    w0, f0 = solve(A, 0)
    assert (f3 == 0).all() and (f2 == 0).all()
    e3, e2 = max_matched_err(w3, w_ref), max_matched_err(w2, w_ref)
    assert e3 <= 1e-11 * nb, e3
    assert e2 <= 1e-11 * nb, e2
    # Without balancing the error grows with ||A||, which is ~2^40 ||B|| here.
    if (f0 == 0).all():
        e0 = max_matched_err(w0, w_ref)
        assert e0 > 100 * e3, (e0, e3)


@pytest.mark.parametrize("n,top,bottom", [(6, 2, 1), (16, 3, 4), (33, 5, 0), (64, 0, 7), (64, 10, 10), (5, 2, 3)])
@pytest.mark.parametrize("mode", [1, 3])
def test_permutation_isolates_exactly(cuda, n, top, bottom, mode):
    A, planted = isolated_blocks(40, n, top, bottom, seed=17 * n + top)
    w, f = solve(A, mode)
    assert (f == 0).all()
    w_ref = lo.zgeev(A)[0]
    na = np.linalg.norm(A, axis=(1, 2)).max()
    assert max_matched_err(w, w_ref) <= 1e-11 * na
    for k in range(len(A)):
        got = set(w[k].tolist())
        for lam in planted[k]:
            assert lam in got, (k, lam)  # bit-exact: isolated entries are never touched


def test_mode0_bitwise_default(cuda):
    from tokura_zgeev_batched_gb300 import api

    A = wl.gaussian(256, 24, seed=5)
    w_default, f_default = solve(A, 0, handle=api.Handle())
    h = api.Handle()
    h.set_balancing(3)
    h.set_balancing(0)
    w0, f0 = solve(A, 0, handle=h)
    assert np.array_equal(w0.view(np.uint64), w_default.view(np.uint64))
    assert np.array_equal(f0, f_default)


@pytest.mark.parametrize("mode", [1, 2, 3])
@pytest.mark.parametrize("cls", ["gaussian", "vdv", "companion"])
def test_modes_keep_parity(cuda, mode, cls):
    n = 32
    A = wl.GENERATORS[cls](128, n, seed=41)
    w, f = solve(A, mode)
    rep = lo.parity_report(A, w, f)
    assert rep["flag_mismatch"] == 0, rep
    if rep["well_conditioned"]:
        assert rep["max_rel_err_well"] <= lo.TOL_REL_FRO, {k: v for k, v in rep.items() if k != "rel_err"}


@pytest.mark.parametrize("lanes", [0, 1, 4])
def test_ragged_balanced(cuda, lanes):
    import torch
    from tokura_zgeev_batched_gb300 import api

    rng = np.random.default_rng(9)
    mats, refs = [], []
    for k, n in enumerate(rng.integers(1, 65, size=150)):
        A, B = scaled_similar(1, int(n), spread=16, seed=1000 + k)
        mats.append(np.ascontiguousarray(A[0].T).reshape(n, n))  # column-major buffer of A
        refs.append(B[0])
    buf, ns, offs, eoffs = wl.pack_ragged(mats)
    h = api.Handle()
    assert h.set_balancing(3) == 0
    assert h.set_ragged_lanes(lanes) == 0
    eig, flag = api.zgeev_ragged(torch.from_numpy(buf).cuda(), torch.from_numpy(ns).cuda(), handle=h)
    torch.cuda.synchronize()
    eig, flag = eig.cpu().numpy(), flag.cpu().numpy()
    assert (flag == 0).all()
    for k, B in enumerate(refs):
        n = B.shape[0]
        w_ref = lo.zgeev(B[None])[0]
        got = eig[eoffs[k]: eoffs[k] + n]
        err = float(lo.matched_abs_errors(got, w_ref[0]).max())
        assert err <= 1e-11 * np.linalg.norm(B), (k, n, err)


def test_host_and_noalloc_balanced(cuda):
    import torch
    from tokura_zgeev_batched_gb300 import api

    A, B = scaled_similar(96, 20, spread=20, seed=77)
    w_ref = lo.zgeev(B)[0]
    nb = np.linalg.norm(B, axis=(1, 2)).max()
    h = api.Handle()
    assert h.set_balancing(3) == 0
    At = np.ascontiguousarray(np.swapaxes(A, -1, -2))
    w_host, f_host = api.zgeev_batched_host(At, handle=h, chunk_matrices=32)
    assert (np.asarray(f_host) == 0).all()
    assert max_matched_err(np.asarray(w_host), w_ref) <= 1e-11 * nb

    Ad = torch.from_numpy(At).cuda()
    eig = torch.empty(96, 20, dtype=torch.complex128, device="cuda")
    flag = torch.empty(96, dtype=torch.int8, device="cuda")
    st = api.tokura_zgeev_batched_gpu_noalloc(h, 20, 96, Ad.data_ptr(), eig.data_ptr(), flag.data_ptr(),
                                              torch.cuda.current_stream().cuda_stream)
    assert st == 0
    torch.cuda.synchronize()
    assert (flag.cpu().numpy() == 0).all()
    assert max_matched_err(eig.cpu().numpy(), w_ref) <= 1e-11 * nb
