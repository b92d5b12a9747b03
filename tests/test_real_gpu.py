"""Real-input path (tokura_dgeev_batched_gpu / tokura_sgeev_batched_gpu).

Oracle: LAPACK dgeev('N','N') on the same matrices. Checks parity within
1e-11 * ||A||_F on well-conditioned spectra, identical flags, and LAPACK's
output convention (conjugate pairs adjacent and exact, positive imaginary
part first, real eigenvalues with wi exactly 0).
"""
import numpy as np
import pytest

from oracle import lapack_oracle as lo

pytestmark = pytest.mark.gpu

TOL = lo.TOL_REL_FRO  # 1e-11, relative to ||A||_F


def real_gaussian(batch, n, seed):
    return np.random.default_rng(seed).standard_normal((batch, n, n))


def real_companion(batch, n, seed):
    rng = np.random.default_rng(seed)
    C = np.zeros((batch, n, n))
    C[:, 0, :] = -rng.standard_normal((batch, n))
    if n > 1:
        C[:, np.arange(1, n), np.arange(n - 1)] = 1.0
    return C


def real_spectrum(batch, n, seed):
    """V diag(lam) V^-1 with real lam and V = I + 0.3 G (real eigenvalues)."""
    rng = np.random.default_rng(seed)
    lam = rng.uniform(-1, 1, (batch, n))
    V = np.eye(n) + 0.3 * rng.standard_normal((batch, n, n))
    return np.einsum("bij,bj,bjk->bik", V, lam, np.linalg.inv(V))


def solve(A_np, handle=None, dtype="float64"):
    """Runs the GPU path on the column-major buffers A_np[k] (as LAPACK reads them)."""
    import torch
    from tokura_zgeev_batched_gb300 import api

    # torch is row-major: the row-major tensor A^T has A's column-major buffer,
    # and dgeev_batched reads exactly that buffer.
    t = torch.from_numpy(np.ascontiguousarray(A_np)).cuda()
    if dtype == "float32":
        t = t.float()
    wr, wi, f = api.dgeev_batched(t, handle=handle)
    torch.cuda.synchronize()
    return wr.cpu().numpy(), wi.cpu().numpy(), f.cpu().numpy()


def check(A, wr, wi, f):
    rep = lo.real_parity_report(A, wr, wi, f)
    assert rep["flag_mismatch"] == 0, rep
    assert rep["pairs_ok"], "conjugate-pair convention violated"
    assert rep["well_conditioned"] > 0
    assert rep["max_rel_err_well"] <= TOL, rep["max_rel_err_well"]
    return rep


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 7, 8, 13, 16, 23, 31, 32, 33, 48, 63, 64])
def test_gaussian_all_sizes(cuda, n):
    A = real_gaussian(300, n, seed=500 + n)
    wr, wi, f = solve(A)
    assert (f == 0).all()
    check(A, wr, wi, f)


@pytest.mark.parametrize("gen", [real_companion, real_spectrum])
@pytest.mark.parametrize("n", [4, 16, 32, 64])
def test_classes(cuda, gen, n):
    A = gen(200, n, seed=9 * n)
    wr, wi, f = solve(A)
    rep = lo.real_parity_report(A, wr, wi, f)
    assert rep["flag_mismatch"] == 0, rep
    assert rep["pairs_ok"]
    if rep["well_conditioned"]:
        assert rep["max_rel_err_well"] <= TOL, rep["max_rel_err_well"]


def test_known_answers(cuda):
    rot = np.array([[0.0, -1.0], [1.0, 0.0]])  # eigenvalues +-i exactly
    wr, wi, f = solve(rot[None])
    assert f[0] == 0
    assert wr[0].tolist() == [0.0, 0.0] and wi[0].tolist() == [1.0, -1.0]
    # upper triangular T (column-major buffer = C-order T^T): the diagonal comes back exactly
    T = np.triu(np.random.default_rng(1).standard_normal((20, 20)))
    wr, wi, f = solve(np.ascontiguousarray(T.T)[None])
    assert sorted(wr[0].tolist()) == sorted(np.diag(T).tolist())
    assert (wi == 0).all()
    # companion matrix of (x-1)(x-2)(x-3)
    c = np.poly([1.0, 2.0, 3.0])  # [1, -6, 11, -6]
    C = np.zeros((3, 3))
    C[0, :] = -c[1:]
    C[1, 0] = C[2, 1] = 1.0
    wr, wi, f = solve(np.ascontiguousarray(C.T)[None])
    assert np.allclose(sorted(wr[0]), [1.0, 2.0, 3.0], atol=1e-12) and (wi == 0).all()


def test_symmetric_real_spectrum(cuda):
    A = real_gaussian(200, 24, seed=3)
    A = A + np.swapaxes(A, 1, 2)
    wr, wi, f = solve(A)
    assert (f == 0).all()
    fro = np.linalg.norm(A, axis=(1, 2))
    assert (np.abs(wi).max(axis=1) <= TOL * fro).all()
    check(A, wr, wi, f)


def test_edge_inputs(cuda):
    A = real_gaussian(6, 9, seed=4)
    A[1] = 0.0
    A[2, 3, 4] = np.nan
    A[3, 0, 0] = np.inf
    A[4] = A[0] * 2.0 ** 300  # exact power-of-two pre-scaling
    A[5] = A[0] * 2.0 ** -300
    wr, wi, f = solve(A)
    assert f.tolist() == [0, 0, 2, 2, 0, 0]
    assert (wr[1] == 0).all() and (wi[1] == 0).all()
    assert np.isnan(wr[2]).all() and np.isnan(wi[3]).all()
    ref = A[0]
    w0 = wr[0] + 1j * wi[0]
    fro0 = np.linalg.norm(A[0])
    for k, s in ((4, 2.0 ** 300), (5, 2.0 ** -300)):
        wk = (wr[k] + 1j * wi[k]) / s
        assert lo.matched_abs_errors(wk, w0).max() <= 1e-13 * fro0, k
    check(ref[None], wr[0][None], wi[0][None], f[0][None])


def test_sweep_cap_flags(cuda):
    from tokura_zgeev_batched_gb300 import api

    h = api.Handle()
    assert h.set_sweep_cap(1) == 0
    A = real_gaussian(64, 32, seed=6)
    _, _, f = solve(A, handle=h)
    assert (f == 1).any()
    assert set(f.tolist()) <= {0, 1}


@pytest.mark.parametrize("lanes", [1, 2, 4, 8])
def test_lane_widths(cuda, lanes):
    from tokura_zgeev_batched_gb300 import api

    h = api.Handle()
    for n in (5, 17, 40, 64):
        assert h.set_real_config(n, lanes, 128) == 0
        A = real_gaussian(97, n, seed=lanes * 100 + n)
        wr, wi, f = solve(A, handle=h)
        assert (f == 0).all()
        check(A, wr, wi, f)


def test_float32_is_rounded_fp64(cuda):
    A = real_gaussian(256, 20, seed=8).astype(np.float32)
    wr32, wi32, f32 = solve(A, dtype="float32")
    assert wr32.dtype == np.float32
    wr, wi, f = solve(A.astype(np.float64))
    assert np.array_equal(wr32, wr.astype(np.float32)) and np.array_equal(wi32, wi.astype(np.float32))
    assert np.array_equal(f32, f)


def test_balancing_real(cuda):
    from tokura_zgeev_batched_gb300 import api

    rng = np.random.default_rng(12)
    n = 24
    B = rng.standard_normal((64, n, n))
    d = np.exp2(rng.integers(-20, 21, size=(64, n)).astype(np.float64))
    A = B * d[:, :, None] / d[:, None, :]
    h = api.Handle()
    assert h.set_balancing(3) == 0
    wr, wi, f = solve(A, handle=h)
    assert (f == 0).all()
    wr_ref, wi_ref, _, _ = lo.dgeev(B)
    nb = np.linalg.norm(B, axis=(1, 2)).max()
    err = max(float(lo.matched_abs_errors(wr[k] + 1j * wi[k], wr_ref[k] + 1j * wi_ref[k]).max()) for k in range(64))
    assert err <= TOL * nb, err
    assert lo.check_conjugate_pairs(wr, wi)


def test_real_path_agrees_with_complex_path(cuda):
    """The same real matrices through the complex entry point: same spectrum."""
    import torch
    from tokura_zgeev_batched_gb300 import api

    A = real_gaussian(128, 30, seed=13)
    wr, wi, f = solve(A)
    t = torch.from_numpy(A).to(torch.complex128).cuda()
    w, fz = api.zgeev_batched(t)
    w = w.cpu().numpy()
    fro = np.linalg.norm(A, axis=(1, 2))
    err = np.array([lo.matched_abs_errors(wr[k] + 1j * wi[k], w[k]).max() for k in range(128)])
    assert (err <= 1e-11 * fro).all()


def test_golden_real_cases(cuda):
    """GPU results against the committed real fixtures (tests/golden/make_golden_real.py):
    LAPACK dgeev's stored outputs and the exact spectra, identical flags, LAPACK's pair convention."""
    import os

    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "dgeev_golden.npz"))
    for name in [str(x) for x in g["names"]]:
        A = g[f"{name}/A"]
        wr, wi, f = solve(A)
        assert np.array_equal(f != 0, g[f"{name}/info"] != 0), name
        ok = f == 0
        assert lo.check_conjugate_pairs(wr[ok], wi[ok]), name
        fro = np.linalg.norm(A, axis=(1, 2))
        fro = np.where(fro == 0, 1.0, fro)
        cond = 1.0 / np.maximum(g[f"{name}/rconde"], 1e-300)
        well = cond.max(axis=1) <= lo.COND_MAX
        w = wr + 1j * wi
        err = lo.matched_abs_errors(w, g[f"{name}/wr"] + 1j * g[f"{name}/wi"]).max(axis=1) / fro
        assert np.all(err[well] <= TOL), (name, err)
        key = f"{name}/exact"
        if key in g.files:
            e = lo.matched_abs_errors(w, g[key]).max(axis=1) / fro
            assert np.all(e[well] <= TOL), (name, e)
