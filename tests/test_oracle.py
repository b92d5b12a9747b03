"""The oracle (LAPACK zgeev via oracle/cpu_zgeev.c) pinned against known answers and the golden fixtures."""
import os

import numpy as np
import pytest

from oracle import lapack_oracle as lo

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "zgeev_golden.npz")


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def cases(g):
    return [str(x) for x in g["names"]]


def test_oracle_reproduces_golden(golden):
    for name in cases(golden):
        A = golden[f"{name}/A"]
        w, info, _ = lo.zgeev(A, threads=2)
        assert np.array_equal(info, golden[f"{name}/info"]), name
        err = lo.matched_abs_errors(w, golden[f"{name}/w"])
        scale = np.maximum(np.sqrt(np.sum(np.abs(A) ** 2, axis=(1, 2))), 1e-300)
        assert np.all(err.max(axis=1) <= 1e-12 * scale + 1e-300) or name.startswith("jordan"), name


def test_oracle_known_answers(golden):
    # Exact spectra: triangular, diagonal, circulant, constructed V diag V^-1.
    for name in cases(golden):
        key = f"{name}/exact"
        if key not in golden.files:
            continue
        A = golden[f"{name}/A"]
        w, info, _ = lo.zgeev(A, threads=2)
        assert (info == 0).all(), name
        err = lo.matched_abs_errors(w, golden[key])
        fro = np.sqrt(np.sum(np.abs(A) ** 2, axis=(1, 2)))
        cond = 1.0 / np.maximum(golden[f"{name}/rconde"], 1e-300)
        bound = np.where(fro > 0, fro, 1.0) * 1e-13 * np.maximum(cond.max(axis=1), 1.0)
        if name.startswith("jordan"):
            # defective eigenvalue: LAPACK error ~ eps^(1/n)
            n = A.shape[-1]
            assert err.max() <= 10 * (2.2e-16 * fro.max()) ** (1.0 / n), name
        else:
            assert np.all(err.max(axis=1) <= bound), (name, err.max(axis=1), bound)


def test_matching_is_optimal():
    rng = np.random.default_rng(0)
    w = rng.standard_normal(8) + 1j * rng.standard_normal(8)
    perm = rng.permutation(8)
    e = lo.matched_abs_errors(w[perm][None] + 1e-14, w[None])
    assert e.max() < 1e-13


def test_parity_report_detects_errors():
    from tokura_zgeev_batched_gb300 import workloads as wl

    A = wl.gaussian(4, 6, seed=1)
    w, info, _ = lo.zgeev(A)
    flags = np.zeros(4, np.int8)
    rep = lo.parity_report(A, w, flags)
    assert rep["max_rel_err"] < 1e-14 and rep["flag_mismatch"] == 0
    bad = w.copy()
    bad[2, 3] += 1e-6
    rep = lo.parity_report(A, bad, flags)
    assert rep["max_rel_err"] > 1e-8
    flags[1] = 1
    rep = lo.parity_report(A, w, flags)
    assert rep["flag_mismatch"] == 1


def test_condition_numbers_match_eigenvector_formula():
    import scipy.linalg as sl

    from tokura_zgeev_batched_gb300 import workloads as wl

    A = wl.gaussian(3, 7, seed=3)
    w, rc, info = lo.zgeevx_rconde(A)
    for k in range(3):
        # The harness reads buffers column-major: it sees A[k].T
        wk, vl, vr = sl.eig(A[k].T, left=True, right=True)
        s = np.abs(np.sum(vl.conj() * vr, axis=0)) / (np.linalg.norm(vl, axis=0) * np.linalg.norm(vr, axis=0))
        order = [int(np.argmin(np.abs(wk - x))) for x in w[k]]
        assert np.allclose(rc[k], s[order], rtol=1e-8)


# ---- CPU restatement of the reference's own algorithm (oracle/ref_algorithm.c)

# Buffers are read column-major, so the row-major array holds H^T for the Hessenberg matrix
# H = [[1, 2, 3], [2i, 4, 5], [0, 3i, 6]].
QUIRK_PURELY_IMAGINARY_SUBDIAGONAL = np.array([[1, 2, 3], [2j, 4, 5], [0, 3j, 6]], np.complex128).T.copy()


def test_reference_algorithm_matches_published_error_level():
    """On U(-1,1) inputs (the reference's distribution) its error vs LAPACK stays within the
    published worst case, max |dl|/|l| = 9.29e-11 over n = 1..62 (stream_test_with_MKL/exetime_precision.csv)."""
    from tokura_zgeev_batched_gb300 import workloads as wl

    for n in (2, 3, 5, 8, 16, 24, 32):
        A = wl.uniform(32, n, seed=40 + n)
        w, flag = lo.reference_algorithm(A)
        wr, info, _ = lo.zgeev(A)
        assert (flag == 0).all() and (info == 0).all()
        rel = lo.matched_abs_errors(w, wr) / np.maximum(np.abs(wr), 1e-300)
        assert rel.max() <= 9.29e-11, (n, rel.max())


def test_reference_algorithm_flags_every_1x1_matrix():
    """Its sweep counter reaches the cap n^4 = 1 on the converging pass, so n = 1 always returns flag 1
    (tokura_zhseqr_MWB_kernel.cuh:655,768-776); LAPACK (and this library) report success."""
    A = np.array([[[2.5 - 1j]], [[-3.0]]])
    w, flag = lo.reference_algorithm(A)
    assert list(flag) == [1, 1]
    assert np.allclose(w[:, 0], A[:, 0, 0])


def test_reference_algorithm_real_part_deflation_quirk():
    """Its negligibility test only inspects real parts, so purely imaginary subdiagonals are
    dropped and the diagonal is returned as the spectrum."""
    w, flag = lo.reference_algorithm(QUIRK_PURELY_IMAGINARY_SUBDIAGONAL)
    wr, info, _ = lo.zgeev(QUIRK_PURELY_IMAGINARY_SUBDIAGONAL)
    assert flag[0] == 0 and info[0] == 0
    assert np.allclose(np.sort_complex(w[0]), [1, 4, 6])
    assert lo.matched_abs_errors(w, wr).max() > 0.1


# ---- real path oracle (LAPACK dgeev via oracle/cpu_zgeev.c)

GOLDEN_REAL = os.path.join(os.path.dirname(__file__), "golden", "dgeev_golden.npz")


@pytest.fixture(scope="module")
def golden_real():
    return np.load(GOLDEN_REAL)


def test_real_oracle_reproduces_golden(golden_real):
    """LAPACK dgeev on this machine reproduces the stored outputs (tests/golden/make_golden_real.py)
    within 1e-12 ||A||_F, with the same INFO and LAPACK's conjugate-pair convention."""
    for name in cases(golden_real):
        A = golden_real[f"{name}/A"]
        wr, wi, info, _ = lo.dgeev(A, threads=2)
        assert np.array_equal(info, golden_real[f"{name}/info"]), name
        assert lo.check_conjugate_pairs(wr, wi), name
        assert lo.check_conjugate_pairs(golden_real[f"{name}/wr"], golden_real[f"{name}/wi"]), name
        err = lo.matched_abs_errors(wr + 1j * wi, golden_real[f"{name}/wr"] + 1j * golden_real[f"{name}/wi"])
        scale = np.maximum(np.linalg.norm(A, axis=(1, 2)), 1e-300)
        assert np.all(err.max(axis=1) <= 1e-12 * scale + 1e-300), name


def test_real_oracle_known_answers(golden_real):
    """Exact spectra (orthogonally similar rotation blocks, triangular, zero, a companion matrix
    with known roots) within 1e-13 ||A||_F times the worst eigenvalue condition number."""
    checked = 0
    for name in cases(golden_real):
        key = f"{name}/exact"
        if key not in golden_real.files:
            continue
        A = golden_real[f"{name}/A"]
        wr, wi, info, _ = lo.dgeev(A, threads=2)
        assert (info == 0).all(), name
        err = lo.matched_abs_errors(wr + 1j * wi, golden_real[key])
        fro = np.linalg.norm(A, axis=(1, 2))
        cond = 1.0 / np.maximum(golden_real[f"{name}/rconde"], 1e-300)
        bound = np.where(fro > 0, fro, 1.0) * 1e-13 * np.maximum(cond.max(axis=1), 1.0)
        assert np.all(err.max(axis=1) <= bound), (name, err.max(axis=1), bound)
        checked += 1
    assert checked >= 10


def test_real_oracle_agrees_with_complex_oracle():
    rng = np.random.default_rng(5)
    A = rng.standard_normal((8, 12, 12))
    wr, wi, info, _ = lo.dgeev(A, threads=2)
    w, zinfo, _ = lo.zgeev(A.astype(np.complex128), threads=2)
    assert (info == 0).all() and (zinfo == 0).all()
    err = lo.matched_abs_errors(wr + 1j * wi, w)
    assert err.max() <= 1e-12 * np.linalg.norm(A, axis=(1, 2)).max()


def test_conjugate_pair_convention_checker():
    wr = np.array([[1.0, 1.0, 3.0]])
    assert lo.check_conjugate_pairs(wr, np.array([[2.0, -2.0, 0.0]]))
    assert not lo.check_conjugate_pairs(wr, np.array([[-2.0, 2.0, 0.0]]))  # negative part first
    assert not lo.check_conjugate_pairs(wr, np.array([[2.0, -2.0 + 1e-15, 0.0]]))  # not exact conjugates
    assert not lo.check_conjugate_pairs(np.array([[1.0, 1.0 + 1e-15, 3.0]]), np.array([[2.0, -2.0, 0.0]]))
    assert not lo.check_conjugate_pairs(wr, np.array([[0.0, 0.0, 2.0]]))  # pair cut off at the end


def test_real_parity_report_detects_errors():
    rng = np.random.default_rng(9)
    A = rng.standard_normal((4, 7, 7))
    wr, wi, _, _ = lo.dgeev(A, threads=2)
    flags = np.zeros(4, np.int8)
    rep = lo.real_parity_report(A, wr, wi, flags)
    assert rep["max_rel_err"] < 1e-14 and rep["flag_mismatch"] == 0 and rep["pairs_ok"]
    bad = wr.copy()
    bad[1, 0] += 1e-6
    rep = lo.real_parity_report(A, bad, wi, flags)
    assert rep["max_rel_err"] > 1e-8
    flags[3] = 1
    assert lo.real_parity_report(A, wr, wi, flags)["flag_mismatch"] == 1
