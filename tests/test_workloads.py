"""Seeded generators: shapes, constructed spectra, separation, ragged packing."""
import numpy as np

from tokura_zgeev_batched_gb300 import workloads as wl


def test_gaussian_reproducible():
    a = wl.gaussian(3, 5, seed=9)
    b = wl.gaussian(3, 5, seed=9)
    assert a.shape == (3, 5, 5) and a.dtype == np.complex128 and np.array_equal(a, b)


def test_vdv_spectrum():
    A, lam = wl.vdv(4, 10, seed=2, min_sep=0.05, return_eigs=True)
    for k in range(4):
        w = np.linalg.eigvals(A[k])
        d = np.abs(w[:, None] - lam[k][None, :]).min(axis=1)
        assert d.max() < 1e-9
        sep = np.abs(lam[k][:, None] - lam[k][None, :]) + np.eye(10) * 9
        assert sep.min() >= 0.05
        assert np.all(np.abs(lam[k]) <= 1.0)


def test_companion_roots():
    A = wl.companion(2, 6, seed=4)
    for k in range(2):
        coeffs = np.concatenate([[1.0], -A[k, 0, :]])
        r = np.roots(coeffs)
        w = np.linalg.eigvals(A[k])
        assert np.abs(np.sort_complex(r) - np.sort_complex(w)).max() < 1e-8


def test_pack_ragged():
    mats = [np.full((n, n), n, np.complex128) for n in (3, 1, 4)]
    buf, ns, offs, eoffs = wl.pack_ragged(mats)
    assert list(ns) == [3, 1, 4] and list(offs) == [0, 9, 10] and list(eoffs) == [0, 3, 4]
    assert buf.shape == (26,) and buf[9] == 1 and buf[10] == 4
