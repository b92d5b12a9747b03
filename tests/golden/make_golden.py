"""Generates tests/golden/zgeev_golden.npz: seeded inputs with LAPACK outputs.

Run:  python tests/golden/make_golden.py

Each case stores the input batch (row-major buffers, read as column-major by
the library and by LAPACK — so both compute the eigenvalues of the
transpose, which are the eigenvalues of the matrix), LAPACK zgeev's
eigenvalues and INFO, zgeevx's RCONDE (BALANC='N'), and, where the spectrum is
known by construction, the exact eigenvalues. The reference repository ships
no golden vectors (its inputs come from std::random_device,
stream_test_with_MKL/main.cu:182-202), so these fixtures are generated from
the oracle (oracle/lapack_oracle.py) on seeded inputs, plus known-answer
cases whose eigenvalues are exact.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import lapack_oracle as lo  # noqa: E402
from tokura_zgeev_batched_gb300 import workloads as wl  # noqa: E402

OUT = os.path.join(HERE, "zgeev_golden.npz")


def known_answer_cases():
    """(name, A[batch,n,n], exact eigenvalues[batch,n] or None)."""
    rng = np.random.default_rng(11)
    cases = []
    # Upper-triangular: eigenvalues are the diagonal (buffer read column-major = lower-triangular transpose).
    for n in (1, 2, 3, 5, 8, 17, 32, 64):
        T = np.triu(wl._cgauss(rng, (2, n, n)))
        cases.append((f"triangular_n{n}", T, np.diagonal(T, axis1=1, axis2=2).copy()))
    # Diagonal with repeated entries.
    for n in (4, 16):
        d = np.repeat(wl._cgauss(rng, (3, n // 2)), 2, axis=1)
        cases.append((f"diag_repeated_n{n}", np.array([np.diag(x) for x in d]), d))
    # Zero and identity-multiple.
    for n in (1, 3, 16, 64):
        cases.append((f"zero_n{n}", np.zeros((2, n, n), np.complex128), np.zeros((2, n), np.complex128)))
        c = np.array([1.5 - 2j, -0.25j])
        cases.append((f"scaled_identity_n{n}", c[:, None, None] * np.eye(n)[None], np.repeat(c[:, None], n, 1)))
    # Constructed spectra (V diag V^-1) with separated eigenvalues.
    for n in (4, 16, 48):
        A, lam = wl.vdv(3, n, seed=100 + n, min_sep=0.05, return_eigs=True)
        cases.append((f"vdv_sep_n{n}", A, lam))
    # Circulant matrices: eigenvalues = DFT of the first column.
    for n in (6, 31):
        c = wl._cgauss(rng, (3, n))
        Cs = np.stack([np.array([[ck[(i - j) % n] for j in range(n)] for i in range(n)]) for ck in c])
        cases.append((f"circulant_n{n}", Cs, np.fft.fft(c, axis=1)))
    # Already Hessenberg, and huge / tiny scalings (exercise the exact power-of-two pre-scaling).
    for n in (8, 33):
        H = np.triu(wl._cgauss(rng, (4, n, n)), -1)
        cases.append((f"hessenberg_n{n}", H, None))
    for sc, tag in ((1e150, "huge"), (1e-150, "tiny"), (2.0 ** 70, "pow2big")):
        A = wl.gaussian(4, 12, seed=5) * sc
        cases.append((f"scaled_{tag}_n12", A, None))
    # Jordan block (defective: eigenvalue 2 with multiplicity n; ill-conditioned).
    for n in (3, 10):
        J = 2.0 * np.eye(n) + np.diag(np.ones(n - 1), 1)
        cases.append((f"jordan_n{n}", J[None].astype(np.complex128), np.full((1, n), 2.0 + 0j)))
    return cases


def random_cases():
    cases = []
    def b(n):
        return 8 if n < 32 else 3

    for n in (1, 2, 3, 4, 5, 7, 8, 9, 16, 24, 32, 47, 64):
        cases.append((f"gaussian_n{n}", wl.gaussian(b(n), n, seed=2000 + n), None))
    for n in (4, 16, 32, 64):
        cases.append((f"uniform_n{n}", wl.uniform(b(n), n, seed=3000 + n), None))
        cases.append((f"vdv_n{n}", wl.vdv(b(n), n, seed=4000 + n), None))
        cases.append((f"companion_n{n}", wl.companion(b(n), n, seed=5000 + n), None))
    return cases


def main():
    data = {}
    names = []
    for name, A, exact in known_answer_cases() + random_cases():
        A = np.ascontiguousarray(A, np.complex128)
        w, info, _ = lo.zgeev(A, threads=1)
        _, rc, _ = lo.zgeevx_rconde(A, threads=1)
        data[f"{name}/A"] = A
        data[f"{name}/w"] = w
        data[f"{name}/info"] = info
        data[f"{name}/rconde"] = rc
        if exact is not None:
            data[f"{name}/exact"] = np.asarray(exact, np.complex128)
        names.append(name)
    data["names"] = np.array(names)
    np.savez_compressed(OUT, **data)
    print(f"wrote {OUT}: {len(names)} cases, {os.path.getsize(OUT) / 1e6:.2f} MB")


if __name__ == "__main__":
    main()
