"""Generates tests/golden/dgeev_golden.npz: seeded real inputs with LAPACK dgeev outputs.

Run:  python tests/golden/make_golden_real.py

Fixtures for the real (tokura_dgeev_batched_gpu / sgeev) path, in the layout of
zgeev_golden.npz: each case stores the input batch (row-major buffers read as
column-major, i.e. the transposes, which have the same eigenvalues), LAPACK
dgeev's wr, wi and INFO (conjugate pairs adjacent, positive imaginary part
first), zgeevx's RCONDE on the same matrices, and, where the spectrum is known
by construction, the exact eigenvalues. The reference has no real path and no
golden vectors; these come from the oracle (oracle/lapack_oracle.py) on seeded
inputs, plus known-answer cases.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import lapack_oracle as lo  # noqa: E402

OUT = os.path.join(HERE, "dgeev_golden.npz")


def rotation_blocks(rng, n: int):
    """Q^T B Q, B block diagonal with 2x2 blocks [[a, -b], [b, a]] (eigenvalues a +- ib) and,
    for odd n, one 1x1 block; Q orthogonal. Returns (matrix, exact spectrum)."""
    B = np.zeros((n, n))
    lam = []
    for k in range(0, n - 1, 2):
        a, b = rng.uniform(-2, 2), rng.uniform(0.5, 2)
        B[k:k + 2, k:k + 2] = [[a, -b], [b, a]]
        lam += [a + 1j * b, a - 1j * b]
    if n % 2:
        B[-1, -1] = rng.uniform(-2, 2)
        lam.append(B[-1, -1])
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    return Q.T @ B @ Q, np.array(lam)


def companion(roots) -> np.ndarray:
    """Companion matrix (row-major buffer) of the monic real polynomial with these roots."""
    c = np.real(np.poly(roots))
    n = len(roots)
    C = np.zeros((n, n))
    C[0, :] = -c[1:]
    C[1:, :-1] = np.eye(n - 1)
    return C


def known_answer_cases():
    rng = np.random.default_rng(21)
    cases = []
    for n in (2, 5, 16, 33):
        mats, lam = zip(*[rotation_blocks(rng, n) for _ in range(4)])
        cases.append((f"rotation_blocks_n{n}", np.stack(mats), np.stack(lam)))
    for n in (1, 3, 8, 64):
        T = np.triu(rng.standard_normal((2, n, n)))
        cases.append((f"triangular_n{n}", T, np.diagonal(T, axis1=1, axis2=2).astype(np.complex128)))
    for n in (1, 4):
        cases.append((f"zero_n{n}", np.zeros((2, n, n)), np.zeros((2, n), np.complex128)))
    roots = np.array([1.0, 2.0, 1j, -1j, 1 + 2j, 1 - 2j])
    cases.append(("companion_known_roots_n6", companion(roots)[None], roots[None]))
    return cases


def random_cases():
    cases = []
    for n in (1, 2, 3, 4, 7, 8, 16, 32, 48, 64):
        b = 8 if n < 32 else 3
        cases.append((f"gaussian_n{n}", np.random.default_rng(6000 + n).standard_normal((b, n, n)), None))
    g = np.random.default_rng(7000).standard_normal((4, 12, 12))
    for sc, tag in ((1e150, "huge"), (1e-150, "tiny")):
        cases.append((f"scaled_{tag}_n12", g * sc, None))
    return cases


def main():
    data = {}
    names = []
    for name, A, exact in known_answer_cases() + random_cases():
        A = np.ascontiguousarray(A, np.float64)
        wr, wi, info, _ = lo.dgeev(A, threads=1)
        _, rc, _ = lo.zgeevx_rconde(A.astype(np.complex128), threads=1)
        data[f"{name}/A"] = A
        data[f"{name}/wr"] = wr
        data[f"{name}/wi"] = wi
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
