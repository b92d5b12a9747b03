"""Seeded synthetic matrix batches for the benchmark configurations.

All generators return complex128 arrays ``[batch, n, n]`` whose row-major
buffer is handed to the library as column-major storage (the eigenvalues of
a matrix and of its transpose coincide, so the distinction is immaterial for
the forward path). numpy versions feed tests and CPU checks; torch versions
build the large batches directly on the GPU.

Classes (the reference itself uses only i.i.d. U(-1,1) entries,
stream_test_with_MKL/main.cu:182-202):
  * ``gaussian``: Re, Im i.i.d. N(0, 1);
  * ``vdv``: A = V diag(lambda) V^-1, V = I + 0.3 G (G complex Gaussian),
    lambda uniform in the unit disk (optionally with a minimum pairwise
    separation, rejection-sampled, and a shift);
  * ``companion``: companion matrix of a monic degree-n polynomial with
    complex Gaussian coefficients;
  * ``uniform``: Re, Im i.i.d. U(-1, 1), the reference's own distribution.
"""
from __future__ import annotations

import numpy as np

SEED = 20261203


def _cgauss(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def gaussian(batch: int, n: int, seed: int = SEED) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return _cgauss(rng, (batch, n, n))


def uniform(batch: int, n: int, seed: int = SEED) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return rng.uniform(-1, 1, (batch, n, n)) + 1j * rng.uniform(-1, 1, (batch, n, n))


def disk_eigenvalues(rng, batch: int, n: int, min_sep: float = 0.0) -> np.ndarray:
    """``[batch, n]`` points uniform in the unit disk, pairwise >= min_sep apart."""
    lam = np.sqrt(rng.uniform(0, 1, (batch, n))) * np.exp(2j * np.pi * rng.uniform(0, 1, (batch, n)))
    if min_sep <= 0 or n < 2:
        return lam
    for k in range(batch):
        row = lam[k]
        for _ in range(10000):
            d = np.abs(row[:, None] - row[None, :]) + np.eye(n) * 10
            bad = np.where(d.min(axis=1) < min_sep)[0]
            if len(bad) == 0:
                break
            i = bad[0]
            row[i] = np.sqrt(rng.uniform()) * np.exp(2j * np.pi * rng.uniform())
        lam[k] = row
    return lam


def vdv(batch: int, n: int, seed: int = SEED, min_sep: float = 0.0, shift: float = 0.0,
        return_eigs: bool = False):
    rng = np.random.default_rng(seed)
    lam = disk_eigenvalues(rng, batch, n, min_sep) + shift
    V = np.eye(n)[None] + 0.3 * _cgauss(rng, (batch, n, n))
    A = np.linalg.solve(V.transpose(0, 2, 1), (V * lam[:, None, :]).transpose(0, 2, 1)).transpose(0, 2, 1)
    return (A, lam) if return_eigs else A


def companion(batch: int, n: int, seed: int = SEED) -> np.ndarray:
    rng = np.random.default_rng(seed)
    c = _cgauss(rng, (batch, n))  # p(z) = z^n + c[0] z^(n-1) + ... + c[n-1]
    A = np.zeros((batch, n, n), np.complex128)
    A[:, 0, :] = -c
    if n > 1:
        idx = np.arange(n - 1)
        A[:, idx + 1, idx] = 1.0
    return A


GENERATORS = {"gaussian": gaussian, "vdv": vdv, "companion": companion, "uniform": uniform}


def ragged_sizes(batch: int, nmin: int, nmax: int, seed: int = SEED) -> np.ndarray:
    return np.random.default_rng(seed).integers(nmin, nmax + 1, size=batch).astype(np.int32)


def pack_ragged(mats: list[np.ndarray]):
    """Packs square matrices contiguously: returns (buffer, n[int32], offsets[int64], eig_offsets[int64])."""
    ns = np.array([m.shape[0] for m in mats], np.int32)
    sizes = ns.astype(np.int64) ** 2
    offs = np.zeros(len(mats), np.int64)
    if len(mats) > 1:
        offs[1:] = np.cumsum(sizes)[:-1]
    eoffs = np.zeros(len(mats), np.int64)
    if len(mats) > 1:
        eoffs[1:] = np.cumsum(ns.astype(np.int64))[:-1]
    buf = np.concatenate([m.reshape(-1) for m in mats]) if mats else np.zeros(0, np.complex128)
    return buf, ns, offs, eoffs


# ---------------------------------------------------------------- torch (GPU)

def torch_gaussian(batch: int, n: int, seed: int = SEED, device: str = "cuda"):
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(seed)
    re = torch.randn(batch, n, n, generator=g, device=device, dtype=torch.float64)
    im = torch.randn(batch, n, n, generator=g, device=device, dtype=torch.float64)
    return torch.complex(re, im)


def torch_vdv(batch: int, n: int, seed: int = SEED, device: str = "cuda", chunk: int = 0):
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(seed)
    out = torch.empty(batch, n, n, dtype=torch.complex128, device=device)
    eye = torch.eye(n, dtype=torch.complex128, device=device)
    chunk = chunk or max(8192, (1 << 25) // (n * n))
    for s in range(0, batch, chunk):
        b = min(chunk, batch - s)
        r = torch.sqrt(torch.rand(b, n, generator=g, device=device, dtype=torch.float64))
        th = 2 * torch.pi * torch.rand(b, n, generator=g, device=device, dtype=torch.float64)
        lam = torch.polar(r, th)
        G = torch.complex(torch.randn(b, n, n, generator=g, device=device, dtype=torch.float64),
                          torch.randn(b, n, n, generator=g, device=device, dtype=torch.float64))
        V = eye + 0.3 * G
        out[s:s + b] = _solve_right(V, V * lam[:, None, :])
    return out


def torch_companion(batch: int, n: int, seed: int = SEED, device: str = "cuda"):
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(seed)
    c = torch.complex(torch.randn(batch, n, generator=g, device=device, dtype=torch.float64),
                      torch.randn(batch, n, generator=g, device=device, dtype=torch.float64))
    A = torch.zeros(batch, n, n, dtype=torch.complex128, device=device)
    A[:, 0, :] = -c
    if n > 1:
        idx = torch.arange(n - 1, device=device)
        A[:, idx + 1, idx] = 1.0
    return A


TORCH_GENERATORS = {"gaussian": torch_gaussian, "vdv": torch_vdv, "companion": torch_companion}


def torch_vdv_separated(batch: int, n: int, seed: int = SEED, min_sep: float = 0.05, shift: float = 0.0,
                        device: str = "cuda", chunk: int = 4096):
    """A = V diag(lambda) V^-1 (V = I + 0.3 G) with lambda in the unit disk, pairwise >= min_sep apart
    (rejection-resampled), plus ``shift``. Returns (A, lambda)."""
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(seed)
    A = torch.empty(batch, n, n, dtype=torch.complex128, device=device)
    lam_all = torch.empty(batch, n, dtype=torch.complex128, device=device)
    eye = torch.eye(n, dtype=torch.complex128, device=device)

    def disk(b):
        r = torch.sqrt(torch.rand(b, n, generator=g, device=device, dtype=torch.float64))
        th = 2 * torch.pi * torch.rand(b, n, generator=g, device=device, dtype=torch.float64)
        return torch.polar(r, th)

    for s in range(0, batch, chunk):
        b = min(chunk, batch - s)
        lam = disk(b)
        if n > 1 and min_sep > 0:
            big = torch.eye(n, device=device, dtype=torch.float64) * 10
            for _ in range(1000):
                d = (lam[:, :, None] - lam[:, None, :]).abs() + big
                bad = d.min(dim=-1).values < min_sep
                if not bool(bad.any()):
                    break
                lam = torch.where(bad, disk(b), lam)
        lam = lam + shift
        G = torch.complex(torch.randn(b, n, n, generator=g, device=device, dtype=torch.float64),
                          torch.randn(b, n, n, generator=g, device=device, dtype=torch.float64))
        V = eye + 0.3 * G
        A[s:s + b] = _solve_right(V, V * lam[:, None, :])
        lam_all[s:s + b] = lam
    return A, lam_all


def _solve_right(V, B):
    """X with X V = B; on the CPU if the GPU linear-algebra library cannot be loaded (e.g. under a profiler)."""
    import torch

    try:
        return torch.linalg.solve(V, B, left=False)
    except RuntimeError:
        return torch.linalg.solve(V.cpu(), B.cpu(), left=False).to(V.device)
