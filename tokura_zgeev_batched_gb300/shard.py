"""One ragged batch split across devices, one process per GPU.

Matrices are independent, so a batch shards with no exchange step: rank r solves a
contiguous range of matrices on its own device and its eigenvalues and flags are a
disjoint slice of the whole batch's outputs. The ranges are balanced by the algorithmic
work of the eigenvalue solve, proportional to n_j^3 per matrix (40 n^3 real flops by the
convention the library is measured with), so each rank gets the same share of work, not
the same number of matrices. The reference has no multi-device code (it always uses
device 0, tokura_zgeev_batched.cu:151); this module is the host-side plan for the case.

Layout: the batch is given as in :func:`tokura_zgeev_batched_gb300.api.zgeev_ragged`
(1-D complex entries, orders ``ns``, element offsets ``offsets``); the assembled
eigenvalues are packed by the exclusive prefix sum of ``ns``, flags one per matrix.
"""
from __future__ import annotations

import numpy as np


def work_per_matrix(ns) -> np.ndarray:
    """Relative work of each matrix's solve: n^3."""
    return np.asarray(ns, dtype=np.float64) ** 3


def balanced_ranges(ns, parts: int) -> np.ndarray:
    """Boundaries ``b[0] = 0 <= b[1] <= ... <= b[parts] = len(ns)``: rank r takes matrices
    ``b[r]:b[r+1]``. Each cut is placed at the matrix boundary nearest to r/parts of the
    total work, so every range's work is within one matrix's work of total/parts."""
    if parts < 1:
        raise ValueError("parts must be >= 1")
    w = work_per_matrix(ns)
    b = w.shape[0]
    c = np.concatenate([[0.0], np.cumsum(w)])
    total = c[-1]
    bounds = [0]
    for k in range(1, parts):
        target = total * k / parts
        i = int(np.searchsorted(c, target, side="left"))  # first prefix >= target
        if i > 0 and (i > b or target - c[i - 1] <= c[i] - target):
            i -= 1
        bounds.append(min(max(i, bounds[-1]), b))
    bounds.append(b)
    return np.asarray(bounds, dtype=np.int64)


def gather_range(A_flat, ns, offsets, start: int, stop: int):
    """The matrices ``start:stop`` of a ragged batch packed contiguously (a copy): returns
    ``(A_part, ns_part, offsets_part)`` with offsets into ``A_part``. Works on numpy arrays
    or torch tensors (then the gather runs on their device)."""
    ns_part = ns[start:stop]
    offs = offsets[start:stop]
    try:
        import torch

        is_torch = isinstance(A_flat, torch.Tensor)
    except ImportError:  # pragma: no cover
        is_torch = False
    if is_torch:
        import torch

        n64 = ns_part.to(torch.int64)
        sizes = n64 * n64
        new_offs = torch.cumsum(sizes, 0) - sizes
        total = int(sizes.sum().item())
        seg = torch.repeat_interleave(torch.arange(n64.numel(), device=A_flat.device), sizes)
        pos = torch.arange(total, device=A_flat.device) - new_offs[seg]
        return A_flat[offs.to(torch.int64)[seg] + pos], ns_part, new_offs
    n64 = np.asarray(ns_part, dtype=np.int64)
    sizes = n64 * n64
    new_offs = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    seg = np.repeat(np.arange(n64.size), sizes)
    pos = np.arange(int(sizes.sum())) - new_offs[seg]
    return np.asarray(A_flat)[np.asarray(offs, dtype=np.int64)[seg] + pos], ns_part, new_offs


def eigen_range(ns, start: int, stop: int) -> tuple[int, int]:
    """Slice ``[lo, hi)`` of the packed eigenvalue array that matrices ``start:stop`` fill."""
    n64 = np.asarray(ns, dtype=np.int64)
    lo = int(n64[:start].sum())
    return lo, lo + int(n64[start:stop].sum())


def solve_shard(A_flat, ns, offsets, rank: int, world: int, solver=None):
    """Solves rank ``rank``'s range of the batch. ``solver(A_part, ns_part, offsets_part)``
    returns ``(eigenvalues, flag)`` packed for the part; by default it is the library's
    ragged entry point on the current CUDA device (inputs must then be CUDA tensors).
    Returns ``(start, stop, eigenvalues, flag)``."""
    bounds = balanced_ranges(np.asarray(ns.cpu() if hasattr(ns, "cpu") else ns), world)
    start, stop = int(bounds[rank]), int(bounds[rank + 1])
    A_part, ns_part, offs_part = gather_range(A_flat, ns, offsets, start, stop)
    if solver is None:
        from .api import zgeev_ragged

        if stop == start:
            import torch

            dev = A_flat.device
            return start, stop, torch.empty(0, dtype=torch.complex128, device=dev), torch.empty(
                0, dtype=torch.int8, device=dev)
        eig, flag = zgeev_ragged(A_part, ns_part, offsets=offs_part)
        return start, stop, eig, flag
    eig, flag = solver(A_part, ns_part, offs_part)
    return start, stop, eig, flag


def assemble(parts, ns):
    """Whole-batch outputs from every rank's ``(start, stop, eigenvalues, flag)`` (host
    arrays, any order): eigenvalues packed by the prefix sum of ``ns``, one flag per
    matrix. Checks that the ranges cover every matrix exactly once."""
    ns = np.asarray(ns, dtype=np.int64)
    b = ns.size
    covered = np.zeros(b, np.int64)
    eig = np.empty(int(ns.sum()), np.complex128)
    flag = np.empty(b, np.int8)
    for start, stop, e, f in parts:
        covered[start:stop] += 1
        lo, hi = eigen_range(ns, start, stop)
        e = np.asarray(e).reshape(-1)
        f = np.asarray(f).reshape(-1)
        if e.size != hi - lo or f.size != stop - start:
            raise ValueError(f"range {start}:{stop}: {e.size} eigenvalues / {f.size} flags, "
                             f"expected {hi - lo} / {stop - start}")
        eig[lo:hi] = e
        flag[start:stop] = f
    if not np.all(covered == 1):
        raise ValueError("ranges do not cover every matrix exactly once")
    return eig, flag


def gather_to_rank0(part, ns, dist):
    """Collects every rank's ``solve_shard`` result on rank 0 (host copies over
    ``torch.distributed``) and returns the assembled ``(eigenvalues, flag)`` there, None
    elsewhere. The only communication is this optional gather of disjoint outputs."""
    start, stop, e, f = part
    e = e.cpu().numpy() if hasattr(e, "cpu") else np.asarray(e)
    f = f.cpu().numpy() if hasattr(f, "cpu") else np.asarray(f)
    objs = [None] * dist.get_world_size()
    dist.all_gather_object(objs, (start, stop, e, f))
    if dist.get_rank() != 0:
        return None
    return assemble(objs, ns)
