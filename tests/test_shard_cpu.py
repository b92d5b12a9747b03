"""Splitting one ragged batch across ranks: balance by sum of n^3, coverage, and a two-rank
gloo run whose assembled outputs equal the unsplit ones (a CPU stand-in solver: the GPU
path is the library's ragged entry point, one device per rank)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from tokura_zgeev_batched_gb300 import shard
from tokura_zgeev_batched_gb300 import workloads as wl


@pytest.mark.parametrize("parts", [1, 2, 3, 4, 8])
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_balanced_within_one_matrix(parts, seed):
    ns = wl.ragged_sizes(5000, 1, 64, seed=seed)
    b = shard.balanced_ranges(ns, parts)
    assert b[0] == 0 and b[-1] == ns.size and np.all(np.diff(b) >= 0)
    w = shard.work_per_matrix(ns)
    share = np.array([w[b[r]:b[r + 1]].sum() for r in range(parts)])
    assert abs(share.sum() - w.sum()) <= 1e-9 * w.sum()
    assert np.all(np.abs(share - w.sum() / parts) <= w.max()), (share, w.sum() / parts)


def test_degenerate_batches():
    assert list(shard.balanced_ranges(np.array([64]), 4)) in ([0, 0, 0, 1, 1], [0, 0, 1, 1, 1], [0, 1, 1, 1, 1])
    b = shard.balanced_ranges(np.array([1, 1, 64]), 2)
    assert b[0] == 0 and b[-1] == 3
    assert list(shard.balanced_ranges(np.array([5, 5, 5, 5]), 2)) == [0, 2, 4]
    with pytest.raises(ValueError):
        shard.balanced_ranges(np.array([3]), 0)


def _diag_solver(A_part, ns_part, offs_part):
    """Stand-in solver: the diagonal entries as 'eigenvalues', flag = n mod 3."""
    e = np.concatenate([A_part[o + np.arange(k) * (k + 1)] for o, k in zip(offs_part, ns_part)]) if len(ns_part) \
        else np.zeros(0, np.complex128)
    return e, (np.asarray(ns_part) % 3).astype(np.int8)


def _batch(seed=7, count=400):
    ns = wl.ragged_sizes(count, 1, 64, seed=seed)
    mats = [wl.gaussian(1, int(k), seed=seed + j)[0] for j, k in enumerate(ns)]
    A, ns_, offs, _ = wl.pack_ragged(mats)
    # scatter the matrices so offsets are not in batch order (as a caller's buffer may be)
    order = np.random.default_rng(seed).permutation(count)
    sizes = ns.astype(np.int64) ** 2
    new_offs = np.empty(count, np.int64)
    new_offs[order] = np.concatenate([[0], np.cumsum(sizes[order])[:-1]])
    A2 = np.empty_like(A)
    for j in range(count):
        A2[new_offs[j]:new_offs[j] + sizes[j]] = A[offs[j]:offs[j] + sizes[j]]
    return A2, ns, new_offs


def test_gather_range_numpy_and_torch_agree():
    import torch

    A, ns, offs = _batch()
    a_np, n_np, o_np = shard.gather_range(A, ns, offs, 50, 170)
    a_t, n_t, o_t = shard.gather_range(torch.from_numpy(A), torch.from_numpy(ns), torch.from_numpy(offs), 50, 170)
    assert np.array_equal(a_np, a_t.numpy()) and np.array_equal(o_np, o_t.numpy())
    for j in range(50, 170):
        k = int(ns[j])
        assert np.array_equal(a_np[o_np[j - 50]:o_np[j - 50] + k * k], A[offs[j]:offs[j] + k * k])


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    A, ns, offs = _batch()
    part = shard.solve_shard(A, ns, offs, rank, world, solver=_diag_solver)
    out = shard.gather_to_rank0(part, ns, dist)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, part[0], part[1], None if out is None else (out[0].tolist(), out[1].tolist())))


def test_two_gloo_ranks_assemble_the_whole_batch():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    # Read the results before joining: a child cannot exit while its queued result is unread.
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    A, ns, offs = _batch()
    assert res[0][1] == 0 and res[0][2] == res[1][1] and res[1][2] == ns.size  # contiguous, complete
    assert res[1][3] is None
    eig, flag = res[0][3]
    e_ref, f_ref = _diag_solver(A, ns, offs)
    assert np.array_equal(np.array(eig), e_ref) and np.array_equal(np.array(flag), f_ref)


def test_assemble_rejects_gaps_and_overlaps():
    ns = np.array([2, 3, 1])
    ok = [(0, 2, np.zeros(5), np.zeros(2)), (2, 3, np.zeros(1), np.zeros(1))]
    shard.assemble(ok, ns)
    with pytest.raises(ValueError):
        shard.assemble(ok[:1], ns)
    with pytest.raises(ValueError):
        shard.assemble(ok + [(2, 3, np.zeros(1), np.zeros(1))], ns)
