"""Ragged entry point (per-matrix n, one persistent launch) against LAPACK and the plain path."""
import numpy as np
import pytest

from oracle import lapack_oracle as lo
from tokura_zgeev_batched_gb300 import api
from tokura_zgeev_batched_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def make_batch(batch, nmin, nmax, seed):
    ns = wl.ragged_sizes(batch, nmin, nmax, seed=seed)
    rng = np.random.default_rng(seed + 1)
    mats = [rng.standard_normal((k, k)) + 1j * rng.standard_normal((k, k)) for k in ns]
    return mats, ns


def check_against_lapack(mats, eig, eoffs, flag):
    by_n = {}
    for j, m in enumerate(mats):
        by_n.setdefault(m.shape[0], []).append(j)
    worst = 0.0
    for k, idx in by_n.items():
        A = np.stack([mats[j] for j in idx])
        w = np.stack([eig[eoffs[j]:eoffs[j] + k] for j in idx])
        rep = lo.parity_report(A, w, flag[idx], with_cond=False)
        assert rep["flag_mismatch"] == 0, k
        worst = max(worst, rep["max_rel_err"])
    return worst


@pytest.mark.parametrize("lanes", [0, 1, 2, 4, 8])
def test_ragged_matches_lapack(cuda, lanes):
    import torch

    mats, ns = make_batch(1500, 1, 64, seed=lanes)
    buf, ns, offs, eoffs = wl.pack_ragged(mats)
    h = api.Handle()
    assert h.set_ragged_lanes(lanes) == 0
    eig, flag = api.zgeev_ragged(torch.from_numpy(buf).cuda(), torch.from_numpy(ns), handle=h)
    torch.cuda.synchronize()
    eig, flag = eig.cpu().numpy(), flag.cpu().numpy()
    assert eig.shape[0] == ns.sum() and (flag == 0).all()
    assert check_against_lapack(mats, eig, eoffs, flag) <= lo.TOL_REL_FRO


def test_ragged_equals_plain_per_size(cuda):
    import torch

    mats, ns = make_batch(800, 5, 40, seed=9)
    buf, ns, offs, eoffs = wl.pack_ragged(mats)
    eig, flag = api.zgeev_ragged(torch.from_numpy(buf).cuda(), torch.from_numpy(ns))
    eig = eig.cpu().numpy()
    for k in np.unique(ns):
        idx = np.where(ns == k)[0]
        A = torch.from_numpy(np.stack([mats[j] for j in idx])).cuda()
        w, f = api.zgeev_batched(A)
        w = w.cpu().numpy()
        wr = np.stack([eig[eoffs[j]:eoffs[j] + k] for j in idx])
        fro = np.sqrt(np.sum(np.abs(A.cpu().numpy()) ** 2, axis=(1, 2)))
        assert (lo.matched_abs_errors(wr, w).max(axis=1) / fro).max() <= 1e-12


def test_ragged_invalid_entries_and_custom_eig_offsets(cuda):
    import torch

    mats, ns = make_batch(100, 1, 20, seed=3)
    buf, ns, offs, _ = wl.pack_ragged(mats)
    ns_bad = ns.copy()
    offs_bad = offs.copy()
    ns_bad[5] = 0
    ns_bad[6] = 65
    offs_bad[7] = buf.size  # out of range
    offs_bad[8] = -1
    # eigenvalues of matrix j at 64*j (strided output)
    eo = (np.arange(100) * 64).astype(np.int64)
    eig, flag = api.zgeev_ragged(torch.from_numpy(buf).cuda(), torch.from_numpy(ns_bad),
                                 offsets=torch.from_numpy(offs_bad), eig_offsets=torch.from_numpy(eo))
    flag = flag.cpu().numpy()
    eig = eig.cpu().numpy()
    assert list(flag[5:9]) == [3, 3, 3, 3]
    good = [j for j in range(100) if j not in (5, 6, 7, 8)]
    assert (flag[good] == 0).all()
    assert check_against_lapack([mats[j] for j in good], eig, {i: eo[j] for i, j in enumerate(good)},
                                flag[good]) <= lo.TOL_REL_FRO


def test_ragged_overflow_is_rejected(cuda):
    import torch

    mats, ns = make_batch(20, 8, 8, seed=4)
    buf, ns, offs, _ = wl.pack_ragged(mats)
    offs[:] = 0  # all matrices share the first 64 entries of a 320-entry buffer: sizes sum past the buffer
    small = np.ascontiguousarray(buf[:320])
    eig, flag = api.zgeev_ragged(torch.from_numpy(small).cuda(), torch.from_numpy(ns), offsets=torch.from_numpy(offs))
    assert (flag.cpu().numpy() == 3).all()


def test_ragged_in_cuda_graph(cuda):
    import torch

    mats, ns = make_batch(600, 1, 64, seed=12)
    buf, ns, offs, eoffs = wl.pack_ragged(mats)
    A = torch.from_numpy(buf).cuda()
    n_d = torch.from_numpy(ns).cuda()
    o_d = torch.from_numpy(offs).cuda()
    total_eig = int(ns.sum())
    eig = torch.empty(total_eig, dtype=torch.complex128, device="cuda")
    flag = torch.empty(600, dtype=torch.int8, device="cuda")
    work = torch.empty(api.tokura_get_zgeev_ragged_workspacesize(600, buf.size), dtype=torch.uint8, device="cuda")
    h = api.default_handle()
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        st = api.tokura_zgeev_ragged_gpu(h, 600, n_d.data_ptr(), o_d.data_ptr(), None, buf.size, A.data_ptr(),
                                         eig.data_ptr(), work.data_ptr(), flag.data_ptr(),
                                         torch.cuda.current_stream().cuda_stream)
        assert st == 0
    for _ in range(2):  # replays reuse the queue: it must be reset inside the graph
        eig.zero_()
        flag.fill_(7)
        g.replay()
        torch.cuda.synchronize()
        f = flag.cpu().numpy()
        assert (f == 0).all()
        assert check_against_lapack(mats, eig.cpu().numpy(), eoffs, f) <= lo.TOL_REL_FRO


def test_split_across_ranks_on_one_device(cuda):
    """shard.solve_shard for ranks 0..2 of a 3-way split, run one after another on one device
    (independent calls, nothing waits on another rank), assembles to LAPACK's results."""
    import torch

    from tokura_zgeev_batched_gb300 import shard

    mats, ns = make_batch(1200, 1, 64, seed=31)
    buf, ns, offs, eoffs = wl.pack_ragged(mats)
    A = torch.from_numpy(buf).cuda()
    n_d = torch.from_numpy(ns).cuda()
    o_d = torch.from_numpy(offs).cuda()
    parts = [shard.solve_shard(A, n_d, o_d, r, 3) for r in range(3)]
    torch.cuda.synchronize()
    parts = [(s, e, w.cpu().numpy(), f.cpu().numpy()) for s, e, w, f in parts]
    eig, flag = shard.assemble(parts, ns)
    rep = lo.ragged_batch_parity(buf, ns, offs, eig, eoffs, flag, subset=1200)
    assert rep["flag_mismatch"] == 0 and rep["gpu_flagged"] == 0, rep
    assert rep["max_rel_err"] <= lo.TOL_REL_FRO, rep
