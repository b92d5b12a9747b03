"""Multi-rank bench path on CPU: two gloo ranks, max-over-ranks timing and per-rank data (weak scaling)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    ws, r, local = bench.dist_env()
    t = bench.max_over_ranks(10.0 + rank, dist, torch.device("cpu"))
    seed = bench.rank_seed(bench.SEED, r)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, ws, r, local, t, seed))


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get() for _ in range(2))
    assert [x[0] for x in res] == [0, 1]
    assert all(x[1] == 2 and x[0] == x[2] == x[3] for x in res)
    assert all(x[4] == 11.0 for x in res)           # every rank sees the slowest rank's time
    assert res[0][5] != res[1][5]                   # each rank generates its own batch


def test_reference_arm_other_ranks_exit_quietly(capsys, monkeypatch):
    import bench

    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")

    class Args:
        steps, warmup = 1, 1

    bench.run_reference(Args())
    assert capsys.readouterr().out == ""
