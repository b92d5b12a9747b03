"""The plain path at 16 and 32 lanes per matrix (small batches).

A batch too small to fill the GPU at four lanes per matrix spreads each matrix
over more lanes, up to n/2 and 32 (one warp per matrix). Every width must agree
with LAPACK zgeev (the oracle) with identical flags, with and without shift
hints, and the launch-shape heuristic must pick the widths that measured best.
"""
import pytest

from oracle import lapack_oracle as lo
from tokura_zgeev_batched_gb300 import api
from tokura_zgeev_batched_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("lanes", [16, 32])
@pytest.mark.parametrize("n", [3, 17, 40, 64])
@pytest.mark.parametrize("hints", [0, 1])
def test_wide_lanes_match_lapack(cuda, lanes, n, hints):
    import torch

    A_np = wl.GENERATORS["companion" if n == 40 else "gaussian"](77, n, seed=60 + n)
    h = api.Handle()
    assert h.set_plain_config(n, lanes, 64) == 0
    assert h.set_shift_hints(hints) == 0
    w, f = api.zgeev_batched(torch.from_numpy(A_np).cuda(), handle=h)
    rep = lo.parity_report(A_np, w.cpu().numpy(), f.cpu().numpy())
    assert rep["flag_mismatch"] == 0, rep["flag_mismatch"]
    if rep["well_conditioned"]:
        assert rep["max_rel_err_well"] <= lo.TOL_REL_FRO, rep["max_rel_err_well"]


def test_heuristic_widens_small_batches(cuda):
    import torch

    sms = torch.cuda.get_device_properties(0).multi_processor_count
    want = sms * 4 * 2 * 32  # lanes that give every SM sub-partition two warps
    h = api.Handle()
    assert h.plain_config(64, want)[0] == 1
    assert h.plain_config(32, want // 4)[0] == 4
    assert h.plain_config(64, 2 * sms)[0] == 32  # two matrices per SM: one warp each
    assert h.plain_config(64, want // 16)[0] == 16
    assert h.plain_config(32, want // 32)[0] == 16  # capped at n / 2
    assert h.plain_config(16, 100)[0] == 8
    assert h.plain_config(2, 10)[0] == 1
