"""GPU parity of the plain entry point against LAPACK zgeev (the oracle)."""
import numpy as np
import pytest

from oracle import lapack_oracle as lo
from tokura_zgeev_batched_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def run_gpu(A_np):
    import torch
    from tokura_zgeev_batched_gb300 import zgeev_batched

    A = torch.from_numpy(np.ascontiguousarray(A_np)).cuda()
    A0 = A.clone()
    w, f = zgeev_batched(A)
    torch.cuda.synchronize()
    assert torch.equal(A, A0), "A must not be modified"
    return w.cpu().numpy(), f.cpu().numpy()


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 7, 8, 12, 16, 23, 32, 33, 48, 63, 64])
def test_gaussian_all_sizes(cuda, n):
    A = wl.gaussian(300, n, seed=1000 + n)
    w, f = run_gpu(A)
    rep = lo.parity_report(A, w, f)
    assert rep["flag_mismatch"] == 0
    assert (f == 0).all()
    assert rep["max_rel_err_well"] <= lo.TOL_REL_FRO, rep


@pytest.mark.parametrize("cls", ["vdv", "companion", "uniform"])
@pytest.mark.parametrize("n", [4, 16, 32, 64])
def test_classes(cuda, cls, n):
    A = wl.GENERATORS[cls](200, n, seed=7 + n)
    w, f = run_gpu(A)
    rep = lo.parity_report(A, w, f)
    assert rep["flag_mismatch"] == 0, rep
    if rep["well_conditioned"]:
        assert rep["max_rel_err_well"] <= lo.TOL_REL_FRO, {k: v for k, v in rep.items() if k != "rel_err"}
