"""GPU parity at configuration scale: every matrix of a 10,000-matrix batch of order 32 (the
small-batch configuration's size) and 2,000 companion matrices per order, against LAPACK zgeev,
flags included (the reference's own check compares every matrix,
stream_test_with_MKL/main.cu:92-181)."""
import numpy as np
import pytest

from oracle import lapack_oracle as lo
from tokura_zgeev_batched_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def solve(A_np):
    import torch
    from tokura_zgeev_batched_gb300 import zgeev_batched

    A = torch.from_numpy(np.ascontiguousarray(A_np)).cuda()
    w, f = zgeev_batched(A)
    torch.cuda.synchronize()
    return w.cpu().numpy(), f.cpu().numpy()


def test_config1_size_every_matrix(cuda):
    """10,000 complex Gaussian 32x32 matrices: all matched against LAPACK (tolerance
    1e-11*||A||_F on eigenvalue condition numbers <= 1e3), identical flags on all."""
    A = wl.gaussian(10000, 32, seed=20261204)
    w, f = solve(A)
    rep = lo.batch_parity(A, w, f, subset=10000, seed=0)
    assert rep["checked"] == 10000 and rep["flags_checked"] == 10000
    assert rep["flag_mismatch"] == 0 and rep["lapack_fail"] == 0, rep
    assert rep["well_conditioned"] >= 9000, rep
    assert rep["max_rel_err_well"] <= lo.TOL_REL_FRO, rep
    assert rep["max_rel_err"] <= 1e-10, rep  # every matrix, ill-conditioned ones included


@pytest.mark.parametrize("n", [16, 32, 48, 64])
def test_companion_2000_per_order(cuda, n):
    """Companion matrices of monic polynomials with complex Gaussian coefficients stress
    deflation and the convergence flag: 2,000 per order, flags identical to LAPACK's."""
    A = wl.companion(2000, n, seed=4000 + n)
    w, f = solve(A)
    rep = lo.batch_parity(A, w, f, subset=2000, seed=1)
    assert rep["checked"] == 2000
    assert rep["flag_mismatch"] == 0, rep
    if rep["well_conditioned"]:
        assert rep["max_rel_err_well"] <= lo.TOL_REL_FRO, rep
