"""GPU results against the committed golden fixtures (LAPACK outputs and exact spectra)."""
import os

import numpy as np
import pytest

from oracle import lapack_oracle as lo

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "zgeev_golden.npz")


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def gpu_eigs(A_np, lanes=0):
    import torch

    from tokura_zgeev_batched_gb300 import api

    h = api.Handle()
    n = A_np.shape[-1]
    if lanes:
        assert h.set_plain_config(n, lanes, 128) == 0
    A = torch.from_numpy(np.ascontiguousarray(A_np)).cuda()
    w, f = api.zgeev_batched(A, handle=h)
    torch.cuda.synchronize()
    return w.cpu().numpy(), f.cpu().numpy()


@pytest.mark.parametrize("lanes", [1, 2, 4, 8])
def test_golden_cases(cuda, golden, lanes):
    for name in [str(x) for x in golden["names"]]:
        A = golden[f"{name}/A"]
        w_ref = golden[f"{name}/w"]
        info = golden[f"{name}/info"]
        w, f = gpu_eigs(A, lanes)
        assert np.array_equal(f != 0, info != 0), name
        fro = np.sqrt(np.sum(np.abs(A) ** 2, axis=(1, 2)))
        fro = np.where(fro == 0, 1.0, fro)
        cond = 1.0 / np.maximum(golden[f"{name}/rconde"], 1e-300)
        err = lo.matched_abs_errors(w, w_ref).max(axis=1) / fro
        well = cond.max(axis=1) <= lo.COND_MAX
        assert np.all(err[well] <= lo.TOL_REL_FRO), (name, err)
        if name.startswith("jordan"):
            n = A.shape[-1]
            assert err.max() <= 10 * 2.2e-16 ** (1.0 / n), name
        key = f"{name}/exact"
        if key in golden.files:
            e = lo.matched_abs_errors(w, golden[key]).max(axis=1) / fro
            if not name.startswith("jordan"):
                assert np.all(e[well] <= lo.TOL_REL_FRO), (name, e)
