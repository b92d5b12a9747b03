"""Python wrappers without a GPU: inputs they cannot hand to the library are
rejected before any device call, and there is no CPU fallback (a handle cannot
be created without a device)."""
import pytest
import torch

from tokura_zgeev_batched_gb300 import api

no_gpu = pytest.mark.skipif(torch.cuda.is_available(), reason="checks the behaviour without a GPU")


def test_wrappers_reject_host_tensors():
    with pytest.raises(TypeError):
        api.zgeev_batched(torch.zeros(2, 3, 3, dtype=torch.complex128))
    with pytest.raises(TypeError):
        api.zgeev_strided(torch.zeros(2, 3, 3, dtype=torch.complex128))
    with pytest.raises(TypeError):
        api.cgeev_batched(torch.zeros(2, 3, 3, dtype=torch.complex64))
    with pytest.raises(TypeError):
        api.dgeev_batched(torch.zeros(2, 3, 3, dtype=torch.float64))
    with pytest.raises(TypeError):
        api.zgeev_ragged(torch.zeros(9, dtype=torch.complex128), torch.tensor([3], dtype=torch.int32))


def test_wrappers_reject_wrong_dtypes_and_shapes():
    with pytest.raises(TypeError):
        api.zgeev_batched(torch.zeros(2, 3, 3, dtype=torch.complex64))
    with pytest.raises(TypeError):
        api.dgeev_batched(torch.zeros(2, 3, 3, dtype=torch.int32))
    with pytest.raises(TypeError):  # the strided wrapper takes one 3-D batch
        api.zgeev_strided(torch.zeros(3, 3, dtype=torch.complex128))
    with pytest.raises(TypeError):
        api.zgeev_ragged(torch.zeros(3, 3, dtype=torch.complex128), torch.tensor([3], dtype=torch.int32))


def test_pointer_wrapper_needs_matrices():
    with pytest.raises(ValueError):
        api.zgeev_pointers([])
    with pytest.raises(ValueError):
        api.zgeev_pointers([None, None])
    with pytest.raises(ValueError):  # mixed orders
        api.zgeev_pointers([torch.zeros(3, 3, dtype=torch.complex128), torch.zeros(4, 4, dtype=torch.complex128)])


@no_gpu
def test_no_handle_without_a_device():
    with pytest.raises(RuntimeError):
        api.Handle()
