"""torch.autograd bindings of the differentiable mode.

``eigvals(A)`` and ``eigvals_ragged(A_packed, n, offsets)`` return eigenvalues
computed by the sm_103a forward kernels and differentiate through the
hand-written backward kernels (``tokura_zgeev_backward_gpu`` /
``tokura_zgeev_ragged_backward_gpu``). Only A and the eigenvalues are saved for
the backward, which recomputes the Schur form. Gradients follow torch's
convention for complex tensors and match ``torch.linalg.eigvals``'s backward.
Both are CUDA-graph capturable when the caller provides static workspaces.
"""
from __future__ import annotations

import torch

from . import api


class _EigvalsFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, A, handle):
        eig, flag = api.zgeev_batched(A, handle=handle)
        ctx.save_for_backward(A, eig)
        ctx.handle = handle
        ctx.mark_non_differentiable(flag)
        return eig, flag

    @staticmethod
    def backward(ctx, g_eig, g_flag):
        A, eig = ctx.saved_tensors
        if g_eig is None:
            return None, None
        gA, _ = api.zgeev_backward(A, eig, g_eig, handle=ctx.handle)
        return gA, None


def eigvals(A: torch.Tensor, handle: api.Handle | None = None, return_flag: bool = False):
    """Differentiable eigenvalues of complex128 CUDA matrices ``A[..., n, n]``."""
    eig, flag = _EigvalsFunction.apply(A, handle)
    return (eig, flag) if return_flag else eig


class _RaggedEigvalsFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, A_packed, n, offsets, handle, work_fwd, work_bwd, total_eig):
        eig, flag = api.zgeev_ragged(A_packed, n, offsets=offsets, handle=handle, work=work_fwd,
                                     total_eigenvalues=total_eig)
        ctx.save_for_backward(A_packed, n, offsets, eig)
        ctx.handle = handle
        ctx.work_bwd = work_bwd
        ctx.mark_non_differentiable(flag)
        return eig, flag

    @staticmethod
    def backward(ctx, g_eig, g_flag):
        A, n, offsets, eig = ctx.saved_tensors
        if g_eig is None:
            return None, None, None, None, None, None, None
        batch = n.numel()
        total = A.numel()
        work = ctx.work_bwd
        need = api.tokura_get_zgeev_ragged_backward_workspacesize(batch, total)
        if work is None or work.numel() * work.element_size() < need:
            work = torch.empty(need, dtype=torch.uint8, device=A.device)
        gA = torch.empty_like(A)
        flag = torch.empty(batch, dtype=torch.int8, device=A.device)
        g = g_eig.to(torch.complex128).contiguous()
        h = ctx.handle if ctx.handle is not None else api.default_handle()
        st = api.tokura_zgeev_ragged_backward_gpu(h, batch, n.data_ptr(), offsets.data_ptr(), None, total,
                                                  A.data_ptr(), eig.data_ptr(), g.data_ptr(), gA.data_ptr(),
                                                  work.data_ptr(), flag.data_ptr(),
                                                  torch.cuda.current_stream(A.device).cuda_stream)
        if st != 0:
            raise RuntimeError(f"tokura_zgeev_ragged_backward_gpu returned {st}")
        return gA, None, None, None, None, None, None


def eigvals_ragged(A_packed: torch.Tensor, n: torch.Tensor, offsets: torch.Tensor | None = None,
                   handle: api.Handle | None = None, work_fwd=None, work_bwd=None, return_flag: bool = False,
                   total_eigenvalues: int | None = None):
    """Differentiable eigenvalues of a packed ragged batch (eigenvalues packed by the prefix sum of n).

    With ``offsets``, ``total_eigenvalues`` and both workspaces given, forward and
    backward run without host synchronisation or allocation inside the library,
    so a training step can be captured in a CUDA graph.
    """
    n = n.to(device=A_packed.device, dtype=torch.int32).contiguous()
    if offsets is None:
        n64 = n.to(torch.int64)
        offsets = torch.cumsum(n64 * n64, 0) - n64 * n64
    offsets = offsets.to(device=A_packed.device, dtype=torch.int64).contiguous()
    eig, flag = _RaggedEigvalsFunction.apply(A_packed, n, offsets, handle, work_fwd, work_bwd, total_eigenvalues)
    return (eig, flag) if return_flag else eig
