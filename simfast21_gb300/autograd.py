"""torch.autograd wrapper of the criterion C(x) = max_R ion_R / rec_R.

For checks only (gradient tests, the differentiation benchmark): the forward
and the hand-written adjoint are the library's C-ABI calls
(sf21_hii_criterion_device / sf21_hii_vjp_device); torch provides device
memory, the stream and the chain rule of whatever loss is put on top.
"""
from __future__ import annotations

import torch

from .hii import SF21_SRC_SFRD, FilterBank


class Criterion(torch.autograd.Function):
    """C = Criterion.apply(delta, src, zeta, bank, z, set, src_kind).

    delta, src: contiguous float32 CUDA tensors (N, N, N); zeta: a 0-d
    tensor holding the set's fesc (the bank was created with that value);
    returns C (float32, N^3).  backward returns dL/d delta, dL/d src, dL/d zeta."""

    @staticmethod
    def forward(ctx, delta, src, zeta, bank: FilterBank, z: float, set_index: int = 0,
                src_kind: int = SF21_SRC_SFRD):
        assert delta.is_cuda and delta.dtype == torch.float32 and delta.is_contiguous()
        assert src.is_cuda and src.dtype == torch.float32 and src.is_contiguous()
        C = torch.empty_like(delta)
        A = torch.empty(delta.shape, dtype=torch.uint8, device=delta.device)
        stream = torch.cuda.current_stream(delta.device).cuda_stream
        bank.criterion_device(z, delta.data_ptr(), src.data_ptr(), C.data_ptr(), A.data_ptr(), s=set_index,
                              src_kind=src_kind, stream=stream)
        ctx.save_for_backward(delta, src)
        ctx.bank, ctx.z, ctx.set_index, ctx.src_kind = bank, z, set_index, src_kind
        ctx.mark_non_differentiable(A)
        return C

    @staticmethod
    def backward(ctx, gC):
        delta, src = ctx.saved_tensors
        gC = gC.contiguous().to(torch.float32)
        gd = torch.empty_like(delta)
        gs = torch.empty_like(src)
        stream = torch.cuda.current_stream(delta.device).cuda_stream
        gz = ctx.bank.vjp_device(ctx.z, delta.data_ptr(), src.data_ptr(), gC.data_ptr(), gd.data_ptr(),
                                 gs.data_ptr(), s=ctx.set_index, src_kind=ctx.src_kind, stream=stream)
        return gd, gs, torch.tensor(gz, dtype=torch.float64, device=delta.device), None, None, None, None
