"""Differentiable jagged-chart sampling (mirror of gstex_cuda/texture_sample.py).

Unlike the reference, whose autograd backward returns no gradients
(gstex_cuda/texture_sample.py:70-78), this one returns the texel gradients
and, when uvs require grad, the uv gradients.
"""
from __future__ import annotations

from torch import Tensor
from torch.autograd import Function

from . import cuda as _C


def texture_sample(texture_info, texture_dims, texture, uvs, use_torch_impl: bool = False) -> Tensor:
    """Bilinear lookups [Q, C] of Q queries; uvs are clamped to [0,1]^2."""
    if use_torch_impl:
        raise NotImplementedError("gstex_cuda_gb300 has no PyTorch sampling path; use_torch_impl must be False")
    return _TextureSample.apply(texture_info, texture_dims.contiguous(), texture.contiguous(), uvs.contiguous())


class _TextureSample(Function):
    @staticmethod
    def forward(ctx, texture_info, texture_dims, texture, uvs):
        ctx.texture_info = texture_info
        ctx.save_for_backward(texture_dims, texture, uvs)
        return _C.texture_sample_forward(texture_info, texture_dims, uvs, texture)

    @staticmethod
    def backward(ctx, v_out):
        texture_dims, texture, uvs = ctx.saved_tensors
        need_uv = ctx.needs_input_grad[3]
        if not (ctx.needs_input_grad[2] or need_uv):
            return None, None, None, None
        res = _C.texture_sample_backward(ctx.texture_info, texture_dims, uvs, texture, v_out.contiguous(),
                                         need_uv_grad=need_uv)
        v_tex, v_uvs = (res if need_uv else (res, None))
        return None, None, (v_tex if ctx.needs_input_grad[2] else None), v_uvs
