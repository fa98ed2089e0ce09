"""Device-side parameter activation for GStex training steps.

``preprocess`` replaces the per-step preprocessing of the reference's demo
trainer (example.py:126-143: exp of the log-scales with the third scale tied
to 1e-5 of their mean, quaternion normalisation, the chart maps rotated by
theta and scaled by exp(log-scale), and the opacity sigmoid of
example.py:155-171) by one CUDA kernel forward and one backward, as a
``torch.autograd.Function``.
"""
from __future__ import annotations

from typing import Optional

import torch
from torch import Tensor
from torch.autograd import Function

from . import _lib
from ._lib import check, ptr


def _need(name, t, shape_tail):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise _lib.GstexError(f"{name} must be a CUDA tensor")
    if t.dtype != torch.float32:
        raise _lib.GstexError(f"{name} must be float32")
    if tuple(t.shape[1:]) != tuple(shape_tail):
        raise _lib.GstexError(f"{name} must be [N, {', '.join(map(str, shape_tail))}], got {tuple(t.shape)}")
    return t.contiguous()


class _Preprocess(Function):
    @staticmethod
    def forward(ctx, raw_scales, raw_quats, mapping, raw_opacity):
        N = raw_scales.shape[0]
        P = mapping.shape[1]
        raw_scales = _need("raw_scales", raw_scales, (3,))
        raw_quats = _need("raw_quats", raw_quats, (4,))
        mapping = _need("mapping", mapping, (P, 4))
        ro = None
        if raw_opacity is not None:
            ro = raw_opacity.contiguous()
            if ro.numel() != N:
                raise _lib.GstexError("raw_opacity must have N entries")
        f32 = dict(dtype=torch.float32, device=raw_scales.device)
        scales, quats = torch.empty((N, 3), **f32), torch.empty((N, 4), **f32)
        uv0, umap, vmap = torch.empty((N, P, 2), **f32), torch.empty((N, P, 3), **f32), torch.empty((N, P, 3), **f32)
        opacity = torch.empty((N, 1), **f32) if ro is not None else None
        check(_lib.lib().gstex_preprocess_forward(N, P, ptr(raw_scales), ptr(raw_quats), ptr(mapping), ptr(ro),
                                                  ptr(scales), ptr(quats), ptr(uv0), ptr(umap), ptr(vmap),
                                                  ptr(opacity), _lib.stream_of(raw_scales)), "preprocess_forward")
        ctx.save_for_backward(raw_scales, raw_quats, mapping, ro if ro is not None else torch.empty(0))
        ctx.has_opacity = ro is not None
        return scales, quats, uv0, umap, vmap, opacity

    @staticmethod
    def backward(ctx, v_scales, v_quats, v_uv0, v_umap, v_vmap, v_opacity):
        raw_scales, raw_quats, mapping, ro = ctx.saved_tensors
        ro = ro if ctx.has_opacity else None
        N, P = raw_scales.shape[0], mapping.shape[1]
        c = lambda t: t.contiguous() if t is not None else None  # noqa: E731
        g_scales, g_quats = torch.empty_like(raw_scales), torch.empty_like(raw_quats)
        g_map = torch.empty_like(mapping)
        g_op = torch.empty_like(ro) if ro is not None else None
        check(_lib.lib().gstex_preprocess_backward(
            N, P, ptr(raw_scales), ptr(raw_quats), ptr(mapping), ptr(ro), ptr(c(v_scales)), ptr(c(v_quats)),
            ptr(c(v_uv0)), ptr(c(v_umap)), ptr(c(v_vmap)), ptr(c(v_opacity)), ptr(g_scales), ptr(g_quats),
            ptr(g_map), ptr(g_op), _lib.stream_of(raw_scales)), "preprocess_backward")
        return g_scales, g_quats, g_map, g_op


def preprocess(raw_scales: Tensor, raw_quats: Tensor, mapping: Tensor, raw_opacity: Optional[Tensor] = None):
    """(scales, quats, uv0, umap, vmap, opacity) from the trainer's raw
    parameters: raw_scales [N,3] (log, first two used), raw_quats [N,4] (wxyz,
    any norm), mapping [N,P,4] (uv0 x, uv0 y, log uv-scale, theta),
    raw_opacity [N] or [N,1] (logit) or None.  Differentiable."""
    return _Preprocess.apply(raw_scales, raw_quats, mapping, raw_opacity)
