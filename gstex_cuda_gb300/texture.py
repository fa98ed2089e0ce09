"""Textured 2D-Gaussian rasterisation (mirror of gstex_cuda/texture.py).

``texture_gaussians`` keeps the reference's signature and return value
(gstex_cuda/texture.py:14-150): a 6-tuple (img, depth, reg, alpha, texture,
normal).  Binning, compositing and the hand-written adjoint run on the CUDA
library; the hot path has no PyTorch or CPU fallback.
"""
from __future__ import annotations

from typing import Optional, Tuple

import torch
from torch import Tensor
from torch.autograd import Function

from . import cuda as _C
from .utils import bin_and_sort_gaussians, compute_cumulative_intersects


def texture_gaussians(texture_info: Tuple[int, int, int], texture_dims: Tensor, centers: Tensor, extents: Tensor,
                      depths: Tensor, num_tiles_hit: Tensor, colors: Tensor, opacity: Tensor, means: Tensor,
                      scales: Tensor, glob_scale, quats: Tensor, uv0: Tensor, umap: Tensor, vmap: Tensor,
                      texture: Tensor, viewmat: Tensor, c2w: Tensor, fx: float, fy: float, cx: float, cy: float,
                      img_height: int, img_width: int, block_width: int, settings: int,
                      background: Optional[Tensor] = None, use_torch_impl: bool = False):
    """Rasterise textured 2D Gaussians.

    Differentiable w.r.t. colors, opacity, means, scales, quats, uv0, umap,
    vmap and texture.  ``texture`` is float32 [T, C] (C = texture_info[2],
    at most 64) or bfloat16 [T, 4] holding 3 channels padded to 4.

    Returns (out_img, out_depth, out_reg, out_alpha, out_texture, out_normal).
    """
    assert 1 < block_width <= 16, "block_width must be between 2 and 16"
    if use_torch_impl:
        raise NotImplementedError("gstex_cuda_gb300 renders on the GPU only; use_torch_impl must be False")
    if colors.dtype == torch.uint8:
        colors = colors.float() / 255
    if background is not None:
        assert background.shape[0] == colors.shape[-1], \
            f"incorrect shape of background color tensor, expected shape {colors.shape[-1]}"
    else:
        background = torch.ones(colors.shape[-1], dtype=torch.float32, device=colors.device)
    if colors.ndimension() != 2:
        raise ValueError("colors must have dimensions (N, D)")
    return _TextureGaussians.apply(
        texture_info, texture_dims.contiguous(), centers.contiguous(), extents.contiguous(), depths.contiguous(),
        num_tiles_hit.contiguous(), colors.contiguous(), opacity.contiguous(), means.contiguous(),
        scales.contiguous(), glob_scale, quats.contiguous(), uv0.contiguous(), umap.contiguous(), vmap.contiguous(),
        texture.contiguous(), viewmat.contiguous(), c2w.contiguous(), fx, fy, cx, cy, img_height, img_width,
        block_width, settings, background.contiguous())


class _TextureGaussians(Function):
    @staticmethod
    def forward(ctx, texture_info, texture_dims, centers, extents, depths, num_tiles_hit, colors, opacity, means,
                scales, glob_scale, quats, uv0, umap, vmap, texture, viewmat, c2w, fx, fy, cx, cy, img_height,
                img_width, block_width, settings, background):
        num_points = centers.size(0)
        tile_bounds = ((img_width + block_width - 1) // block_width, (img_height + block_width - 1) // block_width, 1)
        block = (block_width, block_width, 1)
        img_size = (img_width, img_height, 1)
        num_intersects, cum_tiles_hit = compute_cumulative_intersects(num_tiles_hit)
        dev = centers.device
        if num_intersects < 1:
            # No splat touches the image.  (The reference's branch for this case,
            # gstex_cuda/texture.py:197-205, leaves most outputs undefined.)
            gaussian_ids_sorted = torch.zeros(0, dtype=torch.int32, device=dev)
            tile_bins = torch.zeros(tile_bounds[0] * tile_bounds[1], 2, dtype=torch.int32, device=dev)
        else:
            _, _, _, gaussian_ids_sorted, tile_bins = bin_and_sort_gaussians(
                num_points, num_intersects, centers, extents, depths, cum_tiles_hit, tile_bounds, block_width)
        outs = _C.texture_forward(tile_bounds, block, img_size, texture_info, texture_dims, gaussian_ids_sorted,
                                  tile_bins, colors, opacity, means, scales, glob_scale, quats, uv0, umap, vmap,
                                  texture, viewmat, c2w, fx, fy, cx, cy, settings, background)
        out_img, out_depth, out_reg, out_texture, out_normal, final_Ts, final_idx, depth_idx, out_reg_s = outs
        ctx.img_width, ctx.img_height = img_width, img_height
        ctx.texture_info = texture_info
        ctx.fx, ctx.fy, ctx.cx, ctx.cy = fx, fy, cx, cy
        ctx.glob_scale = glob_scale
        ctx.num_intersects = num_intersects
        ctx.block_width = block_width
        ctx.settings = settings
        ctx.save_for_backward(texture_dims, gaussian_ids_sorted, tile_bins, colors, opacity, means, scales, quats,
                              uv0, umap, vmap, texture, viewmat, c2w, background, final_Ts, final_idx, depth_idx,
                              out_reg_s)
        out_alpha = 1 - final_Ts
        return out_img, out_depth, out_reg, out_alpha, out_texture, out_normal

    @staticmethod
    def backward(ctx, v_out_img, v_out_depth, v_out_reg, v_out_alpha, v_out_texture, v_out_normal):
        (texture_dims, gaussian_ids_sorted, tile_bins, colors, opacity, means, scales, quats, uv0, umap, vmap,
         texture, viewmat, c2w, background, final_Ts, final_idx, depth_idx, out_reg_s) = ctx.saved_tensors

        def g(t, like):
            return torch.zeros_like(like) if t is None else t.contiguous()

        v_out_img = g(v_out_img, final_Ts.unsqueeze(-1).expand(*final_Ts.shape, 3))
        v_out_depth = g(v_out_depth, final_Ts)
        v_out_reg = g(v_out_reg, final_Ts)
        v_out_alpha = g(v_out_alpha, final_Ts)
        C = int(ctx.texture_info[2])
        v_out_texture = g(v_out_texture, final_Ts.new_zeros(*final_Ts.shape, C))
        v_out_normal = g(v_out_normal, final_Ts.new_zeros(*final_Ts.shape, 3))
        if ctx.num_intersects < 1:
            grads = [torch.zeros_like(t) for t in (colors, opacity, means, scales, quats, uv0, umap, vmap, texture)]
        else:
            grads = _C.texture_backward(
                ctx.img_height, ctx.img_width, ctx.block_width, ctx.texture_info, texture_dims, gaussian_ids_sorted,
                tile_bins, colors, opacity, means, scales, ctx.glob_scale, quats, uv0, umap, vmap, texture, viewmat,
                c2w, ctx.fx, ctx.fy, ctx.cx, ctx.cy, ctx.settings, background, final_Ts, final_idx, depth_idx,
                out_reg_s, v_out_img, v_out_depth, v_out_reg, v_out_alpha, v_out_texture, v_out_normal)
        v_colors, v_opacity, v_means, v_scales, v_quats, v_uv0, v_umap, v_vmap, v_texture = grads
        return (None, None, None, None, None, None, v_colors, v_opacity, v_means, v_scales, None, v_quats, v_uv0,
                v_umap, v_vmap, v_texture, None, None, None, None, None, None, None, None, None, None, None)
