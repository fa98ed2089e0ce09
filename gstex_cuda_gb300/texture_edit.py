"""Texture editing (mirror of gstex_cuda/texture_edit.py).

``texture_edit`` keeps the reference's signature (gstex_cuda/texture_edit.py:
14-140): it bins the Gaussians like the renderer and splats an edited image
back into the texels, returning ``updated_texture`` [sum h*w, 5] whose
channels are r*a, g*a, b*a, a (each weighted by the bilinear intersection
weights) and the total weight.  Not differentiable, like the reference's.
"""
from __future__ import annotations

from typing import Optional, Tuple

import torch
from torch import Tensor

from . import cuda as _C
from .utils import bin_and_sort_gaussians, compute_cumulative_intersects


def texture_edit(texture_info: Tuple[int, int, int], texture_dims: Tensor, updated_img: Tensor,
                 updated_alpha: Tensor, depth_lower: Tensor, depth_upper: Tensor, centers: Tensor, extents: Tensor,
                 depths: Tensor, num_tiles_hit: Tensor, opacity: Tensor, means: Tensor, scales: Tensor, glob_scale,
                 quats: Tensor, uv0: Tensor, umap: Tensor, vmap: Tensor, viewmat: Tensor, c2w: Tensor, fx: float,
                 fy: float, cx: float, cy: float, img_height: int, img_width: int, block_width: int, settings: int,
                 background: Optional[Tensor] = None, use_torch_impl: bool = False) -> Tensor:
    """Splat ``updated_img`` (where ``updated_alpha`` > 0 and the hit's camera
    depth lies in [depth_lower, depth_upper]) into the Gaussians' textures.

    ``texture_info[2]`` must be 5.  Settings bit 0 selects the blur filter
    (bit 9 in the renderer).  ``background`` and ``c2w`` are not used."""
    assert 1 < block_width <= 16, "block_width must be between 2 and 16"
    if use_torch_impl:
        raise NotImplementedError("texture_edit has only a CUDA implementation (as in the reference)")
    num_points = centers.size(0)
    tile_bounds = ((img_width + block_width - 1) // block_width, (img_height + block_width - 1) // block_width, 1)
    block = (block_width, block_width, 1)
    img_size = (img_width, img_height, 1)
    texture_total_size = int(torch.sum(texture_dims[:, 0].long() * texture_dims[:, 1].long()).item())
    num_intersects, cum_tiles_hit = compute_cumulative_intersects(num_tiles_hit)
    if num_intersects < 1:
        raise ValueError("texture_edit: no Gaussian intersects the image")
    _, _, _, gaussian_ids_sorted, tile_bins = bin_and_sort_gaussians(
        num_points, num_intersects, centers, extents, depths, cum_tiles_hit, tile_bounds, block_width)
    if background is None:
        background = torch.zeros(3, device=means.device)
    return _C.texture_edit(tile_bounds, block, img_size, texture_info, texture_total_size, texture_dims.contiguous(),
                           updated_img.contiguous(), updated_alpha.contiguous(), depth_lower.contiguous(),
                           depth_upper.contiguous(), gaussian_ids_sorted, tile_bins, opacity.contiguous(),
                           means.contiguous(), scales.contiguous(), glob_scale, quats.contiguous(),
                           uv0.contiguous(), umap.contiguous(), vmap.contiguous(), viewmat.contiguous(),
                           c2w.contiguous(), fx, fy, cx, cy, settings, background.contiguous())
