"""Projection entry points (mirror of gstex_cuda/get_aabb_2d.py of the reference)."""
from __future__ import annotations

import torch

from . import _torch_impl as _T
from . import cuda as _C


def merge_aabbs(centers1, extents1, centers2, extents2):
    """Union of two sets of boxes (gstex_cuda/get_aabb_2d.py:15-20)."""
    lower = torch.minimum(centers1 - extents1, centers2 - extents2)
    upper = torch.maximum(centers1 + extents1, centers2 + extents2)
    return 0.5 * (lower + upper), 0.5 * (upper - lower)


def project_points(points, viewmat, intrins, clip=False):
    """Pixel positions and camera depths of points (gstex_cuda/get_aabb_2d.py:22-32).
    The depths are the per-Gaussian sort keys of the binning stage."""
    view_points = points @ viewmat.T[:3, :3] + viewmat.T[3:, :3]
    if clip:
        with torch.no_grad():
            view_points[:, -1] = torch.clamp(view_points[:, -1], min=0.01, max=1000.0)
    pix = _T.project_pix(intrins[:2], view_points, intrins[2:])
    return pix, view_points[:, -1]


def get_aabb_2d_torch(means, scales, glob_scale, quats, viewmat, intrins):
    """Torch formulation of the AABB kept from the reference (get_aabb_2d.py:34-54);
    it clamps corner depths to [0.01, 1000] and has no near-plane cull."""
    ell = 3.0 * glob_scale
    Rs = _T.normalized_quat_to_rotmat(quats)
    corners = torch.stack([
        means + ell * scales[:, None, 0] * Rs[:, :, 0] + ell * scales[:, None, 1] * Rs[:, :, 1],
        means + ell * scales[:, None, 0] * Rs[:, :, 0] - ell * scales[:, None, 1] * Rs[:, :, 1],
        means - ell * scales[:, None, 0] * Rs[:, :, 0] + ell * scales[:, None, 1] * Rs[:, :, 1],
        means - ell * scales[:, None, 0] * Rs[:, :, 0] - ell * scales[:, None, 1] * Rs[:, :, 1],
    ], dim=1)
    shp = corners.shape
    pc = project_points(corners.reshape(-1, 3), viewmat, intrins, clip=True)[0].reshape(shp[0], shp[1], 2)
    mx = torch.max(pc, dim=1)[0]
    mn = torch.min(pc, dim=1)[0]
    return 0.5 * (mx + mn), 0.5 * (mx - mn)


def get_aabb_2d(means, scales, glob_scale, quats, viewmat, intrins):
    """Screen AABB of each splat's +-3 sigma rectangle (CUDA; csrc/get_aabb_2d.cu:11-89)."""
    fx, fy, cx, cy = intrins
    return _C.get_aabb_2d(means.contiguous(), scales.contiguous(), glob_scale, quats.contiguous(),
                          viewmat.contiguous(), fx, fy, cx, cy)


def get_num_tiles_hit_2d(centers, extents, img_height, img_width, block_width):
    """Tiles overlapped by each AABB, bit-exact with gstex_cuda/get_aabb_2d.py:70-91 (CUDA)."""
    return _C.num_tiles_hit(centers.contiguous(), extents.contiguous(), img_height, img_width, block_width)
