"""The native operator surface of the reference extension, on the GB300 library.

Same names, argument order and return values as the ops the reference binds
in gstex_cuda/cuda/csrc/ext.cpp:8-25 (and looks up in
gstex_cuda/cuda/__init__.py:4-27): torch tensors in, freshly allocated torch
tensors out, launched on the current torch stream.  Like the reference's
CHECK_INPUT (csrc/bindings.h:10-17) every tensor must be a contiguous CUDA
tensor; there is no CPU path.
"""
from __future__ import annotations

import ctypes
from typing import Tuple

import torch

from . import _lib
from ._lib import check, ptr

TEXTURE_FP32 = 0
TEXTURE_BF16X4 = 1


def _chk(*named):
    for name, t in named:
        if t is None:
            continue
        if not isinstance(t, torch.Tensor):
            raise TypeError(f"{name} must be a torch.Tensor")
        if not t.is_cuda:
            raise _lib.GstexError(f"{name} must be a CUDA tensor")
        if not t.is_contiguous():
            raise _lib.GstexError(f"{name} must be contiguous")


def _f32(name, t):
    if t.dtype != torch.float32:
        raise _lib.GstexError(f"{name} must be float32, got {t.dtype}")


def _i32(name, t):
    if t.dtype != torch.int32:
        raise _lib.GstexError(f"{name} must be int32, got {t.dtype}")


def num_sh_bases(degree: int) -> int:
    return {0: 1, 1: 4, 2: 9, 3: 16}.get(degree, 25)


# ---------------------------------------------------------------------------
# SH (csrc/bindings.cu:18-75)
# ---------------------------------------------------------------------------
def compute_sh_forward(num_points, degree, degrees_to_use, viewdirs, coeffs):
    _chk(("viewdirs", viewdirs), ("coeffs", coeffs))
    _f32("viewdirs", viewdirs)
    _f32("coeffs", coeffs)
    nb = num_sh_bases(degree)
    if coeffs.ndim != 3 or coeffs.shape[0] != num_points or coeffs.shape[1] != nb or coeffs.shape[2] != 3:
        raise RuntimeError("coeffs must have dimensions (N, D, 3)")
    colors = torch.empty((num_points, 3), dtype=torch.float32, device=coeffs.device)
    check(_lib.lib().gstex_compute_sh_forward(num_points, degree, degrees_to_use, ptr(viewdirs), ptr(coeffs),
                                              ptr(colors), _lib.stream_of(coeffs)), "compute_sh_forward")
    return colors


def compute_sh_backward(num_points, degree, degrees_to_use, viewdirs, v_colors):
    _chk(("viewdirs", viewdirs), ("v_colors", v_colors))
    if viewdirs.ndim != 2 or viewdirs.shape[0] != num_points or viewdirs.shape[1] != 3:
        raise RuntimeError("viewdirs must have dimensions (N, 3)")
    if v_colors.ndim != 2 or v_colors.shape[0] != num_points or v_colors.shape[1] != 3:
        raise RuntimeError("v_colors must have dimensions (N, 3)")
    _f32("viewdirs", viewdirs)
    _f32("v_colors", v_colors)
    nb = num_sh_bases(degree)
    v_coeffs = torch.empty((num_points, nb, 3), dtype=torch.float32, device=v_colors.device)
    check(_lib.lib().gstex_compute_sh_backward(num_points, degree, degrees_to_use, ptr(viewdirs), ptr(v_colors),
                                               ptr(v_coeffs), _lib.stream_of(v_colors)), "compute_sh_backward")
    return v_coeffs


# ---------------------------------------------------------------------------
# projection (csrc/get_aabb_2d.cu:91-126) and tile counts
# ---------------------------------------------------------------------------
def get_aabb_2d(means, scales, glob_scale, quats, viewmat, fx, fy, cx, cy):
    _chk(("means", means), ("scales", scales), ("quats", quats), ("viewmat", viewmat))
    for n, t in (("means", means), ("scales", scales), ("quats", quats), ("viewmat", viewmat)):
        _f32(n, t)
    n = means.shape[0]
    centers = torch.empty((n, 2), dtype=torch.float32, device=means.device)
    extents = torch.empty((n, 2), dtype=torch.float32, device=means.device)
    check(_lib.lib().gstex_get_aabb_2d(n, ptr(means), ptr(scales), float(glob_scale), ptr(quats), ptr(viewmat),
                                       float(fx), float(fy), float(cx), float(cy), ptr(centers), ptr(extents),
                                       _lib.stream_of(means)), "get_aabb_2d")
    return centers, extents


def num_tiles_hit(centers, extents, img_height, img_width, block_width):
    _chk(("centers", centers), ("extents", extents))
    _f32("centers", centers)
    _f32("extents", extents)
    n = centers.shape[0]
    out = torch.empty(n, dtype=torch.int32, device=centers.device)
    check(_lib.lib().gstex_num_tiles_hit(n, ptr(centers), ptr(extents), int(img_height), int(img_width),
                                         int(block_width), ptr(out), _lib.stream_of(centers)), "num_tiles_hit")
    return out


def inclusive_scan(counts):
    """int32 inclusive prefix sum; returns (cum [n] int32, total [1] int64 on device)."""
    _chk(("counts", counts))
    _i32("counts", counts)
    n = counts.shape[0]
    L = _lib.lib()
    cum = torch.empty(n, dtype=torch.int32, device=counts.device)
    total = torch.empty(1, dtype=torch.int64, device=counts.device)
    wsb = L.gstex_scan_workspace_bytes(n)
    ws = torch.empty(wsb, dtype=torch.uint8, device=counts.device)
    check(L.gstex_inclusive_scan_i32(n, ptr(counts), ptr(cum), ptr(total), ptr(ws), wsb, _lib.stream_of(counts)),
          "inclusive_scan")
    return cum, total


# ---------------------------------------------------------------------------
# binning (csrc/bindings.cu:77-140)
# ---------------------------------------------------------------------------
def map_gaussian_to_intersects(num_points, num_intersects, centers, extents, depths, cum_tiles_hit, tile_bounds,
                               block_width, wrapped=False):
    _chk(("centers", centers), ("extents", extents), ("depths", depths), ("cum_tiles_hit", cum_tiles_hit))
    _i32("cum_tiles_hit", cum_tiles_hit)
    dev = centers.device
    isect_ids = torch.empty(num_intersects, dtype=torch.int64, device=dev)
    gaussian_ids = torch.empty(num_intersects, dtype=torch.int32, device=dev)
    check(_lib.lib().gstex_map_gaussian_to_intersects(
        int(num_points), int(num_intersects), ptr(centers), ptr(extents), ptr(depths), ptr(cum_tiles_hit),
        int(tile_bounds[0]), int(tile_bounds[1]), int(block_width), int(bool(wrapped)), ptr(isect_ids),
        ptr(gaussian_ids), _lib.stream_of(centers)), "map_gaussian_to_intersects")
    return isect_ids, gaussian_ids


def sort_end_bit(num_tiles: int) -> int:
    """Key bits that order (tile, non-negative depth) keys: 32 depth bits plus
    enough tile bits that 2**bits > num_tiles."""
    return 32 + max(1, int(num_tiles).bit_length())


def sort_pairs(keys, vals, end_bit=64):
    """Stable ascending sort of int64 keys (bits [0, end_bit)) with int32 values."""
    _chk(("keys", keys), ("vals", vals))
    n = keys.shape[0]
    L = _lib.lib()
    ko = torch.empty_like(keys)
    vo = torch.empty_like(vals)
    wsb = L.gstex_sort_workspace_bytes(n)
    ws = torch.empty(wsb, dtype=torch.uint8, device=keys.device)
    check(L.gstex_sort_pairs(n, int(end_bit), ptr(keys), ptr(vals), ptr(ko), ptr(vo), ptr(ws), wsb,
                             _lib.stream_of(keys)), "sort_pairs")
    return ko, vo


def get_tile_bin_edges(num_intersects, isect_ids_sorted, tile_bounds):
    _chk(("isect_ids_sorted", isect_ids_sorted))
    num_tiles = int(tile_bounds[0]) * int(tile_bounds[1])
    bins = torch.empty((num_tiles, 2), dtype=torch.int32, device=isect_ids_sorted.device)
    check(_lib.lib().gstex_get_tile_bin_edges(int(num_intersects), ptr(isect_ids_sorted), num_tiles, ptr(bins),
                                              _lib.stream_of(isect_ids_sorted)), "get_tile_bin_edges")
    return bins


# ---------------------------------------------------------------------------
# compositor (csrc/texture.cu:762-1053)
# ---------------------------------------------------------------------------
def _texture_mode(texture, channels):
    if texture.dtype == torch.float32:
        return TEXTURE_FP32
    if texture.dtype == torch.bfloat16:
        if channels != 3 or texture.ndim != 2 or texture.shape[1] != 4:
            raise _lib.GstexError("a bfloat16 texture must be [T, 4] (3 channels padded to 4)")
        return TEXTURE_BF16X4
    raise _lib.GstexError(f"texture must be float32 or bfloat16, got {texture.dtype}")


PIXELS_PER_THREAD = 1  # 1 or 2 (2 halves the threads per tile; even block widths only)
# Lanes that walk one list of staged splats in texture_backward: 32 (a
# warp's 8x4 pixel block), 16 (4x4), 8 (4x2) or 4 (2x2); below 32 only for
# block widths that are multiples of 8, one pixel per thread and 0 or 3
# channels (else 32).  8 measured fastest on the benchmark scenes.
BACKWARD_GROUP_LANES = 8
# texture_forward / texture_backward build one splat record per Gaussian of the
# view first (gstex_view_records) and the tiles copy them; False: every tile
# derives the records of its Gaussians itself.
PREBUILT_RECORDS = True


def _raster_inputs(img_w, img_h, bw, texture_info, texture_dims, gaussian_ids_sorted, tile_bins, colors, opacities,
                   means, scales, glob_scale, quats, uv0, umap, vmap, texture, viewmat, fx, fy, cx, cy, settings,
                   background):
    named = [("texture_dims", texture_dims), ("gaussian_ids_sorted", gaussian_ids_sorted),
             ("tile_bins", tile_bins), ("colors", colors), ("opacities", opacities), ("means", means),
             ("scales", scales), ("quats", quats), ("uv0", uv0), ("umap", umap), ("vmap", vmap),
             ("texture", texture), ("viewmat", viewmat), ("background", background)]
    _chk(*named)
    for n, t in named:
        if n in ("texture_dims", "gaussian_ids_sorted", "tile_bins"):
            _i32(n, t)
        elif n != "texture":
            _f32(n, t)
    if colors.ndim != 2 or colors.shape[1] != 3:
        raise _lib.GstexError("colors must be [N, 3]")
    C = int(texture_info[2])
    mode = _texture_mode(texture, C)
    ri = _lib.RasterInputs()
    ri.num_points = means.shape[0]
    ri.img_width, ri.img_height, ri.block_width = int(img_w), int(img_h), int(bw)
    ri.channels = C
    ri.num_texels = texture.shape[0]
    ri.texture_dtype = mode
    ri.texture_dims, ri.gaussian_ids_sorted, ri.tile_bins = ptr(texture_dims), ptr(gaussian_ids_sorted), ptr(tile_bins)
    ri.colors, ri.opacities, ri.means, ri.scales = ptr(colors), ptr(opacities), ptr(means), ptr(scales)
    ri.glob_scale = float(glob_scale)
    ri.quats, ri.uv0, ri.umap, ri.vmap = ptr(quats), ptr(uv0), ptr(umap), ptr(vmap)
    ri.texture, ri.viewmat = ptr(texture), ptr(viewmat)
    ri.fx, ri.fy, ri.cx, ri.cy = float(fx), float(fy), float(cx), float(cy)
    ri.settings = int(settings)
    ri.background = ptr(background)
    ri.pixels_per_thread = int(PIXELS_PER_THREAD)
    return ri, C


def _attach_records(ri, device):
    """Builds the view's splat records into a fresh buffer and points `ri` at
    it; returns the buffer (kept alive by the caller until the launch is
    queued)."""
    if not PREBUILT_RECORDS or ri.num_points == 0:
        return None
    L = _lib.lib()
    nb = L.gstex_view_records_bytes(ri.num_points)
    buf = torch.empty(nb, dtype=torch.uint8, device=device)
    check(L.gstex_view_records(ctypes.byref(ri), ptr(buf), nb, _lib.stream_of(buf)), "view_records")
    ri.records = ptr(buf)
    return buf


def texture_forward(tile_bounds, block, img_size, texture_info, texture_dims, gaussian_ids_sorted, tile_bins,
                    colors, opacities, means, scales, glob_scale, quats, uv0, umap, vmap, texture, viewmat, c2w, fx,
                    fy, cx, cy, settings, background):
    """Returns (out_img, out_depth, out_reg, out_texture, out_normal, final_Ts, final_idx, depth_idx, out_reg_s).

    c2w is accepted for interface compatibility; rays are built from viewmat
    (the two must be inverses of each other, as in the reference)."""
    W, H = int(img_size[0]), int(img_size[1])
    bw = int(block[0])
    ri, C = _raster_inputs(W, H, bw, texture_info, texture_dims, gaussian_ids_sorted, tile_bins, colors, opacities,
                           means, scales, glob_scale, quats, uv0, umap, vmap, texture, viewmat, fx, fy, cx, cy,
                           settings, background)
    dev = means.device
    f32 = dict(dtype=torch.float32, device=dev)
    out_img = torch.empty((H, W, 3), **f32)
    out_depth = torch.empty((H, W), **f32)
    out_reg = torch.empty((H, W), **f32)
    out_tex = torch.empty((H, W, C), **f32)
    out_normal = torch.empty((H, W, 3), **f32)
    final_T = torch.empty((H, W), **f32)
    final_idx = torch.empty((H, W), dtype=torch.int32, device=dev)
    depth_idx = torch.empty((H, W), dtype=torch.int32, device=dev)
    reg_s = torch.empty((H, W, 3), **f32)
    fo = _lib.ForwardOutputs(ptr(out_img), ptr(out_depth), ptr(out_reg), ptr(out_tex), ptr(out_normal), ptr(final_T),
                             ptr(final_idx), ptr(depth_idx), ptr(reg_s))
    recs = _attach_records(ri, dev)  # noqa: F841 (alive until the launch is queued)
    check(_lib.lib().gstex_texture_forward(ctypes.byref(ri), ctypes.byref(fo), _lib.stream_of(means)),
          "texture_forward")
    return out_img, out_depth, out_reg, out_tex, out_normal, final_T, final_idx, depth_idx, reg_s


def texture_backward(img_height, img_width, block_width, texture_info, texture_dims, gaussian_ids_sorted, tile_bins,
                     colors, opacities, means, scales, glob_scale, quats, uv0, umap, vmap, texture, viewmat, c2w, fx,
                     fy, cx, cy, settings, background, final_Ts, final_idx, depth_idx, final_s, v_output,
                     v_output_depth, v_output_reg, v_output_alpha, v_output_texture, v_output_normal):
    """Returns (v_colors, v_opacity, v_means, v_scales, v_quats, v_uv0, v_umap, v_vmap, v_texture)."""
    ri, C = _raster_inputs(img_width, img_height, block_width, texture_info, texture_dims, gaussian_ids_sorted,
                           tile_bins, colors, opacities, means, scales, glob_scale, quats, uv0, umap, vmap, texture,
                           viewmat, fx, fy, cx, cy, settings, background)
    ri.group_lanes = int(BACKWARD_GROUP_LANES)
    ups = [("final_Ts", final_Ts), ("final_idx", final_idx), ("depth_idx", depth_idx), ("final_s", final_s),
           ("v_output", v_output), ("v_output_depth", v_output_depth), ("v_output_reg", v_output_reg),
           ("v_output_alpha", v_output_alpha), ("v_output_texture", v_output_texture),
           ("v_output_normal", v_output_normal)]
    _chk(*ups)
    dev = means.device
    N = means.shape[0]
    L = _lib.lib()
    v_colors = torch.empty((N, 3), dtype=torch.float32, device=dev)
    v_opacity = torch.empty(opacities.shape, dtype=torch.float32, device=dev)
    v_means = torch.empty((N, 3), dtype=torch.float32, device=dev)
    v_scales = torch.empty((N, 3), dtype=torch.float32, device=dev)
    v_quats = torch.empty((N, 4), dtype=torch.float32, device=dev)
    v_uv0 = torch.empty(uv0.shape, dtype=torch.float32, device=dev)
    v_umap = torch.empty(umap.shape, dtype=torch.float32, device=dev)
    v_vmap = torch.empty(vmap.shape, dtype=torch.float32, device=dev)
    tex_cols = 4 if ri.texture_dtype == TEXTURE_BF16X4 else C
    v_texture = torch.zeros((texture.shape[0], tex_cols), dtype=torch.float32, device=dev)
    wsb = L.gstex_backward_workspace_bytes(N)
    ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
    bio = _lib.BackwardIO(ptr(final_Ts), ptr(final_idx), ptr(depth_idx), ptr(final_s), ptr(v_output),
                          ptr(v_output_depth), ptr(v_output_reg), ptr(v_output_alpha), ptr(v_output_texture),
                          ptr(v_output_normal), ptr(v_colors), ptr(v_opacity), ptr(v_means), ptr(v_scales),
                          ptr(v_quats), ptr(v_uv0), ptr(v_umap), ptr(v_vmap), ptr(v_texture), ptr(ws), wsb)
    recs = _attach_records(ri, dev)  # noqa: F841 (alive until the launch is queued)
    check(L.gstex_texture_backward(ctypes.byref(ri), ctypes.byref(bio), _lib.stream_of(means)), "texture_backward")
    return v_colors, v_opacity, v_means, v_scales, v_quats, v_uv0, v_umap, v_vmap, v_texture


# ---------------------------------------------------------------------------
# texture_sample (csrc/texture_sample.cu:72-141)
# ---------------------------------------------------------------------------
def texture_sample_forward(texture_info, texture_dims, uvs, texture):
    _chk(("texture_dims", texture_dims), ("uvs", uvs), ("texture", texture))
    _i32("texture_dims", texture_dims)
    _f32("uvs", uvs)
    _f32("texture", texture)
    C = int(texture_info[2])
    nq = uvs.shape[0]
    out = torch.empty((nq, C), dtype=torch.float32, device=uvs.device)
    check(_lib.lib().gstex_texture_sample_forward(nq, C, ptr(texture_dims), ptr(uvs), ptr(texture), ptr(out),
                                                  _lib.stream_of(uvs)), "texture_sample_forward")
    return out


def texture_sample_backward(texture_info, texture_dims, uvs, texture, v_output, need_uv_grad=False):
    _chk(("texture_dims", texture_dims), ("uvs", uvs), ("texture", texture), ("v_output", v_output))
    C = int(texture_info[2])
    nq = uvs.shape[0]
    v_texture = torch.zeros((texture.shape[0], C), dtype=torch.float32, device=uvs.device)
    v_uvs = torch.empty((nq, 2), dtype=torch.float32, device=uvs.device) if need_uv_grad else None
    check(_lib.lib().gstex_texture_sample_backward(nq, C, ptr(texture_dims), ptr(uvs), ptr(texture), ptr(v_output),
                                                   ptr(v_texture), ptr(v_uvs), _lib.stream_of(uvs)),
          "texture_sample_backward")
    if need_uv_grad:
        return v_texture, v_uvs
    return v_texture


def texture_edit(tile_bounds, block, img_size, texture_info, texture_total_size, texture_dims, updated_img,
                 updated_alpha, depth_lower, depth_upper, gaussian_ids_sorted, tile_bins, opacities, means, scales,
                 glob_scale, quats, uv0, umap, vmap, viewmat, c2w, fx, fy, cx, cy, settings, background):
    """Returns updated_texture [texture_total_size, 5]: per texel the bilinear
    splat of (r*a, g*a, b*a, a) of the edited image and the total weight
    (csrc/texture_edit.cu).  texture_info[2] must be 5 (the reference writes
    five channels at a stride of texture_info[2]); blur is settings bit 0;
    c2w and background are accepted for interface compatibility."""
    named = [("texture_dims", texture_dims), ("updated_img", updated_img), ("updated_alpha", updated_alpha),
             ("depth_lower", depth_lower), ("depth_upper", depth_upper),
             ("gaussian_ids_sorted", gaussian_ids_sorted), ("tile_bins", tile_bins), ("opacities", opacities),
             ("means", means), ("scales", scales), ("quats", quats), ("uv0", uv0), ("umap", umap), ("vmap", vmap),
             ("viewmat", viewmat)]
    _chk(*named)
    for n, t in named:
        if n in ("texture_dims", "gaussian_ids_sorted", "tile_bins"):
            _i32(n, t)
        else:
            _f32(n, t)
    if int(texture_info[2]) != 5:
        raise _lib.GstexError("texture_edit: texture_info[2] must be 5 (r*a, g*a, b*a, a, weight)")
    W, H = int(img_size[0]), int(img_size[1])
    if updated_img.numel() != H * W * 3 or updated_alpha.numel() != H * W or depth_lower.numel() != H * W \
            or depth_upper.numel() != H * W:
        raise _lib.GstexError("texture_edit: per-pixel inputs must have H*W entries")
    T = int(texture_total_size)
    ri = _lib.RasterInputs()
    ri.num_points = means.shape[0]
    ri.img_width, ri.img_height, ri.block_width = W, H, int(block[0])
    ri.channels = 5
    ri.num_texels = T
    ri.texture_dims, ri.gaussian_ids_sorted, ri.tile_bins = ptr(texture_dims), ptr(gaussian_ids_sorted), ptr(tile_bins)
    ri.opacities, ri.means, ri.scales = ptr(opacities), ptr(means), ptr(scales)
    ri.glob_scale = float(glob_scale)
    ri.quats, ri.uv0, ri.umap, ri.vmap = ptr(quats), ptr(uv0), ptr(umap), ptr(vmap)
    ri.viewmat = ptr(viewmat)
    ri.fx, ri.fy, ri.cx, ri.cy = float(fx), float(fy), float(cx), float(cy)
    ri.settings = int(settings)
    out = torch.empty((T, 5), dtype=torch.float32, device=means.device)
    io = _lib.EditIO(ptr(updated_img), ptr(updated_alpha), ptr(depth_lower), ptr(depth_upper), T, ptr(out))
    check(_lib.lib().gstex_texture_edit(ctypes.byref(ri), ctypes.byref(io), _lib.stream_of(means)), "texture_edit")
    return out
