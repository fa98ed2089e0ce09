"""CPU oracle for the textured 2D-Gaussian rasteriser hot path.

TEST INFRASTRUCTURE ONLY.  The functions here call ``gstex_oracle.c`` (a
plain-C restatement of the reference kernels, built into ``oracle/_build``)
through ctypes.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` use this module,
and only as the checker or the timed CPU baseline.  The product package never
imports it.

Every function takes and returns numpy arrays.  ``prec`` selects the fp32
build (same operation order as the reference kernels, IEEE arithmetic) or the
fp64 build.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIBS: dict = {}

_P = ctypes.c_void_p
_I = ctypes.c_int
_L = ctypes.c_long


def build(force: bool = False) -> None:
    """Compile the oracle with the committed Makefile (gcc, OpenMP)."""
    if force or not all(os.path.exists(os.path.join(_BUILD, f)) for f in ("liboracle32.so", "liboracle64.so")):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)


def _lib(prec: str):
    if prec not in _LIBS:
        build()
        name = {"f32": "liboracle32.so", "f64": "liboracle64.so"}[prec]
        _LIBS[prec] = ctypes.CDLL(os.path.join(_BUILD, name))
    return _LIBS[prec]


def _dt(prec):
    return np.float32 if prec == "f32" else np.float64


def _r(prec):
    return ctypes.c_float if prec == "f32" else ctypes.c_double


def _a(x, dtype):
    return np.ascontiguousarray(x, dtype=dtype)


def _p(x):
    return x.ctypes.data_as(_P)


def _fn(prec, name):
    pre = "or32_" if prec == "f32" else "or64_"
    return getattr(_lib(prec), pre + name)


# --------------------------------------------------------------------------
# projection / SH / texture_sample
# --------------------------------------------------------------------------
def get_aabb_2d(means, scales, glob_scale, quats, viewmat, fx, fy, cx, cy, prec="f32"):
    dt = _dt(prec)
    R = _r(prec)
    means, scales, quats, viewmat = (_a(x, dt) for x in (means, scales, quats, viewmat))
    n = means.shape[0]
    centers = np.zeros((n, 2), dt)
    extents = np.zeros((n, 2), dt)
    f = _fn(prec, "get_aabb_2d")
    f(_I(n), _p(means), _p(scales), R(glob_scale), _p(quats), _p(viewmat), R(fx), R(fy), R(cx), R(cy),
      _p(centers), _p(extents))
    return centers, extents


def num_sh_bases(degree):
    return {0: 1, 1: 4, 2: 9, 3: 16}.get(degree, 25)


def sh_forward(degree, degrees_to_use, viewdirs, coeffs, prec="f32"):
    dt = _dt(prec)
    viewdirs, coeffs = _a(viewdirs, dt), _a(coeffs, dt)
    n = viewdirs.shape[0]
    out = np.zeros((n, 3), dt)
    _fn(prec, "sh_forward")(_I(n), _I(degree), _I(degrees_to_use), _p(viewdirs), _p(coeffs), _p(out))
    return out


def sh_backward(degree, degrees_to_use, viewdirs, v_colors, prec="f32"):
    dt = _dt(prec)
    viewdirs, v_colors = _a(viewdirs, dt), _a(v_colors, dt)
    n = viewdirs.shape[0]
    out = np.zeros((n, num_sh_bases(degree), 3), dt)
    _fn(prec, "sh_backward")(_I(n), _I(degree), _I(degrees_to_use), _p(viewdirs), _p(v_colors), _p(out))
    return out


def texture_sample_forward(texture_dims, uvs, texture, prec="f32"):
    dt = _dt(prec)
    dims = _a(texture_dims, np.int32)
    uvs, texture = _a(uvs, dt), _a(texture, dt)
    nq, C = uvs.shape[0], texture.shape[1]
    out = np.zeros((nq, C), dt)
    _fn(prec, "texture_sample_forward")(_I(nq), _I(C), _p(dims), _p(uvs), _p(texture), _p(out))
    return out


def texture_sample_backward(texture_dims, uvs, texture, v_out, prec="f32"):
    dt = _dt(prec)
    dims = _a(texture_dims, np.int32)
    uvs, texture, v_out = _a(uvs, dt), _a(texture, dt), _a(v_out, dt)
    nq, C = uvs.shape[0], texture.shape[1]
    v_tex = np.zeros_like(texture)
    v_uvs = np.zeros_like(uvs)
    _fn(prec, "texture_sample_backward")(_I(nq), _I(C), _p(dims), _p(uvs), _p(texture), _p(v_out),
                                         _p(v_tex), _p(v_uvs))
    return v_tex, v_uvs


# --------------------------------------------------------------------------
# binning (float32 inputs, integer outputs; bit-exact targets)
# --------------------------------------------------------------------------
def num_tiles_hit(centers, extents, img_height, img_width, block_width):
    centers, extents = _a(centers, np.float32), _a(extents, np.float32)
    n = centers.shape[0]
    out = np.zeros(n, np.int32)
    _lib("f32").or_num_tiles_hit(_I(n), _p(centers), _p(extents), _I(img_height), _I(img_width),
                                 _I(block_width), _p(out))
    return out


def tile_bounds(img_height, img_width, block_width):
    return ((img_width + block_width - 1) // block_width, (img_height + block_width - 1) // block_width, 1)


def map_gaussian_to_intersects(centers, extents, depths, cum_tiles_hit, tile_bnds, block_width,
                               num_intersects, wrapped=False):
    centers, extents = _a(centers, np.float32), _a(extents, np.float32)
    depths, cum = _a(depths, np.float32), _a(cum_tiles_hit, np.int32)
    n = centers.shape[0]
    keys = np.zeros(num_intersects, np.int64)
    gids = np.zeros(num_intersects, np.int32)
    _lib("f32").or_map_gaussian_to_intersects(
        _I(n), _p(centers), _p(extents), _p(depths), _p(cum), _I(tile_bnds[0]), _I(tile_bnds[1]),
        _I(block_width), _I(int(wrapped)), _L(num_intersects), _p(keys), _p(gids))
    return keys, gids


def sort_pairs(keys, vals):
    keys, vals = _a(keys, np.int64), _a(vals, np.int32)
    n = keys.shape[0]
    ko = np.zeros_like(keys)
    vo = np.zeros_like(vals)
    _lib("f32").or_sort_pairs(_L(n), _p(keys), _p(vals), _p(ko), _p(vo))
    return ko, vo


def get_tile_bin_edges(isect_ids_sorted, tile_bnds):
    s = _a(isect_ids_sorted, np.int64)
    nt = tile_bnds[0] * tile_bnds[1]
    bins = np.zeros((nt, 2), np.int32)
    _lib("f32").or_get_tile_bin_edges(_L(s.shape[0]), _p(s), _I(nt), _p(bins))
    return bins


def bin_and_sort(centers, extents, depths, num_tiles, img_height, img_width, block_width):
    """Whole binning stage: cumsum, emission, stable sort, tile ranges."""
    tb = tile_bounds(img_height, img_width, block_width)
    cum = np.cumsum(np.asarray(num_tiles, np.int64)).astype(np.int32)
    n_isect = int(cum[-1]) if cum.size else 0
    keys, gids = map_gaussian_to_intersects(centers, extents, depths, cum, tb, block_width, n_isect)
    ks, gs = sort_pairs(keys, gids)
    bins = get_tile_bin_edges(ks, tb)
    return dict(cum=cum, n_isect=n_isect, isect_ids=keys, gaussian_ids=gids, isect_ids_sorted=ks,
                gaussian_ids_sorted=gs, tile_bins=bins, tile_bounds=tb)


# --------------------------------------------------------------------------
# compositor
# --------------------------------------------------------------------------
@dataclass
class Scene:
    """Per-Gaussian inputs of texture_gaussians (numpy, any float dtype)."""
    means: np.ndarray        # [N,3]
    scales: np.ndarray       # [N,3]
    quats: np.ndarray        # [N,4] wxyz, normalised
    opacity: np.ndarray      # [N,1]
    colors: np.ndarray       # [N,3]
    uv0: np.ndarray          # [N,1,2]
    umap: np.ndarray         # [N,1,3]
    vmap: np.ndarray         # [N,1,3]
    texture_dims: np.ndarray  # [N,3] int32 (h, w, start)
    texture: np.ndarray      # [T,C]
    glob_scale: float = 1.0


@dataclass
class Camera:
    viewmat: np.ndarray  # [4,4] world->camera, row-major
    c2w: np.ndarray      # [4,4]
    fx: float
    fy: float
    cx: float
    cy: float
    height: int
    width: int


def texture_forward(scene: Scene, cam: Camera, gids_sorted, tile_bins, block_width, settings, background,
                    prec="f32", nthreads=0):
    dt = _dt(prec)
    R = _r(prec)
    C = scene.texture.shape[1]
    H, W = cam.height, cam.width
    tb = tile_bounds(H, W, block_width)
    a = [_a(x, dt) for x in (scene.colors, scene.opacity, scene.means, scene.scales)]
    b = [_a(x, dt) for x in (scene.quats, scene.uv0, scene.umap, scene.vmap, scene.texture,
                             cam.viewmat, cam.c2w)]
    dims = _a(scene.texture_dims, np.int32)
    gs = _a(gids_sorted, np.int32)
    bins = _a(tile_bins, np.int32)
    bg = _a(background, dt)
    out = dict(
        final_T=np.zeros((H, W), dt), final_idx=np.zeros((H, W), np.int32), depth_idx=np.zeros((H, W), np.int32),
        reg_s=np.zeros((H, W, 3), dt), img=np.zeros((H, W, 3), dt), depth=np.zeros((H, W), dt),
        reg=np.zeros((H, W), dt), texture=np.zeros((H, W, C), dt), normal=np.zeros((H, W, 3), dt))
    rc = _fn(prec, "texture_forward")(
        _I(tb[0]), _I(tb[1]), _I(block_width), _I(W), _I(H), _I(C), _p(dims), _p(gs), _p(bins),
        _p(a[0]), _p(a[1]), _p(a[2]), _p(a[3]), R(scene.glob_scale), _p(b[0]), _p(b[1]), _p(b[2]), _p(b[3]),
        _p(b[4]), _p(b[5]), _p(b[6]), R(cam.fx), R(cam.fy), R(cam.cx), R(cam.cy), _I(settings), _p(bg),
        _p(out["final_T"]), _p(out["final_idx"]), _p(out["depth_idx"]), _p(out["reg_s"]), _p(out["img"]),
        _p(out["depth"]), _p(out["reg"]), _p(out["texture"]), _p(out["normal"]), _I(nthreads))
    if rc != 0:
        raise ValueError("oracle texture_forward: unsupported channel count")
    out["alpha"] = 1 - out["final_T"]
    return out


def texture_backward(scene: Scene, cam: Camera, gids_sorted, tile_bins, block_width, settings, background,
                     fwd: dict, v_img, v_depth, v_reg, v_alpha, v_texture, v_normal, prec="f32", nthreads=0):
    dt = _dt(prec)
    R = _r(prec)
    C = scene.texture.shape[1]
    H, W = cam.height, cam.width
    tb = tile_bounds(H, W, block_width)
    N = scene.means.shape[0]
    a = [_a(x, dt) for x in (scene.colors, scene.opacity, scene.means, scene.scales)]
    b = [_a(x, dt) for x in (scene.quats, scene.uv0, scene.umap, scene.vmap, scene.texture,
                             cam.viewmat, cam.c2w)]
    dims = _a(scene.texture_dims, np.int32)
    gs = _a(gids_sorted, np.int32)
    bins = _a(tile_bins, np.int32)
    bg = _a(background, dt)
    f = [_a(fwd["final_T"], dt), _a(fwd["final_idx"], np.int32), _a(fwd["depth_idx"], np.int32),
         _a(fwd["reg_s"], dt)]
    g = [_a(x, dt) for x in (v_img, v_depth, v_reg, v_alpha, v_texture, v_normal)]
    out = dict(colors=np.zeros((N, 3), dt), opacity=np.zeros((N, 1), dt), means=np.zeros((N, 3), dt),
               scales=np.zeros((N, 3), dt), quats=np.zeros((N, 4), dt), uv0=np.zeros((N, 1, 2), dt),
               umap=np.zeros((N, 1, 3), dt), vmap=np.zeros((N, 1, 3), dt),
               texture=np.zeros(scene.texture.shape, dt))
    rc = _fn(prec, "texture_backward")(
        _I(tb[0]), _I(tb[1]), _I(block_width), _I(W), _I(H), _I(C), _p(dims), _p(gs), _p(bins),
        _p(a[0]), _p(a[1]), _p(a[2]), _p(a[3]), R(scene.glob_scale), _p(b[0]), _p(b[1]), _p(b[2]), _p(b[3]),
        _p(b[4]), _p(b[5]), _p(b[6]), R(cam.fx), R(cam.fy), R(cam.cx), R(cam.cy), _I(settings), _p(bg),
        _p(f[0]), _p(f[1]), _p(f[2]), _p(f[3]), _p(g[0]), _p(g[1]), _p(g[2]), _p(g[3]), _p(g[4]), _p(g[5]),
        _p(out["colors"]), _p(out["opacity"]), _p(out["means"]), _p(out["scales"]), _p(out["quats"]),
        _p(out["uv0"]), _p(out["umap"]), _p(out["vmap"]), _p(out["texture"]), _I(nthreads))
    if rc != 0:
        raise ValueError("oracle texture_backward: unsupported channel count")
    return out


def texture_edit(scene: Scene, cam: Camera, gids_sorted, tile_bins, block_width, settings, updated_img,
                 updated_alpha, depth_lower, depth_upper, num_texels, prec="f32", nthreads=0):
    """csrc/texture_edit.cu:11-236: the five-channel splat of an edited image
    into the texels ([num_texels, 5]: r*a, g*a, b*a, a, total weight)."""
    dt = _dt(prec)
    R = _r(prec)
    H, W = cam.height, cam.width
    tb = tile_bounds(H, W, block_width)
    a = [_a(x, dt) for x in (updated_img, updated_alpha, depth_lower, depth_upper, scene.opacity, scene.means,
                             scene.scales, scene.quats, scene.uv0, scene.umap, scene.vmap, cam.viewmat, cam.c2w)]
    dims = _a(scene.texture_dims, np.int32)
    gs = _a(gids_sorted, np.int32)
    bins = _a(tile_bins, np.int32)
    out = np.zeros((int(num_texels), 5), dt)
    _fn(prec, "texture_edit")(
        _I(tb[0]), _I(tb[1]), _I(block_width), _I(W), _I(H), _p(dims), _p(a[0]), _p(a[1]), _p(a[2]), _p(a[3]),
        _p(gs), _p(bins), _p(a[4]), _p(a[5]), _p(a[6]), R(scene.glob_scale), _p(a[7]), _p(a[8]), _p(a[9]),
        _p(a[10]), _p(a[11]), _p(a[12]), R(cam.fx), R(cam.fy), R(cam.cx), R(cam.cy), _I(settings), _p(out),
        _I(nthreads))
    return out


def render(scene: Scene, cam: Camera, depths=None, block_width=16, settings=1 << 8, background=None,
           prec="f32", nthreads=0, binning=None):
    """Projection + binning (float32, like the reference) + forward."""
    if background is None:
        background = np.ones(3)
    if binning is None:
        c, e = get_aabb_2d(scene.means, scene.scales, scene.glob_scale, scene.quats, cam.viewmat,
                           cam.fx, cam.fy, cam.cx, cam.cy, prec="f32")
        if depths is None:
            depths = project_depths(scene.means, cam.viewmat)
        nt = num_tiles_hit(c, e, cam.height, cam.width, block_width)
        binning = bin_and_sort(c, e, depths, nt, cam.height, cam.width, block_width)
    fwd = texture_forward(scene, cam, binning["gaussian_ids_sorted"], binning["tile_bins"], block_width,
                          settings, background, prec=prec, nthreads=nthreads)
    return binning, fwd


def project_depths(means, viewmat):
    """Camera-space z of each mean in float32 (gstex_cuda/get_aabb_2d.py:22-32)."""
    m = np.asarray(means, np.float32)
    v = np.asarray(viewmat, np.float32)
    return (m @ v[:3, :3].T + v[:3, 3])[:, 2].astype(np.float32)


def project_points(means, viewmat, fx, fy, cx, cy):
    """Pixel means and depths (gstex_cuda/get_aabb_2d.py:22-32, 140-147)."""
    m = np.asarray(means, np.float32)
    v = np.asarray(viewmat, np.float32)
    p = (m @ v[:3, :3].T + v[:3, 3]).astype(np.float32)
    rw = np.float32(1) / (p[:, 2] + np.float32(1e-6))
    pix = np.stack([p[:, 0] * rw * np.float32(fx) + np.float32(cx),
                    p[:, 1] * rw * np.float32(fy) + np.float32(cy)], -1)
    return pix, p[:, 2].copy()


def camera_depths(means, viewmat):
    """Camera-space z of each mean with the float32 operation order of the
    kernels' transform (m8*x + m9*y + m10*z + m11, no fused multiply-add)."""
    m = np.asarray(means, np.float32)
    v = np.asarray(viewmat, np.float32).reshape(-1)
    return (((v[8] * m[:, 0] + v[9] * m[:, 1]) + v[10] * m[:, 2]) + v[11]).astype(np.float32)
