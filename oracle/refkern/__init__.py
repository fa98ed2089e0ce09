"""The reference's own CUDA kernels, run on the GPU from cubins.

TEST INFRASTRUCTURE ONLY.  ``build_ref.py`` compiles the reference's kernel
sources (gstex_cuda/cuda/csrc/*.cu, device code only) into ``oracle/_ref/*.cubin``;
this module loads those cubins through the CUDA driver API (ctypes on
libcuda) into the context that torch uses, and launches the kernels with the
grid, block and argument lists of the reference's host wrappers.  The tests
use it to check the product kernels against the reference kernels on the same
inputs.  The product package never imports it.

Each wrapper restates one host function of the reference (file:line given);
outputs are zero-filled like the reference's ``torch::zeros`` outputs.  All
tensors are float32 / int32 / int64 CUDA tensors, contiguous.
"""
from __future__ import annotations

import ctypes
import os
from typing import Dict, Tuple

import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(os.path.dirname(_HERE), "_ref")
UNITS = ("forward", "get_aabb_2d", "texture", "texture_sample", "texture_edit", "sh")
N_THREADS = 256  # config.h:2

_cu = None
_mods: Dict[str, Dict[str, int]] = {}


class RefUnavailable(RuntimeError):
    pass


class Dim3(ctypes.Structure):
    _fields_ = [("x", ctypes.c_uint), ("y", ctypes.c_uint), ("z", ctypes.c_uint)]


class Int3(ctypes.Structure):
    _fields_ = [("x", ctypes.c_int), ("y", ctypes.c_int), ("z", ctypes.c_int)]


class Float4(ctypes.Structure):
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float), ("z", ctypes.c_float), ("w", ctypes.c_float)]


def cubin(unit: str) -> str:
    return os.path.join(REF_DIR, unit + ".cubin")


def available() -> bool:
    """True when every cubin exists and a CUDA device is present."""
    return torch.cuda.is_available() and all(os.path.exists(cubin(u)) for u in UNITS)


def _driver():
    global _cu
    if _cu is None:
        cu = ctypes.CDLL("libcuda.so.1")
        cu.cuGetErrorString.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]
        cu.cuCtxGetCurrent.argtypes = [ctypes.POINTER(ctypes.c_void_p)]
        cu.cuModuleLoad.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p]
        cu.cuModuleGetFunctionCount.argtypes = [ctypes.POINTER(ctypes.c_uint), ctypes.c_void_p]
        cu.cuModuleEnumerateFunctions.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_uint, ctypes.c_void_p]
        cu.cuFuncGetName.argtypes = [ctypes.POINTER(ctypes.c_char_p), ctypes.c_void_p]
        cu.cuFuncGetParamInfo.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t),
                                          ctypes.POINTER(ctypes.c_size_t)]
        cu.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 7 + [ctypes.c_void_p,
                                                                              ctypes.POINTER(ctypes.c_void_p),
                                                                              ctypes.c_void_p]
        _cu = cu
    return _cu


def _check(rc: int, what: str) -> None:
    if rc != 0:
        s = ctypes.c_char_p()
        _driver().cuGetErrorString(rc, ctypes.byref(s))
        raise RuntimeError(f"{what}: CUDA driver error {rc} ({(s.value or b'?').decode()})")


def _module(unit: str) -> Dict[str, int]:
    """Load a cubin into torch's current context; map kernel name -> CUfunction."""
    if unit in _mods:
        return _mods[unit]
    if not os.path.exists(cubin(unit)):
        raise RefUnavailable(f"reference cubin {cubin(unit)} is missing (built by oracle/refkern/build_ref.py)")
    torch.zeros(1, device="cuda")  # makes torch's primary context current on this thread
    cu = _driver()
    ctx = ctypes.c_void_p()
    _check(cu.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
    if not ctx.value:
        raise RefUnavailable("no current CUDA context")
    mod = ctypes.c_void_p()
    _check(cu.cuModuleLoad(ctypes.byref(mod), cubin(unit).encode()), f"cuModuleLoad({unit})")
    n = ctypes.c_uint()
    _check(cu.cuModuleGetFunctionCount(ctypes.byref(n), mod), "cuModuleGetFunctionCount")
    fns = (ctypes.c_void_p * n.value)()
    _check(cu.cuModuleEnumerateFunctions(fns, n.value, mod), "cuModuleEnumerateFunctions")
    table = {}
    for f in fns:
        name = ctypes.c_char_p()
        _check(cu.cuFuncGetName(ctypes.byref(name), f), "cuFuncGetName")
        table[name.value.decode()] = f
    _mods[unit] = table
    return table


def kernel_names(unit: str):
    return sorted(_module(unit))


def _fn(unit: str, kernel: str) -> int:
    """The (unique, non-overloaded) kernel whose mangled name starts _Z<len><name>."""
    prefix = f"_Z{len(kernel)}{kernel}"
    hits = [f for n, f in _module(unit).items() if n.startswith(prefix)]
    if len(hits) != 1:
        raise RefUnavailable(f"kernel {kernel} not found once in {unit}.cubin")
    return hits[0]


def _ptr(t: torch.Tensor):
    assert t.is_cuda and t.is_contiguous(), "reference kernels take contiguous CUDA tensors"
    return ctypes.c_void_p(t.data_ptr())


def _check_params(fn, kernel: str, args) -> None:
    """Refuse a launch whose argument list does not match the kernel's
    parameter list (count and byte size of every parameter)."""
    cu = _driver()
    off, size = ctypes.c_size_t(), ctypes.c_size_t()
    for i, a in enumerate(args):
        _check(cu.cuFuncGetParamInfo(fn, i, ctypes.byref(off), ctypes.byref(size)), f"{kernel} parameter {i}")
        if size.value != ctypes.sizeof(a):
            raise RuntimeError(f"{kernel}: parameter {i} is {size.value} bytes, given {ctypes.sizeof(a)}")
    if cu.cuFuncGetParamInfo(fn, len(args), ctypes.byref(off), ctypes.byref(size)) == 0:
        raise RuntimeError(f"{kernel}: more than {len(args)} parameters")


def _launch(unit: str, kernel: str, grid, block, args) -> None:
    fn = _fn(unit, kernel)
    _check_params(fn, kernel, args)
    params = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p) for a in args])
    stream = torch.cuda.current_stream().cuda_stream
    _check(_driver().cuLaunchKernel(fn, grid[0], grid[1], grid[2], block[0], block[1], block[2], 0,
                                    ctypes.c_void_p(stream), params, None), f"launch {kernel}")


def _blocks(n: int) -> Tuple[int, int, int]:
    return (max(1, (n + N_THREADS - 1) // N_THREADS), 1, 1)


_f = ctypes.c_float
_i = ctypes.c_int
_u = ctypes.c_uint


# ---------------------------------------------------------------------------
# Native ops (the reference's gstex_cuda.cuda._C surface)
# ---------------------------------------------------------------------------
def compute_sh_forward(num_points, degree, degrees_to_use, viewdirs, coeffs):
    """bindings.cu:18-43."""
    nb = (degree + 1) ** 2
    assert coeffs.shape == (num_points, nb, 3)
    colors = torch.zeros((num_points, 3), device=coeffs.device)
    if num_points:
        _launch("sh", "compute_sh_forward_kernel", _blocks(num_points), (N_THREADS, 1, 1),
                [_u(num_points), _u(degree), _u(degrees_to_use), _ptr(viewdirs), _ptr(coeffs), _ptr(colors)])
    return colors


def compute_sh_backward(num_points, degree, degrees_to_use, viewdirs, v_colors):
    """bindings.cu:45-75."""
    nb = (degree + 1) ** 2
    assert viewdirs.shape == (num_points, 3) and v_colors.shape == (num_points, 3)
    v_coeffs = torch.zeros((num_points, nb, 3), device=v_colors.device)
    if num_points:
        _launch("sh", "compute_sh_backward_kernel", _blocks(num_points), (N_THREADS, 1, 1),
                [_u(num_points), _u(degree), _u(degrees_to_use), _ptr(viewdirs), _ptr(v_colors), _ptr(v_coeffs)])
    return v_coeffs


def get_aabb_2d(means, scales, glob_scale, quats, viewmat, fx, fy, cx, cy):
    """get_aabb_2d.cu:91-126."""
    n = means.shape[0]
    assert viewmat.numel() == 16
    centers = torch.zeros((n, 2), device=means.device)
    extents = torch.zeros((n, 2), device=means.device)
    if n:
        _launch("get_aabb_2d", "get_aabb_2d_kernel", _blocks(n), (N_THREADS, 1, 1),
                [_i(n), _ptr(means), _ptr(scales), _f(glob_scale), _ptr(quats), _ptr(viewmat), Float4(fx, fy, cx, cy),
                 _ptr(centers), _ptr(extents)])
    return centers, extents


def map_gaussian_to_intersects(num_points, num_intersects, centers, extents, depths, cum_tiles_hit, tile_bounds,
                               block_width, wrapped=False):
    """bindings.cu:77-121.  cum_tiles_hit is the int32 inclusive sum of the
    per-Gaussian tile counts.  The kernel derives its tile rectangle from
    c/bw - e/bw (helpers.cuh:85-91) while the counts come from (c - e)/bw
    (get_aabb_2d.py:70-91); where the two round apart a Gaussian writes past
    its own slots, so the outputs here carry one tile grid of slack after
    the last slot and are returned trimmed to num_intersects."""
    assert cum_tiles_hit.dtype == torch.int32 and cum_tiles_hit.numel() == num_points
    dev = centers.device
    slack = int(tile_bounds[0]) * int(tile_bounds[1])
    gids = torch.zeros(num_intersects + slack, dtype=torch.int32, device=dev)
    isect = torch.zeros(num_intersects + slack, dtype=torch.int64, device=dev)
    if num_points and num_intersects:
        _launch("forward", "map_gaussian_to_intersects", _blocks(num_points), (N_THREADS, 1, 1),
                [_i(num_points), _ptr(centers), _ptr(extents), _ptr(depths), _ptr(cum_tiles_hit), Dim3(*tile_bounds),
                 _u(block_width), ctypes.c_bool(wrapped), _ptr(isect), _ptr(gids)])
    return isect[:num_intersects], gids[:num_intersects]


def get_tile_bin_edges(num_intersects, isect_ids_sorted, tile_bounds):
    """bindings.cu:123-140."""
    num_tiles = tile_bounds[0] * tile_bounds[1]
    bins = torch.zeros((num_tiles, 2), dtype=torch.int32, device=isect_ids_sorted.device)
    if num_intersects:
        _launch("forward", "get_tile_bin_edges", _blocks(num_intersects), (N_THREADS, 1, 1),
                [_i(num_intersects), _ptr(isect_ids_sorted), _ptr(bins)])
    return bins


def texture_forward(tile_bounds, block, img_size, texture_info, texture_dims, gaussian_ids_sorted, tile_bins, colors,
                    opacity, means, scales, glob_scale, quats, uv0, umap, vmap, texture, viewmat, c2w, fx, fy, cx,
                    cy, settings, background):
    """texture.cu:766-901.  Returns (img, depth, reg, texture, normal,
    final_T, final_idx, depth_idx, reg_s)."""
    W, H = img_size[0], img_size[1]
    C = texture_info[2]
    assert colors.shape[1] == 3 and block[0] * block[1] <= 256 and C <= 64
    assert texture.dim() == 2 and texture.shape[1] == C and background.numel() == 3
    dev = means.device
    z = lambda *s, dt=torch.float32: torch.zeros(s, dtype=dt, device=dev)  # noqa: E731
    img, final_T, final_idx, depth = z(H, W, 3), z(H, W), z(H, W, dt=torch.int32), z(H, W)
    depth_idx, reg, reg_s, tex, normal = z(H, W, dt=torch.int32), z(H, W), z(H, W, 3), z(H, W, C), z(H, W, 3)
    _launch("texture", "texture_forward", tile_bounds, block,
            [Dim3(*tile_bounds), Dim3(*img_size), Int3(*texture_info), _ptr(texture_dims), _ptr(gaussian_ids_sorted),
             _ptr(tile_bins), _ptr(colors), _ptr(opacity), _ptr(means), _ptr(scales), _f(glob_scale), _ptr(quats),
             _ptr(uv0), _ptr(umap), _ptr(vmap), _ptr(texture), _ptr(viewmat), _ptr(c2w), Float4(fx, fy, cx, cy),
             _i(settings), _ptr(background), _ptr(final_T), _ptr(final_idx), _ptr(depth_idx), _ptr(reg_s), _ptr(img),
             _ptr(depth), _ptr(reg), _ptr(tex), _ptr(normal)])
    return img, depth, reg, tex, normal, final_T, final_idx, depth_idx, reg_s


def texture_backward(img_height, img_width, block_width, texture_info, texture_dims, gaussian_ids_sorted, tile_bins,
                     colors, opacity, means, scales, glob_scale, quats, uv0, umap, vmap, texture, viewmat, c2w, fx,
                     fy, cx, cy, settings, background, final_T, final_idx, depth_idx, reg_s, v_img, v_depth, v_reg,
                     v_alpha, v_texture_out, v_normal):
    """texture.cu:915-1052.  Returns (v_colors, v_opacity, v_means, v_scales,
    v_quats, v_uv0, v_umap, v_vmap, v_texture)."""
    tb = ((img_width + block_width - 1) // block_width, (img_height + block_width - 1) // block_width, 1)
    N = means.shape[0]
    P = texture_info[1]
    C = texture_info[2]
    assert block_width * block_width <= 256 and C <= 64 and texture.shape[1] == C
    dev = means.device
    z = lambda *s: torch.zeros(s, dtype=torch.float32, device=dev)  # noqa: E731
    v_colors, v_opac, v_means, v_scales, v_quats = z(N, 3), z(N, 1), z(N, 3), z(N, 3), z(N, 4)
    v_uv0, v_umap, v_vmap, v_tex = z(N, P, 2), z(N, P, 3), z(N, P, 3), z(texture.shape[0], C)
    _launch("texture", "texture_backward", tb, (block_width, block_width, 1),
            [Dim3(*tb), Dim3(img_width, img_height, 1), Int3(*texture_info), _ptr(texture_dims),
             _ptr(gaussian_ids_sorted), _ptr(tile_bins), _ptr(colors), _ptr(opacity), _ptr(means), _ptr(scales),
             _f(glob_scale), _ptr(quats), _ptr(uv0), _ptr(umap), _ptr(vmap), _ptr(texture), _ptr(viewmat), _ptr(c2w),
             Float4(fx, fy, cx, cy), _i(settings), _ptr(background), _ptr(final_T), _ptr(final_idx), _ptr(depth_idx),
             _ptr(reg_s), _ptr(v_img), _ptr(v_depth), _ptr(v_reg), _ptr(v_alpha), _ptr(v_texture_out),
             _ptr(v_normal), _ptr(v_colors), _ptr(v_opac), _ptr(v_means), _ptr(v_scales), _ptr(v_quats), _ptr(v_uv0),
             _ptr(v_umap), _ptr(v_vmap), _ptr(v_tex)])
    return v_colors, v_opac, v_means, v_scales, v_quats, v_uv0, v_umap, v_vmap, v_tex


def texture_sample_forward(texture_info, texture_dims, uvs, texture):
    """texture_sample.cu:72-106.  The kernel clamps only the upper texel
    index (texture_helpers.cuh:155-160) and the reference wrapper passes the
    uvs through unclamped, so uvs must lie in [0, 1] here."""
    assert bool(((uvs >= 0) & (uvs <= 1)).all()), "reference texture_sample_forward reads out of range for uv < 0"
    Q = uvs.shape[0]
    out = torch.zeros((Q, texture_info[2]), device=uvs.device)
    if Q:
        _launch("texture_sample", "texture_sample_forward", _blocks(Q), (N_THREADS, 1, 1),
                [_i(Q), Int3(*texture_info), _ptr(texture_dims), _ptr(uvs), _ptr(texture), _ptr(out)])
    return out


def texture_edit(tile_bounds, block, img_size, texture_info, texture_total_size, texture_dims, updated_img,
                 updated_alpha, depth_lower, depth_upper, gaussian_ids_sorted, tile_bins, opacity, means, scales,
                 glob_scale, quats, uv0, umap, vmap, viewmat, c2w, fx, fy, cx, cy, settings, background):
    """texture_edit.cu:238-346.  The kernel writes five channels at a stride
    of texture_info[2], so anything but 5 would write out of range."""
    assert texture_info[2] == 5, "reference texture_edit needs texture_info[2] == 5"
    assert block[0] * block[1] <= 256 and background.numel() == 3
    out = torch.zeros((int(texture_total_size), 5), device=means.device)
    _launch("texture_edit", "texture_edit", tile_bounds, block,
            [Dim3(*tile_bounds), Dim3(*img_size), Int3(*texture_info), _ptr(texture_dims), _ptr(updated_img),
             _ptr(updated_alpha), _ptr(depth_lower), _ptr(depth_upper), _ptr(gaussian_ids_sorted), _ptr(tile_bins),
             _ptr(opacity), _ptr(means), _ptr(scales), _f(glob_scale), _ptr(quats), _ptr(uv0), _ptr(umap),
             _ptr(vmap), _ptr(viewmat), _ptr(c2w), Float4(fx, fy, cx, cy), _i(settings), _ptr(background),
             _ptr(out)])
    return out


# texture_sample_backward (texture_sample.cu:38-70) is not wrapped: it reads
# its upstream gradient from its own output array (v_texture indexed by the
# query), which races with its own atomics and reads past that array when
# there are more queries than texels.


# ---------------------------------------------------------------------------
# The reference's Python glue for one view (restated)
# ---------------------------------------------------------------------------
def num_tiles_hit(centers, extents, img_height, img_width, block_width):
    """get_aabb_2d.py:70-91: floor((c - e)/bw) and floor((c + e)/bw + 1),
    clamped to the tile grid, product of the two spans."""
    tx = (img_width + block_width - 1) // block_width
    ty = (img_height + block_width - 1) // block_width
    lo = torch.floor((centers - extents) / block_width).to(torch.int32)
    hi = torch.floor((centers + extents) / block_width + 1).to(torch.int32)
    lo = torch.stack([lo[:, 0].clamp(0, tx), lo[:, 1].clamp(0, ty)], -1)
    hi = torch.stack([hi[:, 0].clamp(0, tx), hi[:, 1].clamp(0, ty)], -1)
    span = hi - lo
    return (span[:, 0] * span[:, 1]).to(torch.int32)


def bin_and_sort(num_points, centers, extents, depths, counts, tile_bounds, block_width):
    """utils.py:40-59 and 117-161: int32 inclusive sum and its host read,
    emission, ``torch.sort`` of the 64-bit keys, gather of the ids, tile
    ranges.  Returns (n_isect, isect_sorted, gids_sorted, bins)."""
    cum = torch.cumsum(counts, dim=0, dtype=torch.int32)
    n = int(cum[-1].item()) if num_points else 0
    isect, gids = map_gaussian_to_intersects(num_points, n, centers, extents, depths, cum, tile_bounds, block_width)
    isect_sorted, order = torch.sort(isect)
    gids_sorted = torch.gather(gids, 0, order)
    bins = get_tile_bin_edges(n, isect_sorted, tile_bounds)
    return n, isect_sorted, gids_sorted, bins


# ---------------------------------------------------------------------------
# One view the way a caller of the reference renders it (restated glue of
# example.py:121-209: SH colours, AABBs, depths, tile counts, host-synchronising
# binning, texture_forward; texture_backward and the SH adjoint), used by the
# full-size batched parity test and by the benchmark's timing of the
# reference's plain per-view fp32 path.
# ---------------------------------------------------------------------------
def view_forward(t, cam, sh_degree, block_width=16, settings=1 << 8, background=None, binning=None):
    """t: dict of float32 / int32 CUDA tensors means, scales, quats, opacity,
    uv0, umap, vmap, dims, texture [T, C], sh [N, B, 3]; cam: a camera with
    viewmat, c2w (CPU [4, 4]), fx, fy, cx, cy, width, height.  Returns a dict
    with the view's colours, binning (n, gids_sorted, bins, tile_bounds),
    inputs of texture_backward and the nine forward outputs.  binning =
    (gaussian_ids_sorted, tile_bins) replaces the reference's own binning
    (the compositor kernels then run on the given lists)."""
    dev = t["means"].device
    N = t["means"].shape[0]
    H, W, bw = cam.height, cam.width, block_width
    vm = cam.viewmat.contiguous().to(dev)
    c2w = cam.c2w.contiguous().to(dev)
    dirs = (t["means"] - c2w[:3, 3][None]).contiguous()
    colors = compute_sh_forward(N, sh_degree, sh_degree, dirs, t["sh"])
    intr = (cam.fx, cam.fy, cam.cx, cam.cy)
    tb = ((W + bw - 1) // bw, (H + bw - 1) // bw, 1)
    if binning is None:
        centers, extents = get_aabb_2d(t["means"], t["scales"], 1.0, t["quats"], vm, *intr)
        depths = (t["means"] @ vm.T[:3, :3] + vm.T[3:, :3])[:, 2].contiguous()
        counts = num_tiles_hit(centers, extents, H, W, bw)
        n, isect_sorted, gids, bins = bin_and_sort(N, centers, extents, depths, counts, tb, bw)
    else:
        gids, bins = binning
        n, isect_sorted = int(gids.numel()), None
    bg = background if background is not None else torch.zeros(3, device=dev)
    C = t["texture"].shape[1]
    common = ((N, 1, C), t["dims"], gids, bins, colors, t["opacity"], t["means"], t["scales"], 1.0, t["quats"],
              t["uv0"], t["umap"], t["vmap"], t["texture"], vm, c2w, *intr, settings, bg)
    names = ("img", "depth", "reg", "texture", "normal", "final_T", "final_idx", "depth_idx", "reg_s")
    outs = dict(zip(names, texture_forward(tb, (bw, bw, 1), (W, H, 1), *common)))
    return dict(colors=colors, dirs=dirs, n=n, isect_sorted=isect_sorted, gids_sorted=gids, bins=bins,
                tile_bounds=tb, common=common, out=outs)


def view_backward(t, cam, sh_degree, fwd, ups, block_width=16):
    """texture_backward and the SH adjoint of one view rendered by
    view_forward, for upstream gradients ups (dict of CUDA tensors img,
    texture, normal, reg; depth and alpha optional).  Returns the nine
    gradients of texture_backward plus 'sh_coeffs'."""
    o = fwd["out"]
    z = torch.zeros_like(o["reg"])
    g = texture_backward(cam.height, cam.width, block_width, *fwd["common"], o["final_T"], o["final_idx"],
                         o["depth_idx"].clone(), o["reg_s"], ups["img"].contiguous(),
                         ups.get("depth", z).contiguous(), ups["reg"].contiguous(), ups.get("alpha", z).contiguous(),
                         ups["texture"].contiguous(), ups["normal"].contiguous())
    names = ("colors", "opacity", "means", "scales", "quats", "uv0", "umap", "vmap", "texture")
    grads = dict(zip(names, g))
    N = t["means"].shape[0]
    grads["sh_coeffs"] = compute_sh_backward(N, sh_degree, sh_degree, fwd["dirs"], grads["colors"])
    return grads


def image_loss_grads(out, tgt_img, tgt_tex, weights):
    """Upstream gradients of the demo's image losses (example.py:189-209:
    w_img MSE(img) + w_tex MSE(texture) + w_reg mean(reg) + w_normal
    mean |n - (0, 0, 1)|^2), by elementwise torch as the reference's autograd
    computes them."""
    H, W = out["reg"].shape
    inv = 1.0 / (H * W)
    z = torch.tensor([0.0, 0.0, 1.0], device=out["img"].device)
    return dict(img=(2 * weights["img"] * inv / 3) * (out["img"] - tgt_img),
                texture=(2 * weights["texture"] * inv / 3) * (out["texture"] - tgt_tex),
                reg=torch.full_like(out["reg"], weights["reg"] * inv),
                normal=(2 * weights["normal"] * inv) * (out["normal"] - z))
