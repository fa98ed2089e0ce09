"""Per-output error of the CUDA path against the fp64 oracle.

For each configuration the CUDA library renders one view (texture_forward,
texture_backward through the C ABI) and the fp64 oracle (the C restatement
of the reference's kernels, compiled with doubles) renders the same view from
the same float32 inputs on the same binning; both backward passes get the
same upstream gradients (seeded standard normal per pixel on every output,
so that each adjoint path is exercised).  For every output (img, depth, reg,
alpha = 1 - final_T, texture, normal) the report gives the largest and the
99.9th-percentile absolute error; for every gradient (colours, opacity,
means, scales, quaternions, uv0, umap, vmap, texels) the same absolute
figures and both divided by the largest |fp64 gradient| entry.

Configurations (the reference's benchmark shapes):
  config1        32x32, 10 Gaussians, 4x4 RGB charts (fp32 texels)
  fd_crop        64x64 crop with 200 Gaussians (the finite-difference scene)
  config2        800x800, 100k untextured Gaussians (1x1 charts), SH degree 3
  config3_crop   the central 512x512 window of the 1920x1080, 200k-Gaussian,
                 8M-texel view (fp32 texels, then bf16 texels compared with the
                 fp64 oracle at the stored bf16 values and at the fp32 values)

Test infrastructure (runs on a GPU; the oracle is the checker).  Used by
tests/test_gpu_fp64_report.py, which asserts the bars and, when
GSTEX_FP64_REPORT names a file, writes the report there as JSON.
"""
from __future__ import annotations

import numpy as np
import torch

import oracle
from gpu_helpers import Case, colors_of, np_, small_scene, upstream

OUTPUTS = ("img", "depth", "reg", "alpha", "texture", "normal")
GRADS = ("colors", "opacity", "means", "scales", "quats", "uv0", "umap", "vmap", "texture")


def _stats(err, scale=None):
    err = np.abs(np.asarray(err, np.float64)).reshape(-1)
    if err.size == 0:
        return {"max_abs": 0.0, "p999_abs": 0.0}
    d = {"max_abs": float(err.max()), "p999_abs": float(np.quantile(err, 0.999))}
    if scale is not None:
        s = max(float(scale), 1e-30)
        d["max_rel"] = d["max_abs"] / s
        d["p999_rel"] = d["p999_abs"] / s
    return d


def _crop_1080p():
    """The central 512x512 window of the 1920x1080 view (f = 960): the same
    Gaussians and texels, a camera whose principal point is shifted so that
    pixel (0, 0) of the window is pixel (704, 284) of the full view."""
    from gstex_cuda_gb300 import synthetic
    spec = synthetic.textured_1080p(seed=2)
    full = spec.cameras[0]
    spec.cameras = [synthetic.make_camera(full.viewmat, 512, 512, f=full.fx, cx=full.cx - 704.0,
                                          cy=full.cy - 284.0)]
    return spec


def _fd_scene():
    spec = small_scene(n=200, width=64, height=64, seed=21, f=96.0, chart=(3, 6))
    spec.umap.mul_(0.5)
    spec.vmap.mul_(0.5)
    spec.opacity.clamp_(max=0.95)
    return spec


def config_report(spec, texture_mode="f32", oracle_texture="stored", bw=16, settings=1 << 8):
    """Errors of one view.  texture_mode "bf16" renders with bf16 texels
    [T, 4]; oracle_texture "stored" gives the oracle the values the CUDA path
    computes with, "fp32" the unrounded ones (the storage error included)."""
    case = Case(spec, colors=colors_of(spec, spec.cameras[0]))
    cam = case.cam
    H, W = cam.height, cam.width
    C = spec.texture.shape[1]
    b = case.binning_cuda(bw)
    gids, bins = b["gaussian_ids_sorted"], b["tile_bins"]
    tex_cuda = None
    tex_oracle = spec.texture.double().numpy()
    if texture_mode == "bf16":
        t16 = torch.zeros(spec.texture.shape[0], 4, dtype=torch.bfloat16)
        t16[:, :3] = spec.texture.to(torch.bfloat16)
        tex_cuda = t16.to(case.dev)
        if oracle_texture == "stored":
            tex_oracle = t16[:, :3].double().numpy()
    bg = np.zeros(3)
    fwd, bgt = case.forward_cuda(gids, bins, bw, settings, bg, texture=tex_cuda, channels=C)
    ups = upstream(H, W, C, seed=7)
    grads = case.backward_cuda(fwd, gids, bins, ups, bw, settings, bgt, texture=tex_cuda, channels=C)
    torch.cuda.synchronize()
    sc = case.scene_np
    sc.texture = tex_oracle
    # integer arrays straight to numpy (through float32 the offsets above 2^24 would round)
    gn, bn = gids.cpu().numpy().astype(np.int32), bins.cpu().numpy().astype(np.int32)
    ref = oracle.texture_forward(sc, case.cam_np, gn, bn, bw, settings, bg, prec="f64")
    gref = oracle.texture_backward(sc, case.cam_np, gn, bn, bw, settings, bg, ref, ups["img"], ups["depth"],
                                   ups["reg"], ups["alpha"], ups["texture"], ups["normal"], prec="f64")
    outs = {}
    for k in OUTPUTS:
        if k == "alpha":
            got, want = 1.0 - np_(fwd["final_T"]), 1.0 - np.asarray(ref["final_T"])
        else:
            got, want = np_(fwd[k]), np.asarray(ref[k])
        outs[k] = _stats(got.reshape(-1) - want.reshape(-1))
    gr = {}
    for k in GRADS:
        want = np.asarray(gref[k], np.float64)
        got = np_(grads[k])
        if want.size == 0:
            continue
        want = want.reshape(want.shape[0], -1)
        got = got.reshape(want.shape[0], -1)[:, :want.shape[1]]
        if k == "scales":  # the third scale gets no gradient
            got, want = got[:, :2], want[:, :2]
        gr[k] = _stats(got - want, np.abs(want).max())
    info = {"width": W, "height": H, "gaussians": spec.num_points, "texels": int(spec.texture.shape[0]),
            "intersections": int(b["n_isect"]), "texture": texture_mode,
            "oracle_texture": oracle_texture if texture_mode == "bf16" else "fp32"}
    return {"info": info, "outputs": outs, "gradients": gr}


def build_report():
    from gstex_cuda_gb300 import synthetic
    rep = {}
    rep["config1_32x32_10"] = config_report(synthetic.tiny(0))
    rep["fd_crop_64x64_200"] = config_report(_fd_scene())
    rep["config2_800x800_100k_untextured"] = config_report(synthetic.untextured(seed=1))
    crop = _crop_1080p()
    rep["config3_crop512_fp32"] = config_report(crop)
    rep["config3_crop512_bf16_vs_stored"] = config_report(crop, "bf16", "stored")
    rep["config3_crop512_bf16_vs_fp32"] = config_report(crop, "bf16", "fp32")
    return rep
