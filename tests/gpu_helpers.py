"""Shared helpers of the GPU parity tests: one seeded scene, fed identically
to the CUDA library (torch tensors on cuda:0) and to the CPU oracle (numpy)."""
from __future__ import annotations

import numpy as np
import torch

import oracle
from gstex_cuda_gb300 import synthetic


def colors_of(spec, cam):
    """Per-Gaussian RGB from the SH coefficients, float64 numpy (test input)."""
    d = (spec.means - cam.position[None, :]).double().numpy()
    return oracle.sh_forward(spec.sh_degree, spec.sh_degree, d, spec.sh_coeffs.double().numpy(), prec="f64")


def small_scene(n=200, width=64, height=64, seed=5, f=None, chart=(4, 6), scale=(0.05, 0.5), z=(2.0, 4.0),
                channels=3):
    """Random textured scene in front of an identity camera."""
    g = torch.Generator().manual_seed(seed)
    f = f if f is not None else float(max(width, height))
    means = torch.empty(n, 3)
    means[:, 0].uniform_(-0.6 * width / f * 2, 0.6 * width / f * 2, generator=g)
    means[:, 1].uniform_(-0.6 * height / f * 2, 0.6 * height / f * 2, generator=g)
    means[:, 2].uniform_(*z, generator=g)
    s2 = torch.exp(torch.empty(n, 2).uniform_(np.log(scale[0]), np.log(scale[1]), generator=g))
    scales = torch.cat([s2, 1e-5 * s2.mean(-1, keepdim=True)], -1)
    quats = torch.randn(n, 4, generator=g)
    quats = quats / quats.norm(dim=-1, keepdim=True)
    opacity = torch.sigmoid(torch.randn(n, 1, generator=g))
    w, x, y, zq = quats.unbind(-1)
    ax1 = torch.stack([1 - 2 * (y * y + zq * zq), 2 * (x * y + w * zq), 2 * (x * zq - w * y)], -1)
    ax2 = torch.stack([2 * (x * y - w * zq), 1 - 2 * (x * x + zq * zq), 2 * (y * zq + w * x)], -1)
    hw = torch.randint(chart[0], chart[1] + 1, (n, 2), generator=g).to(torch.int32)
    dims = torch.zeros(n, 3, dtype=torch.int32)
    dims[:, :2] = hw
    sizes = dims[:, 0].long() * dims[:, 1].long()
    dims[:, 2] = (torch.cumsum(sizes, 0) - sizes).to(torch.int32)
    tex = torch.rand(int(sizes.sum()), channels, generator=g)
    cam = synthetic.make_camera(torch.eye(4), width, height, f=f)
    return synthetic.SceneSpec(means=means, scales=scales, quats=quats, opacity=opacity, sh_degree=0,
                               sh_coeffs=torch.rand(n, 1, 3, generator=g), uv0=torch.full((n, 1, 2), 0.5),
                               umap=(ax1 / (6 * scales[:, :1]))[:, None], vmap=(ax2 / (6 * scales[:, 1:2]))[:, None],
                               texture_dims=dims, texture=tex, cameras=[cam], name="small")


class Case:
    """CUDA tensors and oracle inputs of one (scene, camera)."""

    def __init__(self, spec, cam_index=0, colors=None, dev="cuda:0"):
        self.spec = spec
        self.cam = cam = spec.cameras[cam_index]
        col = colors if colors is not None else colors_of(spec, cam)
        self.colors_np = np.asarray(col, np.float32)
        self.dev = torch.device(dev)
        t = dict(means=spec.means, scales=spec.scales, quats=spec.quats, opacity=spec.opacity,
                 colors=torch.from_numpy(self.colors_np), uv0=spec.uv0, umap=spec.umap, vmap=spec.vmap,
                 dims=spec.texture_dims, texture=spec.texture, viewmat=cam.viewmat, c2w=cam.c2w)
        self.t = {k: v.contiguous().to(self.dev) for k, v in t.items()}
        self.intr = (cam.fx, cam.fy, cam.cx, cam.cy)
        self.scene_np = oracle.Scene(means=spec.means.numpy(), scales=spec.scales.numpy(), quats=spec.quats.numpy(),
                                     opacity=spec.opacity.numpy(), colors=self.colors_np, uv0=spec.uv0.numpy(),
                                     umap=spec.umap.numpy(), vmap=spec.vmap.numpy(),
                                     texture_dims=spec.texture_dims.numpy(), texture=spec.texture.numpy())
        self.cam_np = oracle.Camera(cam.viewmat.numpy(), cam.c2w.numpy(), *self.intr, cam.height, cam.width)

    def binning_np(self, bw=16):
        sp, cam = self.spec, self.cam
        c, e = oracle.get_aabb_2d(sp.means.numpy(), sp.scales.numpy(), sp.glob_scale, sp.quats.numpy(),
                                  cam.viewmat.numpy(), *self.intr)
        depths = oracle.project_depths(sp.means.numpy(), cam.viewmat.numpy())
        nt = oracle.num_tiles_hit(c, e, cam.height, cam.width, bw)
        return dict(centers=c, extents=e, depths=depths, counts=nt,
                    **oracle.bin_and_sort(c, e, depths, nt, cam.height, cam.width, bw))

    def binning_cuda(self, bw=16):
        import gstex_cuda_gb300 as G
        cam = self.cam
        t = self.t
        c, e = G.get_aabb_2d.get_aabb_2d(t["means"], t["scales"], self.spec.glob_scale, t["quats"], t["viewmat"],
                                         self.intr)
        depths = torch.from_numpy(oracle.project_depths(self.spec.means.numpy(), cam.viewmat.numpy())).to(self.dev)
        nt = G.get_aabb_2d.get_num_tiles_hit_2d(c, e, cam.height, cam.width, bw)
        n_isect, cum = G.utils.compute_cumulative_intersects(nt)
        tb = ((cam.width + bw - 1) // bw, (cam.height + bw - 1) // bw, 1)
        res = G.utils.bin_and_sort_gaussians(self.spec.num_points, n_isect, c, e, depths, cum, tb, bw)
        return dict(centers=c, extents=e, depths=depths, counts=nt, cum=cum, n_isect=n_isect,
                    isect_ids=res[0], gaussian_ids=res[1], isect_ids_sorted=res[2], gaussian_ids_sorted=res[3],
                    tile_bins=res[4], tile_bounds=tb)

    def forward_cuda(self, gids_sorted, tile_bins, bw=16, settings=1 << 8, background=None, texture=None,
                     channels=None):
        import gstex_cuda_gb300 as G
        cam = self.cam
        t = self.t
        C = channels if channels is not None else self.spec.texture.shape[1]
        bg = torch.as_tensor(background if background is not None else np.zeros(3), dtype=torch.float32).to(self.dev)
        tb = ((cam.width + bw - 1) // bw, (cam.height + bw - 1) // bw, 1)
        tex = texture if texture is not None else t["texture"]
        outs = G.cuda.texture_forward(tb, (bw, bw, 1), (cam.width, cam.height, 1), (self.spec.num_points, 1, C),
                                      t["dims"], gids_sorted, tile_bins, t["colors"], t["opacity"], t["means"],
                                      t["scales"], self.spec.glob_scale, t["quats"], t["uv0"], t["umap"], t["vmap"],
                                      tex, t["viewmat"], t["c2w"], *self.intr, settings, bg)
        names = ("img", "depth", "reg", "texture", "normal", "final_T", "final_idx", "depth_idx", "reg_s")
        return dict(zip(names, outs)), bg

    def backward_cuda(self, fwd, gids_sorted, tile_bins, ups, bw=16, settings=1 << 8, bg=None, texture=None,
                      channels=None):
        import gstex_cuda_gb300 as G
        cam = self.cam
        t = self.t
        C = channels if channels is not None else self.spec.texture.shape[1]
        tex = texture if texture is not None else t["texture"]
        u = {k: torch.as_tensor(v, dtype=torch.float32).contiguous().to(self.dev) for k, v in ups.items()}
        grads = G.cuda.texture_backward(cam.height, cam.width, bw, (self.spec.num_points, 1, C), t["dims"],
                                        gids_sorted, tile_bins, t["colors"], t["opacity"], t["means"], t["scales"],
                                        self.spec.glob_scale, t["quats"], t["uv0"], t["umap"], t["vmap"], tex,
                                        t["viewmat"], t["c2w"], *self.intr, settings, bg, fwd["final_T"],
                                        fwd["final_idx"], fwd["depth_idx"], fwd["reg_s"], u["img"], u["depth"],
                                        u["reg"], u["alpha"], u["texture"], u["normal"])
        names = ("colors", "opacity", "means", "scales", "quats", "uv0", "umap", "vmap", "texture")
        return dict(zip(names, grads))


def close_frac(got, ref, tol, frac, name, cap=None):
    """|got - ref| <= tol everywhere, except for at most a fraction ``frac`` of
    elements (pixels where a float rounding difference flips one of the
    reference's hard thresholds: alpha >= 1/255, T <= 1e-4, T > 0.5), which
    must still stay below 1e-2 (relative to the value's size)."""
    err = np.abs(np.asarray(got, np.float64) - np.asarray(ref, np.float64))
    if err.size == 0:
        return
    bad = err > tol
    assert bad.mean() <= frac, (name, float(bad.mean()), float(err.max()))
    cap = 1e-2 * (1 + np.abs(ref)) if cap is None else cap
    assert np.all(err < np.maximum(cap, tol)), (name, float(err.max()))


def upstream(H, W, C, seed=7):
    g = np.random.default_rng(seed)
    return dict(img=g.standard_normal((H, W, 3)), depth=g.standard_normal((H, W)), reg=g.standard_normal((H, W)),
                alpha=g.standard_normal((H, W)), texture=g.standard_normal((H, W, C)),
                normal=g.standard_normal((H, W, 3)))


def np_(t):
    """numpy copy of a tensor: floating types as float32, integer types kept
    (a float32 copy would round indices above 2^24)."""
    if not isinstance(t, torch.Tensor):
        return np.asarray(t)
    t = t.detach()
    return (t if not t.is_floating_point() else t.float()).cpu().numpy()
