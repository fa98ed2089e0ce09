"""Seeded synthetic scenes with the shapes of the reference's benchmark workloads.

Conventions follow the reference demo (example.py:62-143 of the reference
project): OpenCV pinhole cameras (x right, y down, +z forward), ``viewmat`` is
world->camera row-major 4x4 and ``c2w`` its inverse, ``glob_scale = 1``, the
third scale axis is ``1e-5 * mean(scale_x, scale_y)``, quaternions are
normalised (w, x, y, z), each Gaussian's texture chart maps its +-3 sigma
ellipse onto [0,1]^2 (``uv0 = (0.5, 0.5)``, ``umap = ax1 / (6 s_x)``,
``vmap = ax2 / (6 s_y)``), ``texture_dims[:, 2]`` is the exclusive cumsum of
``h * w`` and ``settings = 1 << 8``.

Everything is generated on the CPU with ``torch.Generator().manual_seed``;
callers move tensors to the device they want.  The five workloads:

* ``tiny``      - one 32x32 view (f=32), 10 Gaussians, 4x4 RGB charts, SH deg 0.
* ``untextured``- one 800x800 view (f=400) from distance 8, 100k Gaussians in
  [-3,3]^3, scales log-U[0.005,0.05], SH deg 3, 1x1 charts.
* ``textured_1080p`` - one 1920x1080 view (f=960), 200k Gaussians with the tiny
  scene's distributions, an 8M-texel budget split by projected area.
* ``batched``   - 32 cameras on a radius-8 sphere with resolutions drawn from
  {512^2, 800^2, 1280x720, 1920x1080}, 500k Gaussians, 16M texels, SH deg 3.
* ``stress``    - 8 1080p views, 1M Gaussians clustered in 64 blobs
  (sigma 0.3), 32M texels, SH deg 3.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional

import torch

SETTINGS_DEFAULT = 1 << 8


@dataclass
class Camera:
    viewmat: torch.Tensor  # [4,4] float32 world->camera
    c2w: torch.Tensor      # [4,4] float32
    fx: float
    fy: float
    cx: float
    cy: float
    height: int
    width: int

    @property
    def position(self) -> torch.Tensor:
        return self.c2w[:3, 3]


@dataclass
class SceneSpec:
    means: torch.Tensor
    scales: torch.Tensor
    quats: torch.Tensor
    opacity: torch.Tensor
    sh_degree: int
    sh_coeffs: torch.Tensor        # [N, B, 3]
    uv0: torch.Tensor
    umap: torch.Tensor
    vmap: torch.Tensor
    texture_dims: torch.Tensor     # [N,3] int32
    texture: torch.Tensor          # [T,C] float32
    cameras: List[Camera]
    glob_scale: float = 1.0
    settings: int = SETTINGS_DEFAULT
    background: torch.Tensor = field(default_factory=lambda: torch.zeros(3))
    name: str = ""
    loss_weights: dict = field(default_factory=dict)

    @property
    def num_points(self) -> int:
        return self.means.shape[0]

    @property
    def num_texels(self) -> int:
        return self.texture.shape[0]

    def texture_info(self):
        return (self.num_points, 1, self.texture.shape[1])


def look_at(position, target=(0.0, 0.0, 0.0)) -> tuple:
    """World->camera (OpenCV axes) for a camera at ``position`` looking at ``target``."""
    c = torch.as_tensor(position, dtype=torch.float64)
    f = torch.as_tensor(target, dtype=torch.float64) - c
    f = f / f.norm()
    up = torch.tensor([0.0, -1.0, 0.0], dtype=torch.float64)
    if abs(float(f @ up)) > 0.99:
        up = torch.tensor([0.0, 0.0, 1.0], dtype=torch.float64)
    right = torch.linalg.cross(f, up)
    right = right / right.norm()
    down = torch.linalg.cross(f, right)
    Rc2w = torch.stack([right, down, f], dim=1)
    c2w = torch.eye(4, dtype=torch.float64)
    c2w[:3, :3] = Rc2w
    c2w[:3, 3] = c
    viewmat = torch.linalg.inv(c2w)
    return viewmat.float(), c2w.float()


def make_camera(viewmat, width, height, f=None, cx=None, cy=None) -> Camera:
    viewmat = viewmat.float()
    c2w = torch.linalg.inv(viewmat.double()).float()
    f = float(width) / 2.0 if f is None else float(f)
    return Camera(viewmat, c2w, f, f, width / 2.0 if cx is None else cx, height / 2.0 if cy is None else cy,
                  int(height), int(width))


def _quat_axes(q: torch.Tensor):
    w, x, y, z = q.unbind(-1)
    ax1 = torch.stack([1 - 2 * (y * y + z * z), 2 * (x * y + w * z), 2 * (x * z - w * y)], -1)
    ax2 = torch.stack([2 * (x * y - w * z), 1 - 2 * (x * x + z * z), 2 * (y * z + w * x)], -1)
    return ax1, ax2


def _finish(g, means, log_lo, log_hi, sh_degree, sh_mode, charts_hw, cameras, name, loss_weights):
    n = means.shape[0]
    s2 = torch.exp(torch.empty(n, 2).uniform_(math.log(log_lo), math.log(log_hi), generator=g))
    scales = torch.cat([s2, 1e-5 * s2.mean(-1, keepdim=True)], -1)
    quats = torch.randn(n, 4, generator=g)
    quats = quats / quats.norm(dim=-1, keepdim=True)
    opacity = torch.sigmoid(torch.randn(n, 1, generator=g))
    nb = {0: 1, 1: 4, 2: 9, 3: 16}.get(sh_degree, 25)
    if sh_mode == "uniform":
        sh = torch.rand(n, nb, 3, generator=g)
    else:
        sh = 0.2 * torch.randn(n, nb, 3, generator=g)
    ax1, ax2 = _quat_axes(quats)
    uv0 = torch.full((n, 1, 2), 0.5)
    umap = (ax1 / (6.0 * scales[:, :1]))[:, None, :]
    vmap = (ax2 / (6.0 * scales[:, 1:2]))[:, None, :]
    hw = charts_hw(scales) if callable(charts_hw) else charts_hw
    dims = torch.zeros(n, 3, dtype=torch.int32)
    dims[:, 0] = hw[:, 0]
    dims[:, 1] = hw[:, 1]
    sizes = (dims[:, 0].long() * dims[:, 1].long())
    dims[:, 2] = (torch.cumsum(sizes, 0) - sizes).to(torch.int32)
    T = int(sizes.sum())
    texture = torch.rand(T, 3, generator=g)
    return SceneSpec(means=means, scales=scales, quats=quats, opacity=opacity, sh_degree=sh_degree,
                     sh_coeffs=sh, uv0=uv0, umap=umap, vmap=vmap, texture_dims=dims, texture=texture,
                     cameras=cameras, name=name, loss_weights=loss_weights)


def _aabb_area(means, scales, quats, cam: Camera):
    """4 * ext_x * ext_y of the 4-corner +-3 sigma screen AABB (float64, torch)."""
    ax1, ax2 = _quat_axes(quats.double())
    m = means.double()
    s = scales.double()
    V = cam.viewmat.double()
    corners = []
    for a in (1, -1):
        for b in (1, -1):
            corners.append(m + 3 * a * s[:, :1] * ax1 + 3 * b * s[:, 1:2] * ax2)
    pix = []
    for c in corners:
        pv = c @ V[:3, :3].T + V[:3, 3]
        z = pv[:, 2].clamp(min=0.01)
        pix.append(torch.stack([pv[:, 0] / z * cam.fx + cam.cx, pv[:, 1] / z * cam.fy + cam.cy], -1))
    p = torch.stack(pix, 1)
    ext = 0.5 * (p.max(1).values - p.min(1).values)
    zc = (m @ V[:3, :3].T + V[:3, 3])[:, 2]
    a = 4 * ext[:, 0] * ext[:, 1]
    return torch.where(zc > 0.01, a, torch.zeros_like(a))


def tiny(seed: int = 0) -> SceneSpec:
    g = torch.Generator().manual_seed(seed)
    n = 10
    means = torch.empty(n, 3)
    means[:, :2].uniform_(-1, 1, generator=g)
    means[:, 2].uniform_(2, 4, generator=g)
    cam = make_camera(torch.eye(4), 32, 32, f=32, cx=16, cy=16)
    hw = torch.full((n, 2), 4, dtype=torch.int32)
    return _finish(g, means, 0.05, 0.5, 0, "uniform", hw, [cam], "tiny", dict(texture=1.0, img=1.0))


def untextured(seed: int = 1, n: int = 100_000, size: int = 800) -> SceneSpec:
    g = torch.Generator().manual_seed(seed)
    means = torch.empty(n, 3).uniform_(-3, 3, generator=g)
    vm, _ = look_at((0.0, 0.0, -8.0))
    cam = make_camera(vm, size, size, f=size / 2)
    hw = torch.ones(n, 2, dtype=torch.int32)
    return _finish(g, means, 0.005, 0.05, 3, "normal", hw, [cam], "untextured",
                   dict(texture=1.0, reg=100.0, normal=0.05))


def textured_1080p(seed: int = 2, n: int = 200_000, texels: int = 8_000_000) -> SceneSpec:
    g = torch.Generator().manual_seed(seed)
    means = torch.empty(n, 3)
    means[:, :2].uniform_(-1, 1, generator=g)
    means[:, 2].uniform_(2, 4, generator=g)
    cam = make_camera(torch.eye(4), 1920, 1080, f=960)
    return _finish_with_area(g, means, 0.05, 0.5, 0, "uniform", [cam], texels, "textured_1080p",
                             dict(texture=1.0, img=1.0, reg=100.0, normal=0.05))


def _finish_with_area(g, means, log_lo, log_hi, sh_degree, sh_mode, cameras, texels, name, lw):
    n = means.shape[0]
    s2 = torch.exp(torch.empty(n, 2).uniform_(math.log(log_lo), math.log(log_hi), generator=g))
    scales = torch.cat([s2, 1e-5 * s2.mean(-1, keepdim=True)], -1)
    quats = torch.randn(n, 4, generator=g)
    quats = quats / quats.norm(dim=-1, keepdim=True)
    area = torch.zeros(n, dtype=torch.float64)
    for cam in cameras:
        area += _aabb_area(means, scales, quats, cam)
    area = area / len(cameras)
    side = torch.sqrt(texels * area / max(float(area.sum()), 1e-30)).round().clamp(2, 16).to(torch.int32)
    hw = torch.stack([side, side], -1)
    opacity = torch.sigmoid(torch.randn(n, 1, generator=g))
    nb = {0: 1, 1: 4, 2: 9, 3: 16}.get(sh_degree, 25)
    sh = torch.rand(n, nb, 3, generator=g) if sh_mode == "uniform" else 0.2 * torch.randn(n, nb, 3, generator=g)
    ax1, ax2 = _quat_axes(quats)
    uv0 = torch.full((n, 1, 2), 0.5)
    umap = (ax1 / (6.0 * scales[:, :1]))[:, None, :]
    vmap = (ax2 / (6.0 * scales[:, 1:2]))[:, None, :]
    dims = torch.zeros(n, 3, dtype=torch.int32)
    dims[:, 0] = hw[:, 0]
    dims[:, 1] = hw[:, 1]
    sizes = dims[:, 0].long() * dims[:, 1].long()
    dims[:, 2] = (torch.cumsum(sizes, 0) - sizes).to(torch.int32)
    texture = torch.rand(int(sizes.sum()), 3, generator=g)
    return SceneSpec(means=means, scales=scales, quats=quats, opacity=opacity, sh_degree=sh_degree,
                     sh_coeffs=sh, uv0=uv0, umap=umap, vmap=vmap, texture_dims=dims, texture=texture,
                     cameras=cameras, name=name, loss_weights=lw)


def sphere_cameras(g, count, radius=8.0, resolutions=None):
    cams = []
    res = resolutions or [(512, 512), (800, 800), (1280, 720), (1920, 1080)]
    for _ in range(count):
        v = torch.randn(3, generator=g)
        v = v / v.norm() * radius
        w, h = res[int(torch.randint(len(res), (1,), generator=g))]
        vm, _ = look_at(tuple(float(x) for x in v))
        cams.append(make_camera(vm, w, h))
    return cams


def batched(seed: int = 3, n: int = 500_000, texels: int = 16_000_000, views: int = 32) -> SceneSpec:
    g = torch.Generator().manual_seed(seed)
    cams = sphere_cameras(g, views)
    means = torch.empty(n, 3).uniform_(-3, 3, generator=g)
    return _finish_with_area(g, means, 0.005, 0.05, 3, "normal", cams, texels, "batched",
                             dict(texture=1.0, img=1.0, reg=100.0, normal=0.05))


def stress(seed: int = 4, n: int = 1_000_000, texels: int = 32_000_000, views: int = 8) -> SceneSpec:
    g = torch.Generator().manual_seed(seed)
    cams = sphere_cameras(g, views, resolutions=[(1920, 1080)])
    centres = torch.empty(64, 3).uniform_(-3, 3, generator=g)
    which = torch.randint(64, (n,), generator=g)
    means = centres[which] + 0.3 * torch.randn(n, 3, generator=g)
    return _finish_with_area(g, means, 0.005, 0.05, 3, "normal", cams, texels, "stress",
                             dict(texture=1.0, img=1.0, reg=100.0, normal=0.05))


def sh_viewdirs(spec: SceneSpec, cam: Camera) -> torch.Tensor:
    return spec.means - cam.position[None, :]
