"""Edge cases of the rasteriser path: scenes with nothing on screen, a view
with no intersections inside a batch, intersection-buffer overflow in the
batched path, screen-covering splats, and an empty scene."""
import numpy as np
import pytest
import torch

import oracle
from gpu_helpers import Case, np_, small_scene, upstream

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


@pytest.fixture(scope="module", autouse=True)
def _require():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import gstex_cuda_gb300  # noqa: F401


def _render(spec, bg=(0.25, 0.5, 0.75), grad=True):
    import gstex_cuda_gb300 as G
    case = Case(spec)
    cam, t = case.cam, case.t
    intr = case.intr
    for k in ("means", "scales", "quats", "opacity", "colors", "uv0", "umap", "vmap", "texture"):
        t[k].requires_grad_(grad)
    c, e = G.get_aabb_2d.get_aabb_2d(t["means"].detach(), t["scales"].detach(), 1.0, t["quats"].detach(),
                                     t["viewmat"], intr)
    _, depths = G.get_aabb_2d.project_points(t["means"].detach(), t["viewmat"], intr)
    nt = G.get_aabb_2d.get_num_tiles_hit_2d(c, e, cam.height, cam.width, 16)
    bgt = torch.tensor(bg, dtype=torch.float32, device=DEV)
    outs = G.texture_gaussians((spec.num_points, 1, spec.texture.shape[1]), t["dims"], c, e, depths.contiguous(),
                               nt, t["colors"], t["opacity"], t["means"], t["scales"], 1.0, t["quats"], t["uv0"],
                               t["umap"], t["vmap"], t["texture"], t["viewmat"], t["c2w"], *intr, cam.height,
                               cam.width, 16, 1 << 8, bgt)
    return case, outs, nt


def test_nothing_on_screen_renders_the_background():
    """Every splat behind the camera: no intersections; the image is the
    background, alpha 0, and all gradients are zero (the reference leaves
    its outputs undefined here, texture.py:197-205)."""
    spec = small_scene(n=50, width=48, height=32, seed=3)
    spec.means[:, 2] = -3.0
    case, outs, nt = _render(spec)
    img, depth, reg, alpha, tex, normal = outs
    np.testing.assert_allclose(np_(img), np.broadcast_to([0.25, 0.5, 0.75], img.shape), atol=1e-7)
    assert float(alpha.detach().abs().max()) == 0.0 and float(tex.detach().abs().max()) == 0.0
    (img.sum() + tex.sum() + normal.sum() + reg.sum() + depth.sum()).backward()
    for k in ("means", "opacity", "texture", "quats"):
        assert float(case.t[k].grad.abs().max()) == 0.0, k


def test_screen_covering_splats_vs_oracle():
    """Splats much larger than the image, close to the camera: every tile
    holds them; forward and backward against the fp64 oracle."""
    spec = small_scene(n=40, width=64, height=48, seed=9, scale=(0.5, 2.0), z=(1.0, 2.0))
    case = Case(spec)
    b = case.binning_cuda(16)
    assert int(b["counts"].max()) == (64 // 16) * (48 // 16)
    bg = np.array([0.1, 0.1, 0.1])
    ref = oracle.texture_forward(case.scene_np, case.cam_np, b["gaussian_ids_sorted"].cpu().numpy(),
                                 b["tile_bins"].cpu().numpy(), 16, 1 << 8, bg, prec="f64")
    out, bgt = case.forward_cuda(b["gaussian_ids_sorted"], b["tile_bins"], 16, 1 << 8, bg)
    for k in ("img", "texture", "normal", "final_T"):
        err = np.abs(np_(out[k]) - ref[k])
        assert (err > 1e-4).mean() <= 1e-3 and err.max() < 1e-2, (k, float(err.max()))
    ups = upstream(case.cam.height, case.cam.width, spec.texture.shape[1])
    gref = oracle.texture_backward(case.scene_np, case.cam_np, b["gaussian_ids_sorted"].cpu().numpy(),
                                   b["tile_bins"].cpu().numpy(), 16, 1 << 8, bg, ref, ups["img"], ups["depth"],
                                   ups["reg"], ups["alpha"], ups["texture"], ups["normal"], prec="f64")
    g = case.backward_cuda(out, b["gaussian_ids_sorted"], b["tile_bins"], ups, 16, 1 << 8, bgt)
    for k in ("colors", "opacity", "means", "scales", "quats", "uv0", "umap", "vmap", "texture"):
        r = gref[k].reshape(-1)
        err = np.abs(np_(g[k]).reshape(-1) - r).max() / (np.abs(r).max() + 1e-12)
        assert err < 1e-3, (k, err)


def _batch(cams, spec, capacity):
    from gstex_cuda_gb300 import batch as B
    scene = B.Scene(means=spec.means.to(DEV), scales=spec.scales.to(DEV), quats=spec.quats.to(DEV),
                    opacity=spec.opacity.to(DEV), sh_coeffs=spec.sh_coeffs.to(DEV), sh_degree=spec.sh_degree,
                    uv0=spec.uv0.to(DEV), umap=spec.umap.to(DEV), vmap=spec.vmap.to(DEV),
                    texture_dims=spec.texture_dims.to(DEV), texture=spec.texture.to(DEV))
    bcams = [B.Camera(c.viewmat, c.fx, c.fy, c.cx, c.cy, c.width, c.height) for c in cams]
    return B.BatchRenderer(bcams, spec.num_points, capacity=capacity, background=(0.3, 0.2, 0.1)), scene


def test_batch_overflow_is_detected_and_grown():
    """An intersection buffer that is too small is reported by
    check_capacity (no write past it), and after grow() the step equals one
    rendered with ample capacity."""
    from gstex_cuda_gb300 import synthetic
    g = torch.Generator().manual_seed(4)
    cams = synthetic.sphere_cameras(g, 3, radius=8.0, resolutions=[(96, 64), (64, 64), (80, 48)])
    spec = synthetic._finish_with_area(g, torch.empty(2000, 3).uniform_(-3, 3, generator=g), 0.01, 0.1, 3, "normal",
                                       cams, 20_000, "multi", {})
    big, scene = _batch(cams, spec, 1 << 20)
    gen = torch.Generator().manual_seed(1)
    tgt_img = torch.rand(big.total_pixels, 3, generator=gen).to(DEV)
    tgt_tex = torch.rand(big.total_pixels, 3, generator=gen).to(DEV)
    l_big = float(big.step(scene, tgt_img, tgt_tex).item())
    assert big.check_capacity()
    n = big.intersections()
    small, _ = _batch(cams, spec, max(1, n // 3))
    small.step(scene, tgt_img, tgt_tex)
    assert not small.check_capacity()
    small.grow(1.25)
    l_small = float(small.step(scene, tgt_img, tgt_tex).item())
    assert small.check_capacity() and small.intersections() == n
    assert abs(l_small - l_big) <= 1e-6 * abs(l_big)
    for k in ("img", "texture", "final_T"):
        np.testing.assert_allclose(small.out[k].cpu().numpy(), big.out[k].cpu().numpy(), atol=1e-6, err_msg=k)


def test_batch_view_without_intersections():
    """A camera that sees nothing renders its background and contributes
    nothing to the gradients; the other views are unaffected."""
    from gstex_cuda_gb300 import synthetic
    g = torch.Generator().manual_seed(6)
    cams = synthetic.sphere_cameras(g, 2, radius=8.0, resolutions=[(64, 64), (64, 48)])
    # camera z = world z - 50: every mean (|z| <= 3) lies behind this camera
    away = synthetic.make_camera(torch.tensor([[1.0, 0, 0, 0], [0, 1.0, 0, 0], [0, 0, 1.0, -50.0],
                                               [0, 0, 0, 1.0]]), 64, 48)
    spec = synthetic._finish_with_area(g, torch.empty(1500, 3).uniform_(-3, 3, generator=g), 0.01, 0.1, 3, "normal",
                                       cams, 15_000, "multi", {})
    both, scene = _batch(cams + [away], spec, 1 << 20)
    two, _ = _batch(cams, spec, 1 << 20)
    for r in (both, two):
        r.bin(scene)
        r.forward(scene)
    torch.cuda.synchronize()
    img = both.view_output("img", 2).cpu().numpy()
    np.testing.assert_allclose(img, np.broadcast_to([0.3, 0.2, 0.1], img.shape), atol=1e-7)
    for v in range(2):
        np.testing.assert_allclose(both.view_output("img", v).cpu().numpy(), two.view_output("img", v).cpu().numpy(),
                                   atol=1e-6)


def test_empty_scene_batch():
    """Zero Gaussians: the batched step renders backgrounds and returns."""
    from gstex_cuda_gb300 import synthetic
    g = torch.Generator().manual_seed(8)
    cams = synthetic.sphere_cameras(g, 2, radius=8.0, resolutions=[(32, 32), (48, 32)])
    spec = synthetic._finish_with_area(g, torch.empty(1, 3).uniform_(-3, 3, generator=g), 0.01, 0.1, 3, "normal",
                                       cams, 100, "multi", {})
    from gstex_cuda_gb300 import batch as B
    z = lambda *s: torch.zeros(*s, device=DEV)  # noqa: E731
    scene = B.Scene(means=z(0, 3), scales=z(0, 3), quats=z(0, 4), opacity=z(0, 1), sh_coeffs=z(0, 16, 3),
                    sh_degree=3, uv0=z(0, 1, 2), umap=z(0, 1, 3), vmap=z(0, 1, 3),
                    texture_dims=torch.zeros(0, 3, dtype=torch.int32, device=DEV), texture=z(0, 3))
    bcams = [B.Camera(c.viewmat, c.fx, c.fy, c.cx, c.cy, c.width, c.height) for c in cams]
    r = B.BatchRenderer(bcams, 0, capacity=16, background=(0.5, 0.5, 0.5))
    P = r.total_pixels
    loss = r.step(scene, torch.zeros(P, 3, device=DEV), torch.zeros(P, 3, device=DEV))
    torch.cuda.synchronize()
    assert np.isfinite(float(loss.item()))
    np.testing.assert_allclose(r.out["img"].cpu().numpy(), 0.5, atol=1e-7)
