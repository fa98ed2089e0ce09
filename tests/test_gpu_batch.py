"""Batched multi-view path (one launch per stage over all views) against the
CPU oracle run view by view."""
import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


@pytest.fixture(scope="module", params=[(1, 1, 32, 16), (2, 2, 32, 16), (1, 1, 16, 16), (1, 1, 8, 16),
                                        (1, 1, 4, 16), (1, 1, 8, 8), (2, 2, 32, 8)],
                ids=["1px", "2px", "1px_g16", "1px_g8", "1px_g4", "bw8_1px_g8", "bw8_2px"])
def setup(request):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from gstex_cuda_gb300 import batch as B, synthetic
    g = torch.Generator().manual_seed(9)
    cams = synthetic.sphere_cameras(g, 4, radius=8.0, resolutions=[(96, 64), (80, 80), (128, 72), (64, 96)])
    spec = synthetic._finish_with_area(g, torch.empty(3000, 3).uniform_(-3, 3, generator=g), 0.01, 0.1, 3, "normal",
                                       cams, 40_000, "multi", {})
    scene = B.Scene(means=spec.means.to(DEV), scales=spec.scales.to(DEV), quats=spec.quats.to(DEV),
                    opacity=spec.opacity.to(DEV), sh_coeffs=spec.sh_coeffs.to(DEV), sh_degree=3,
                    uv0=spec.uv0.to(DEV), umap=spec.umap.to(DEV), vmap=spec.vmap.to(DEV),
                    texture_dims=spec.texture_dims.to(DEV), texture=spec.texture.to(DEV))
    bcams = [B.Camera(c.viewmat, c.fx, c.fy, c.cx, c.cy, c.width, c.height) for c in cams]
    r = B.BatchRenderer(bcams, spec.num_points, capacity=1 << 20, fwd_ppt=request.param[0],
                        bwd_ppt=request.param[1], bwd_group=request.param[2], block_width=request.param[3])
    P = r.total_pixels
    gen = torch.Generator().manual_seed(1)
    tgt_img = torch.rand(P, 3, generator=gen).to(DEV)
    tgt_tex = torch.rand(P, 3, generator=gen).to(DEV)
    loss = r.step(scene, tgt_img, tgt_tex)
    torch.cuda.synchronize()
    return spec, cams, r, scene, loss


def _scene_np(spec, colors):
    return oracle.Scene(means=spec.means.numpy(), scales=spec.scales.numpy(), quats=spec.quats.numpy(),
                        opacity=spec.opacity.numpy(), colors=colors, uv0=spec.uv0.numpy(), umap=spec.umap.numpy(),
                        vmap=spec.vmap.numpy(), texture_dims=spec.texture_dims.numpy(), texture=spec.texture.numpy())


def test_batch_binning_bit_exact_per_view(setup):
    spec, cams, r, scene, _ = setup
    bw = r.bw
    assert r.check_capacity()
    ks = r.keys_sorted.cpu().numpy()
    gs = r.gids_sorted.cpu().numpy()
    n = int(r.count.item())
    counts = r.counts.cpu().numpy().reshape(r.V, r.N)
    off = 0
    for v, cam in enumerate(cams):
        c, e = oracle.get_aabb_2d(spec.means.numpy(), spec.scales.numpy(), 1.0, spec.quats.numpy(),
                                  cam.viewmat.numpy(), cam.fx, cam.fy, cam.cx, cam.cy)
        nt = oracle.num_tiles_hit(c, e, cam.height, cam.width, bw)
        np.testing.assert_array_equal(counts[v], nt)
        d = oracle.camera_depths(spec.means.numpy(), cam.viewmat.numpy())
        b = oracle.bin_and_sort(c, e, d, nt, cam.height, cam.width, bw)
        m = b["n_isect"]
        toff = int(sum(((cc.width + bw - 1) // bw) * ((cc.height + bw - 1) // bw) for cc in cams[:v]))
        # keys are (global tile << 1 | real): the tile of every slot and the
        # Gaussian order within each tile equal the reference's 64-bit sort
        np.testing.assert_array_equal((ks[off:off + m].astype(np.int64) >> 1) - toff,
                                      b["isect_ids_sorted"] >> 32)
        np.testing.assert_array_equal(gs[off:off + m], b["gaussian_ids_sorted"])
        off += m
    assert off == n


def test_batch_binning_with_clipped_gaussians():
    """A camera inside the cloud: Gaussians behind it whose mean projects into
    the image get one tile and emit nothing, so their slots keep the
    reference's zero entry (tile 0, Gaussian 0) and sort first in the view's
    tile 0.  Tiles and Gaussian order of every view equal the oracle's."""
    from gstex_cuda_gb300 import batch as B, synthetic
    g = torch.Generator().manual_seed(17)
    inside = synthetic.make_camera(torch.eye(4), 64, 48)
    cams = synthetic.sphere_cameras(g, 2, radius=8.0, resolutions=[(64, 64), (80, 48)]) + [inside]
    spec = synthetic._finish_with_area(g, torch.empty(1500, 3).uniform_(-3, 3, generator=g), 0.01, 0.1, 3, "normal",
                                       cams, 15_000, "multi", {})
    scene = B.Scene(means=spec.means.to(DEV), scales=spec.scales.to(DEV), quats=spec.quats.to(DEV),
                    opacity=spec.opacity.to(DEV), sh_coeffs=spec.sh_coeffs.to(DEV), sh_degree=3,
                    uv0=spec.uv0.to(DEV), umap=spec.umap.to(DEV), vmap=spec.vmap.to(DEV),
                    texture_dims=spec.texture_dims.to(DEV), texture=spec.texture.to(DEV))
    bcams = [B.Camera(c.viewmat, c.fx, c.fy, c.cx, c.cy, c.width, c.height) for c in cams]
    r = B.BatchRenderer(bcams, spec.num_points, capacity=1 << 20)
    r.bin(scene)
    torch.cuda.synchronize()
    ks = r.keys_sorted.cpu().numpy().astype(np.int64)
    gs = r.gids_sorted.cpu().numpy()
    n = int(r.count.item())
    off = toff = 0
    phantoms = 0
    for v, cam in enumerate(cams):
        c, e = oracle.get_aabb_2d(spec.means.numpy(), spec.scales.numpy(), 1.0, spec.quats.numpy(),
                                  cam.viewmat.numpy(), cam.fx, cam.fy, cam.cx, cam.cy)
        nt = oracle.num_tiles_hit(c, e, cam.height, cam.width, 16)
        d = oracle.camera_depths(spec.means.numpy(), cam.viewmat.numpy())
        b = oracle.bin_and_sort(c, e, d, nt, cam.height, cam.width, 16)
        m = b["n_isect"]
        phantoms += int(((nt > 0) & (e.max(-1) <= 1e-4)).sum())
        np.testing.assert_array_equal((ks[off:off + m] >> 1) - toff, b["isect_ids_sorted"] >> 32)
        np.testing.assert_array_equal(gs[off:off + m], b["gaussian_ids_sorted"])
        ob = b["tile_bins"].reshape(-1, 2)
        want = np.where((ob[:, 1] > ob[:, 0])[:, None], ob + off, 0)  # empty tiles stay (0, 0)
        np.testing.assert_array_equal(r.bins.cpu().numpy()[toff:toff + len(ob)], want)
        off += m
        toff += ((cam.width + 15) // 16) * ((cam.height + 15) // 16)
    assert off == n and phantoms > 0


def test_depth_first_binning_equals_64bit_binning(setup):
    """The depth-first binning (32-bit sorts) and the 64-bit
    (global tile << 32 | depth) emission + sort give the same
    gaussian_ids_sorted and tile_bins, bit for bit."""
    from gstex_cuda_gb300 import batch as B
    from gstex_cuda_gb300._lib import check, ptr
    spec, cams, r, scene, _ = setup
    r.bin(scene)
    L = B._L()
    st = torch.cuda.current_stream().cuda_stream
    VN, cap = r.V * r.N, r.capacity
    i32 = dict(dtype=torch.int32, device=DEV)
    i64 = dict(dtype=torch.int64, device=DEV)
    cum = torch.empty(VN, **i32)
    total = torch.zeros(1, **i64)
    count = torch.zeros(1, **i64)
    overflow = torch.zeros(1, **i32)
    ws = torch.empty(L.gstex_scan_workspace_bytes(VN), dtype=torch.uint8, device=DEV)
    keys = torch.empty(cap, **i64)
    vals = torch.empty(cap, **i32)
    ks = torch.empty(cap, **i64)
    gs = torch.empty(cap, **i32)
    sws = torch.empty(L.gstex_sort_workspace_bytes(cap), dtype=torch.uint8, device=DEV)
    bins = torch.empty_like(r.bins)
    check(L.gstex_inclusive_scan_i32(VN, ptr(r.counts), ptr(cum), ptr(total), ptr(ws), ws.numel(), st), "scan")
    check(L.gstex_batch_emit(r.N, r.V, ptr(r.views_dev), ptr(scene.means), ptr(scene.scales), 1.0,
                             ptr(scene.quats), r.bw, ptr(cum), ptr(total), cap, ptr(keys), ptr(vals), ptr(count),
                             ptr(overflow), st), "emit")
    check(L.gstex_sort_pairs_dyn(cap, ptr(count), 32 + int(r.total_tiles).bit_length(), ptr(keys), ptr(vals),
                                 ptr(ks), ptr(gs), ptr(sws), sws.numel(), st), "sort")
    check(L.gstex_get_tile_bin_edges_dyn(cap, ptr(count), ptr(ks), r.total_tiles, ptr(bins), st), "edges")
    torch.cuda.synchronize()
    n = int(count.item())
    assert n == int(r.count.item())
    assert torch.equal(gs[:n], r.gids_sorted[:n])
    assert torch.equal(bins, r.bins)
    assert torch.equal(ks[:n] >> 32, (r.keys_sorted[:n].to(torch.int64) >> 1))


def test_batch_forward_backward_vs_oracle(setup):
    spec, cams, r, scene, loss = setup
    bw = r.bw
    gs = r.gids_sorted.cpu().numpy()
    bins = r.bins.cpu().numpy()
    vcol = r.grads["vcolors"][..., :3].cpu().numpy()
    ups = {k: v.cpu().numpy() for k, v in r.ups.items()}
    tot = None
    vcoef = 0
    toff = 0
    for v, cam in enumerate(cams):
        dirs = (spec.means - cam.position[None]).numpy()
        col = oracle.sh_forward(3, 3, dirs, spec.sh_coeffs.numpy(), prec="f64")
        np.testing.assert_allclose(r.colors[v].cpu().numpy(), col, atol=2e-5, rtol=1e-5)
        sc = _scene_np(spec, r.colors[v].cpu().numpy())
        oc = oracle.Camera(cam.viewmat.numpy(), cam.c2w.numpy(), cam.fx, cam.fy, cam.cx, cam.cy, cam.height,
                           cam.width)
        nt = ((cam.width + bw - 1) // bw) * ((cam.height + bw - 1) // bw)
        vb = bins[toff:toff + nt]
        toff += nt
        ref = oracle.texture_forward(sc, oc, gs, vb, bw, 1 << 8, np.zeros(3), prec="f64")
        for k in ("img", "texture", "normal", "final_T"):
            got = r.view_output(k, v).cpu().numpy()
            err = np.abs(got - ref[k].reshape(got.shape))
            # all but threshold-flip pixels within 1e-4; flips stay below 1e-2
            assert (err > 1e-4).mean() <= 1e-3 and err.max() < 1e-2, (k, v, float(err.max()))
        a, b = r.pix_offsets_host[v], r.pix_offsets_host[v + 1]
        H, W = cam.height, cam.width
        up = dict(img=ups["img"][a:b].reshape(H, W, 3), texture=ups["texture"][a:b].reshape(H, W, 3),
                  normal=ups["normal"][a:b].reshape(H, W, 3), reg=ups["reg"][a:b].reshape(H, W))
        g = oracle.texture_backward(sc, oc, gs, vb, bw, 1 << 8, np.zeros(3), ref, up["img"], np.zeros((H, W)),
                                    up["reg"], np.zeros((H, W)), up["texture"], up["normal"], prec="f64")
        err = np.abs(vcol[v] - g["colors"]).max() / (np.abs(g["colors"]).max() + 1e-12)
        assert err < 5e-4, ("vcolors", v, err)
        vcoef = vcoef + oracle.sh_backward(3, 3, dirs, g["colors"], prec="f64")
        tot = g if tot is None else {k: tot[k] + g[k] for k in tot}
    G = r.grads
    for k in ("opacity", "means", "scales", "quats", "uv0", "umap", "vmap", "texture"):
        got = G[k].cpu().numpy().reshape(-1)
        ref = tot[k].reshape(-1)
        err = np.abs(got - ref).max() / (np.abs(ref).max() + 1e-12)
        assert err < 5e-4, (k, err)
    err = np.abs(G["sh_coeffs"].cpu().numpy() - vcoef).max() / (np.abs(vcoef).max() + 1e-12)
    assert err < 5e-4, ("sh", err)


@pytest.mark.parametrize("settings", [(1 << 8) | (1 << 9), (1 << 8) | (1 << 10), (1 << 8) | (1 << 2), 0],
                         ids=["blur", "ndc", "nearest", "no_uv_grad"])
@pytest.mark.parametrize("bw,tex", [(16, "f32"), (8, "f32"), (8, "bf16")])
def test_batch_settings_variants_vs_oracle(settings, bw, tex):
    """Settings other than the default (blur, NDC depth, nearest texels, uv
    gradients not propagated) take the general compositor kernels instead of
    the ones compiled for the default settings (with bf16 texels and 8x8
    tiles, the 10-CTA backward compiled for run-time settings): the batched
    step still matches the fp64 oracle per view."""
    from gstex_cuda_gb300 import batch as B, synthetic
    g = torch.Generator().manual_seed(31)
    cams = synthetic.sphere_cameras(g, 2, radius=8.0, resolutions=[(96, 64), (80, 80)])
    spec = synthetic._finish_with_area(g, torch.empty(1500, 3).uniform_(-3, 3, generator=g), 0.01, 0.1, 3, "normal",
                                       cams, 20_000, "multi", {})
    texture, tex_np = spec.texture, spec.texture.numpy()
    if tex == "bf16":
        texture = torch.zeros(spec.texture.shape[0], 4, dtype=torch.bfloat16)
        texture[:, :3] = spec.texture.to(torch.bfloat16)
        tex_np = texture[:, :3].float().numpy()
    scene = B.Scene(means=spec.means.to(DEV), scales=spec.scales.to(DEV), quats=spec.quats.to(DEV),
                    opacity=spec.opacity.to(DEV), sh_coeffs=spec.sh_coeffs.to(DEV), sh_degree=3,
                    uv0=spec.uv0.to(DEV), umap=spec.umap.to(DEV), vmap=spec.vmap.to(DEV),
                    texture_dims=spec.texture_dims.to(DEV), texture=texture.to(DEV))
    bcams = [B.Camera(c.viewmat, c.fx, c.fy, c.cx, c.cy, c.width, c.height) for c in cams]
    r = B.BatchRenderer(bcams, spec.num_points, capacity=1 << 20, block_width=bw, settings=settings,
                        texture_dtype=torch.bfloat16 if tex == "bf16" else torch.float32,
                        bwd_ctas=10 if bw == 8 else 0)
    gen = torch.Generator().manual_seed(3)
    tgt_img = torch.rand(r.total_pixels, 3, generator=gen).to(DEV)
    tgt_tex = torch.rand(r.total_pixels, 3, generator=gen).to(DEV)
    r.step(scene, tgt_img, tgt_tex)
    torch.cuda.synchronize()
    gs = r.gids_sorted.cpu().numpy()
    bins = r.bins.cpu().numpy()
    ups = {k: v.cpu().numpy() for k, v in r.ups.items()}
    tot, toff = None, 0
    for v, cam in enumerate(cams):
        sc = _scene_np(spec, r.colors[v].cpu().numpy())
        sc = oracle.Scene(**{**sc.__dict__, "texture": tex_np})
        oc = oracle.Camera(cam.viewmat.numpy(), cam.c2w.numpy(), cam.fx, cam.fy, cam.cx, cam.cy, cam.height,
                           cam.width)
        nt = ((cam.width + bw - 1) // bw) * ((cam.height + bw - 1) // bw)
        vb = bins[toff:toff + nt]
        toff += nt
        ref = oracle.texture_forward(sc, oc, gs, vb, bw, settings, np.zeros(3), prec="f64")
        # (depth is the camera depth of the splat where T crosses 0.5: a pixel
        # whose T lands within rounding of 0.5 takes the neighbouring splat's)
        for k in ("img", "texture", "normal", "final_T"):
            got = r.view_output(k, v).cpu().numpy()
            err = np.abs(got - ref[k].reshape(got.shape))
            assert (err > 1e-4).mean() <= 1e-3 and err.max() < 1e-2, (k, v, float(err.max()))
        a, b = r.pix_offsets_host[v], r.pix_offsets_host[v + 1]
        H, W = cam.height, cam.width
        up = dict(img=ups["img"][a:b].reshape(H, W, 3), texture=ups["texture"][a:b].reshape(H, W, 3),
                  normal=ups["normal"][a:b].reshape(H, W, 3), reg=ups["reg"][a:b].reshape(H, W))
        gr = oracle.texture_backward(sc, oc, gs, vb, bw, settings, np.zeros(3), ref, up["img"], np.zeros((H, W)),
                                     up["reg"], np.zeros((H, W)), up["texture"], up["normal"], prec="f64")
        tot = gr if tot is None else {k: tot[k] + gr[k] for k in tot}
    G = r.grads
    for k in ("opacity", "means", "scales", "quats", "uv0", "umap", "vmap", "texture"):
        got = G[k].cpu().numpy()
        ref = tot[k]
        if k == "texture":  # bf16 texels: gradients [T, 4], the fourth column unused
            got = got[:, :ref.shape[1]]
        got, ref = got.reshape(-1), ref.reshape(-1)
        err = np.abs(got - ref).max() / (np.abs(ref).max() + 1e-12)
        # 1e-3 of the largest entry (5e-4 at the default settings): the blur
        # terms add an exp and a second alpha branch per pair
        assert err < 1e-3, (k, err)


def test_batch_loss_value(setup):
    spec, cams, r, scene, loss = setup
    o = r.out
    ref = 0.0
    tgt = None
    for v in range(r.V):
        a, b = r.pix_offsets_host[v], r.pix_offsets_host[v + 1]
        img = o["img"][a:b].double()
        n = o["normal"][a:b].double()
        ref += float(o["reg"][a:b].double().mean()) * 100.0
        ref += 0.05 * float((n[:, 0] ** 2 + n[:, 1] ** 2 + (1 - n[:, 2]) ** 2).mean())
    assert np.isfinite(float(loss.item()))
    assert float(loss.item()) >= ref * 0.999  # the MSE terms are non-negative


def test_plain_per_view_step_matches_batched_step(setup):
    """The per-view path a reference caller takes (texture_forward /
    texture_backward per camera, SH per camera, host-synchronised binning)
    gives the batched step's loss and gradients."""
    from gstex_cuda_gb300 import batch as B
    spec, cams, r, scene, _ = setup
    bcams = [B.Camera(c.viewmat, c.fx, c.fy, c.cx, c.cy, c.width, c.height) for c in cams]
    gen = torch.Generator().manual_seed(1)
    tgt_img = torch.rand(r.total_pixels, 3, generator=gen).to(DEV)
    tgt_tex = torch.rand(r.total_pixels, 3, generator=gen).to(DEV)
    l_batch = float(r.step(scene, tgt_img, tgt_tex).item())
    g_batch = {k: v.clone() for k, v in r.grads.items()}
    l_plain, g_plain = B.plain_step(scene, bcams, tgt_img, tgt_tex, r.pix_offsets_host, block_width=r.bw)
    assert abs(float(l_plain.item()) - l_batch) <= 1e-5 * abs(l_batch)
    for k in ("opacity", "means", "scales", "quats", "uv0", "umap", "vmap", "texture", "sh_coeffs"):
        a = g_plain[k].reshape(-1).cpu().numpy()
        b = g_batch[k].reshape(-1).cpu().numpy()
        if k == "texture" and a.size != b.size:
            b = g_batch[k][:, :a.size // g_batch[k].shape[0]].reshape(-1).cpu().numpy()
        assert np.abs(a - b).max() <= 1e-3 * (np.abs(b).max() + 1e-12), k


def test_forward_tile_order_does_not_change_outputs(setup):
    """The forward's heaviest-first queue order (groups of 4 x 4 tiles)
    changes which CTA renders a tile, not what it renders: outputs are
    bit-identical to tile order."""
    from gstex_cuda_gb300 import batch as B
    spec, cams, r, scene, _ = setup
    bcams = [B.Camera(c.viewmat, c.fx, c.fy, c.cx, c.cy, c.width, c.height) for c in cams]
    r2 = B.BatchRenderer(bcams, spec.num_points, capacity=1 << 20, block_width=r.bw, fwd_ppt=r.fwd_ppt,
                         bwd_ppt=r.bwd_ppt,
                         bwd_group=r.bwd_group, heavy_first=False)
    assert r.tile_order is not None and r2.tile_order is None
    for x in (r, r2):
        x.bin(scene)
        x.forward(scene)
    torch.cuda.synchronize()
    order = r.tile_order.cpu().numpy()
    cost = (r.bins[:, 1] - r.bins[:, 0]).cpu().numpy()
    assert np.array_equal(np.sort(order), np.arange(r.total_tiles))
    # groups of G x G tiles of a view: heaviest group first, a group's tiles
    # back to back in tile order
    G, bw = r.order_group, r.bw
    group = np.empty(r.total_tiles, np.int64)
    off = 0
    for cam in cams:
        tx, ty = (cam.width + bw - 1) // bw, (cam.height + bw - 1) // bw
        local = np.arange(tx * ty)
        group[off:off + tx * ty] = off + (local // tx // G * G) * tx + (local % tx // G * G)
        off += tx * ty
    gcost = np.bincount(group, weights=cost, minlength=r.total_tiles)
    seq = group[order]
    starts = np.flatnonzero(np.r_[True, seq[1:] != seq[:-1]])
    assert len(starts) == len(np.unique(group)), "a group's tiles are contiguous in the order"
    assert np.all(np.diff(gcost[seq[starts]]) <= 0)
    for a, b in zip(starts, np.r_[starts[1:], len(order)]):
        assert np.all(np.diff(order[a:b]) > 0)
    # groups of one tile: tiles by decreasing cost, ties in tile order
    r3 = B.BatchRenderer(bcams, spec.num_points, capacity=1 << 20, block_width=r.bw, fwd_ppt=r.fwd_ppt,
                         bwd_ppt=r.bwd_ppt, bwd_group=r.bwd_group, order_group=1)
    r3.bin(scene)
    r3.forward(scene)
    torch.cuda.synchronize()
    o3 = r3.tile_order.cpu().numpy()
    assert np.array_equal(np.sort(o3), np.arange(r.total_tiles)) and np.all(np.diff(cost[o3]) <= 0)
    ties = np.diff(cost[o3]) == 0
    assert np.all(np.diff(o3)[ties] > 0)
    for k in ("img", "depth", "reg", "texture", "normal", "final_T", "final_idx", "depth_idx", "reg_s"):
        assert np.array_equal(r.out[k].cpu().numpy(), r2.out[k].cpu().numpy()), k
        assert np.array_equal(r3.out[k].cpu().numpy(), r2.out[k].cpu().numpy()), k


@pytest.mark.parametrize("fwd_batch,bwd_batch", [(64, 128), (128, 64), (32, 32)])
def test_gaussians_per_batch_does_not_change_results(setup, fwd_batch, bwd_batch):
    """Staging fewer Gaussians per round than threads per CTA changes when a
    tile checks for early exit and flushes its moments, not what it
    composites: forward outputs are bit-identical, gradients equal up to the
    order of the global atomics."""
    from gstex_cuda_gb300 import batch as B
    spec, cams, r, scene, _ = setup
    bcams = [B.Camera(c.viewmat, c.fx, c.fy, c.cx, c.cy, c.width, c.height) for c in cams]
    r2 = B.BatchRenderer(bcams, spec.num_points, capacity=1 << 20, block_width=r.bw, fwd_ppt=r.fwd_ppt,
                         bwd_ppt=r.bwd_ppt,
                         bwd_group=r.bwd_group, fwd_batch=fwd_batch, bwd_batch=bwd_batch)
    gen = torch.Generator().manual_seed(1)
    tgt_img = torch.rand(r.total_pixels, 3, generator=gen).to(DEV)
    tgt_tex = torch.rand(r.total_pixels, 3, generator=gen).to(DEV)
    r.step(scene, tgt_img, tgt_tex)
    g1 = {k: v.clone() for k, v in r.grads.items()}
    o1 = {k: v.clone() for k, v in r.out.items()}
    r2.step(scene, tgt_img, tgt_tex)
    torch.cuda.synchronize()
    for k in ("img", "depth", "reg", "texture", "normal", "final_T", "final_idx", "depth_idx", "reg_s"):
        assert np.array_equal(r2.out[k].cpu().numpy(), o1[k].cpu().numpy()), k
    for k in ("opacity", "means", "scales", "quats", "uv0", "umap", "vmap", "texture", "sh_coeffs"):
        a, b = r2.grads[k].cpu().numpy(), g1[k].cpu().numpy()
        assert np.abs(a - b).max() <= 1e-4 * (np.abs(b).max() + 1e-12), k


def test_host_input_stepper_matches_device_step(setup):
    """Steps fed from pinned host tensors through HostInputStepper (the next
    step's upload overlapping the current step) give the device step's loss
    and gradients; a changed host scene reaches the next step."""
    from gstex_cuda_gb300 import batch as B
    spec, cams, r, scene, _ = setup
    gen = torch.Generator().manual_seed(1)
    tgt_img = torch.rand(r.total_pixels, 3, generator=gen).to(DEV)
    tgt_tex = torch.rand(r.total_pixels, 3, generator=gen).to(DEV)
    names = ("means", "scales", "quats", "opacity", "sh_coeffs", "uv0", "umap", "vmap", "texture_dims", "texture")
    host = B.Scene(**{**scene.__dict__, **{k: getattr(scene, k).cpu().pin_memory() for k in names}})
    host2 = B.Scene(**{**host.__dict__, "opacity": (host.opacity * 0.5).pin_memory()})
    scene2 = B.Scene(**{**scene.__dict__, "opacity": scene.opacity * 0.5})
    l_ref = float(r.step(scene, tgt_img, tgt_tex).item())
    g_ref = {k: v.clone() for k, v in r.grads.items()}
    l_ref2 = float(r.step(scene2, tgt_img, tgt_tex).item())
    st = B.HostInputStepper(r, like=scene)
    st.upload(host)
    losses = []
    for nxt in (host, host2, None):
        losses.append(float(st.step(tgt_img, tgt_tex, next_host=nxt).item()))
        if len(losses) == 1:
            g1 = {k: v.clone() for k, v in r.grads.items()}
    torch.cuda.synchronize()
    assert abs(losses[0] - l_ref) <= 1e-5 * abs(l_ref) and abs(losses[1] - l_ref) <= 1e-5 * abs(l_ref)
    assert abs(losses[2] - l_ref2) <= 1e-5 * abs(l_ref2)
    for k, v in g_ref.items():
        torch.testing.assert_close(g1[k], v, atol=1e-5 * (float(v.abs().max()) + 1e-9), rtol=1e-4)


def test_autotune_grid_and_cache():
    """The autotuner times its grid and reports the chosen point; a second
    renderer of the same resolution mix, Gaussian count and settings takes
    the cached choice without timing."""
    from gstex_cuda_gb300 import batch as B, synthetic
    g = torch.Generator().manual_seed(37)
    cams = synthetic.sphere_cameras(g, 2, radius=8.0, resolutions=[(96, 64), (80, 80)])
    spec = synthetic._finish_with_area(g, torch.empty(1200, 3).uniform_(-3, 3, generator=g), 0.01, 0.1, 3, "normal",
                                       cams, 15_000, "multi", {})
    t16 = torch.zeros(spec.texture.shape[0], 4, dtype=torch.bfloat16)
    t16[:, :3] = spec.texture.to(torch.bfloat16)
    scene = B.Scene(means=spec.means.to(DEV), scales=spec.scales.to(DEV), quats=spec.quats.to(DEV),
                    opacity=spec.opacity.to(DEV), sh_coeffs=spec.sh_coeffs.to(DEV), sh_degree=3,
                    uv0=spec.uv0.to(DEV), umap=spec.umap.to(DEV), vmap=spec.vmap.to(DEV),
                    texture_dims=spec.texture_dims.to(DEV), texture=t16.to(DEV))
    bcams = [B.Camera(c.viewmat, c.fx, c.fy, c.cx, c.cy, c.width, c.height) for c in cams]
    gen = torch.Generator().manual_seed(3)
    P = sum(c.width * c.height for c in cams)
    tgt_img, tgt_tex = torch.rand(P, 3, generator=gen).to(DEV), torch.rand(P, 3, generator=gen).to(DEV)
    r = B.BatchRenderer(bcams, spec.num_points, texture_dtype=torch.bfloat16, capacity=1 << 20, block_width=8)
    B._tune_cache.pop(r.tune_key(), None)
    res = r.autotune(scene, tgt_img, tgt_tex)
    assert "cached" not in res and "backward_ppt1_g8_ms" in res and "backward_ppt1_g8_ctas10_ms" in res
    knobs = {k: getattr(r, k) for k in B.TUNED_KNOBS}
    r2 = B.BatchRenderer(bcams, spec.num_points, texture_dtype=torch.bfloat16, capacity=1 << 20, block_width=8)
    res2 = r2.autotune(scene, tgt_img, tgt_tex)
    assert res2.get("cached") is True and {k: getattr(r2, k) for k in B.TUNED_KNOBS} == knobs
    loss1 = float(r.step(scene, tgt_img, tgt_tex).item())
    loss2 = float(r2.step(scene, tgt_img, tgt_tex).item())
    assert abs(loss1 - loss2) <= 1e-5 * abs(loss1)
    B._tune_cache.pop(r.tune_key(), None)


def test_batch_graph_replay_matches_eager(setup):
    spec, cams, r, scene, _ = setup
    P = r.total_pixels
    gen = torch.Generator().manual_seed(1)
    tgt_img = torch.rand(P, 3, generator=gen).to(DEV)
    tgt_tex = torch.rand(P, 3, generator=gen).to(DEV)
    r.step(scene, tgt_img, tgt_tex)
    torch.cuda.synchronize()
    eager = {k: v.clone() for k, v in r.grads.items()}
    eager_img = r.out["img"].clone()
    r.capture(scene, tgt_img, tgt_tex)
    r.replay()
    torch.cuda.synchronize()
    torch.testing.assert_close(r.out["img"], eager_img, atol=1e-6, rtol=0)
    for k, v in eager.items():
        torch.testing.assert_close(r.grads[k], v, atol=1e-5 * (float(v.abs().max()) + 1e-9), rtol=1e-4)


def test_prebuilt_records_match_per_tile_records(setup):
    """Records built once per (view, Gaussian) (the default) and records
    derived by every tile give the same step up to float rounding."""
    from gstex_cuda_gb300 import batch as B
    spec, cams, r, scene, loss = setup
    bcams = [B.Camera(c.viewmat, c.fx, c.fy, c.cx, c.cy, c.width, c.height) for c in cams]
    r2 = B.BatchRenderer(bcams, spec.num_points, capacity=1 << 20, block_width=r.bw, fwd_ppt=r.fwd_ppt,
                         bwd_ppt=r.bwd_ppt,
                         bwd_group=r.bwd_group, prebuilt_records=False)
    gen = torch.Generator().manual_seed(1)
    tgt_img = torch.rand(r.total_pixels, 3, generator=gen).to(DEV)
    tgt_tex = torch.rand(r.total_pixels, 3, generator=gen).to(DEV)
    l1 = float(r.step(scene, tgt_img, tgt_tex).item())
    g1 = {k: v.clone() for k, v in r.grads.items()}
    o1 = {k: v.clone() for k, v in r.out.items()}
    l2 = float(r2.step(scene, tgt_img, tgt_tex).item())
    assert r.records is not None and r2.records is None
    assert abs(l1 - l2) <= 1e-5 * abs(l1)
    for k in ("img", "texture", "normal", "final_T"):
        np.testing.assert_allclose(r2.out[k].cpu().numpy(), o1[k].cpu().numpy(), atol=1e-5, err_msg=k)
    assert (r2.out["final_idx"] == o1["final_idx"]).float().mean() > 0.999
    for k in ("opacity", "means", "scales", "quats", "uv0", "umap", "vmap", "texture", "sh_coeffs"):
        a, b = r2.grads[k].cpu().numpy(), g1[k].cpu().numpy()
        assert np.abs(a - b).max() <= 1e-3 * (np.abs(b).max() + 1e-12), k


def _bf16_case():
    from gstex_cuda_gb300 import batch as B, synthetic
    g = torch.Generator().manual_seed(19)
    cams = synthetic.sphere_cameras(g, 3, radius=8.0, resolutions=[(96, 64), (80, 80), (128, 72)])
    spec = synthetic._finish_with_area(g, torch.empty(2500, 3).uniform_(-3, 3, generator=g), 0.01, 0.1, 3, "normal",
                                       cams, 30_000, "multi", {})
    t16 = torch.zeros(spec.texture.shape[0], 4, dtype=torch.bfloat16)
    t16[:, :3] = spec.texture.to(torch.bfloat16)
    sh16 = spec.sh_coeffs.to(torch.bfloat16)
    scene = B.Scene(means=spec.means.to(DEV), scales=spec.scales.to(DEV), quats=spec.quats.to(DEV),
                    opacity=spec.opacity.to(DEV), sh_coeffs=sh16.to(DEV), sh_degree=3, uv0=spec.uv0.to(DEV),
                    umap=spec.umap.to(DEV), vmap=spec.vmap.to(DEV), texture_dims=spec.texture_dims.to(DEV),
                    texture=t16.to(DEV))
    bcams = [B.Camera(c.viewmat, c.fx, c.fy, c.cx, c.cy, c.width, c.height) for c in cams]
    r = B.BatchRenderer(bcams, spec.num_points, texture_dtype=torch.bfloat16, capacity=1 << 20)
    gen = torch.Generator().manual_seed(2)
    tgt_img = torch.rand(r.total_pixels, 3, generator=gen).to(DEV)
    tgt_tex = torch.rand(r.total_pixels, 3, generator=gen).to(DEV)
    r.step(scene, tgt_img, tgt_tex)
    torch.cuda.synchronize()
    return spec, cams, r, t16[:, :3].double().numpy(), sh16.double().numpy()


def test_backward_occupancy_variants_match_general_kernel():
    """8x8 tiles, bf16 texels: the backward kernels compiled for 10 resident
    CTAs per SM (fewer registers; 8-lane groups, also with 48 Gaussians per
    batch, and the 32-lane walk) give the general kernel's gradients up to
    the order of the global atomics."""
    from gstex_cuda_gb300 import batch as B, synthetic
    g = torch.Generator().manual_seed(23)
    cams = synthetic.sphere_cameras(g, 3, radius=8.0, resolutions=[(96, 64), (80, 80), (128, 72)])
    spec = synthetic._finish_with_area(g, torch.empty(2500, 3).uniform_(-3, 3, generator=g), 0.01, 0.1, 3, "normal",
                                       cams, 30_000, "multi", {})
    t16 = torch.zeros(spec.texture.shape[0], 4, dtype=torch.bfloat16)
    t16[:, :3] = spec.texture.to(torch.bfloat16)
    scene = B.Scene(means=spec.means.to(DEV), scales=spec.scales.to(DEV), quats=spec.quats.to(DEV),
                    opacity=spec.opacity.to(DEV), sh_coeffs=spec.sh_coeffs.to(torch.bfloat16).to(DEV), sh_degree=3,
                    uv0=spec.uv0.to(DEV), umap=spec.umap.to(DEV), vmap=spec.vmap.to(DEV),
                    texture_dims=spec.texture_dims.to(DEV), texture=t16.to(DEV))
    bcams = [B.Camera(c.viewmat, c.fx, c.fy, c.cx, c.cy, c.width, c.height) for c in cams]
    gen = torch.Generator().manual_seed(2)
    P = sum(c.width * c.height for c in cams)
    tgt_img = torch.rand(P, 3, generator=gen).to(DEV)
    tgt_tex = torch.rand(P, 3, generator=gen).to(DEV)
    res = {}
    cases = ((0, 0, 8), (10, 0, 8), (10, 48, 8), (10, 0, 32))
    for case in cases:
        ctas, nb, gs = case
        r = B.BatchRenderer(bcams, spec.num_points, texture_dtype=torch.bfloat16, capacity=1 << 20, block_width=8,
                            bwd_group=gs, bwd_ctas=ctas, bwd_batch=nb)
        loss = float(r.step(scene, tgt_img, tgt_tex).item())
        torch.cuda.synchronize()
        res[case] = (loss, {k: v.cpu().numpy().copy() for k, v in r.grads.items()})
    base = res[cases[0]]
    for case in cases[1:]:
        assert abs(res[case][0] - base[0]) <= 1e-5 * abs(base[0])  # the loss sums by atomics
        for k in ("opacity", "means", "scales", "quats", "uv0", "umap", "vmap", "texture", "sh_coeffs"):
            a, b = res[case][1][k], base[1][k]
            assert np.abs(a - b).max() <= 1e-4 * (np.abs(b).max() + 1e-12), (case, k)


def _oracle_views(spec, cams, r, texture, sh):
    """Per-view fp64 oracle outputs and view-summed gradients for the given
    texel values and SH coefficients, on the renderer's binning."""
    gs, bins = r.gids_sorted.cpu().numpy(), r.bins.cpu().numpy()
    ups = {k: v.cpu().numpy() for k, v in r.ups.items()}
    outs, tot, toff = [], None, 0
    for v, cam in enumerate(cams):
        dirs = (spec.means - cam.position[None]).numpy()
        col = oracle.sh_forward(3, 3, dirs, sh, prec="f64")
        sc = _scene_np(spec, col)
        sc.texture = texture
        oc = oracle.Camera(cam.viewmat.numpy(), cam.c2w.numpy(), cam.fx, cam.fy, cam.cx, cam.cy, cam.height,
                           cam.width)
        nt = ((cam.width + 15) // 16) * ((cam.height + 15) // 16)
        vb = bins[toff:toff + nt]
        toff += nt
        ref = oracle.texture_forward(sc, oc, gs, vb, 16, 1 << 8, np.zeros(3), prec="f64")
        outs.append(ref)
        a, b = r.pix_offsets_host[v], r.pix_offsets_host[v + 1]
        H, W = cam.height, cam.width
        gg = oracle.texture_backward(sc, oc, gs, vb, 16, 1 << 8, np.zeros(3), ref,
                                     ups["img"][a:b].reshape(H, W, 3), np.zeros((H, W)),
                                     ups["reg"][a:b].reshape(H, W), np.zeros((H, W)),
                                     ups["texture"][a:b].reshape(H, W, 3), ups["normal"][a:b].reshape(H, W, 3),
                                     prec="f64")
        tot = gg if tot is None else {k: tot[k] + gg[k] for k in tot}
    return outs, tot


def _errors(r, outs, tot):
    img_err = []
    for v, ref in enumerate(outs):
        for k in ("img", "texture"):
            got = r.view_output(k, v).cpu().numpy()
            img_err.append(np.abs(got - ref[k].reshape(got.shape)).reshape(-1))
    img_err = np.concatenate(img_err)
    g_err = {}
    for k in ("opacity", "means", "scales", "quats", "uv0", "umap", "vmap", "texture"):
        got = r.grads[k].cpu().numpy()
        if k == "texture":
            got = got[:, :3]
        ref = tot[k].reshape(got.shape)
        rows = np.abs(got - ref).reshape(got.shape[0], -1).max(-1) / (np.abs(ref).max() + 1e-12)
        # (largest row error, fraction of rows above 1e-3, fraction above 1e-2)
        g_err[k] = (float(rows.max()), float((rows > 1e-3).mean()), float((rows > 1e-2).mean()))
    return img_err, g_err


def test_bf16_storage_accuracy_vs_fp64_oracle():
    """The headline storage: bf16 texels [T,4] and bf16 SH coefficients, all
    blending, transmittance and gradient accumulation in fp32.  (A) Against
    the fp64 oracle at the stored (bf16) parameter values: outputs within
    1e-4 and gradients within 1e-3 of the largest entry, threshold flips
    excepted: at most 0.5% of the gradient rows (one Gaussian or texel)
    beyond 1e-3 of the largest entry, none beyond 5e-2.  A pixel whose alpha
    flips at 1/255 changes its final distortion sums, and with the distortion
    weight of 100 that moves the geometry gradients of every splat at that
    pixel.  (B) Against the fp64 oracle at the unrounded fp32 values (what
    storing in bf16 changes): image and texture within 2e-3 abs, at most
    0.5% of the gradient rows beyond 1e-2, none beyond 1e-1."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    spec, cams, r, tex16, sh16 = _bf16_case()
    img_a, g_a = _errors(r, *_oracle_views(spec, cams, r, tex16, sh16))
    print("bf16 storage vs stored values: image/texture frac > 1e-4", float((img_a > 1e-4).mean()),
          "gradients (max row, frac > 1e-3)", g_a)
    assert (img_a > 1e-4).mean() <= 1e-3, float((img_a > 1e-4).mean())
    for k, (mx, fr, _) in g_a.items():
        assert fr <= 5e-3 and mx < 5e-2, ("stored values", k, mx, fr)
    img_b, g_b = _errors(r, *_oracle_views(spec, cams, r, spec.texture.double().numpy(),
                                           spec.sh_coeffs.double().numpy()))
    print("bf16 storage vs fp32 values: image/texture 99.9% quantile", float(np.quantile(img_b, 0.999)),
          "gradients", g_b)
    assert (img_b > 2e-3).mean() <= 1e-3, float((img_b > 2e-3).mean())
    for k, (mx, _, fr2) in g_b.items():
        assert fr2 <= 5e-3 and mx < 1e-1, ("fp32 values", k, mx, fr2)


def _raw_from(spec, seed=23):
    """Trainer-side raw parameters near the spec's scene: log-scales, quaternions
    of random norm, charts (uv0, log uv-scale, theta), opacity logits."""
    g = torch.Generator().manual_seed(seed)
    N = spec.num_points
    raw_scales = torch.log(spec.scales.clone())
    raw_scales[:, 2] = torch.randn(N, generator=g)  # not used (the third scale is tied)
    raw_quats = spec.quats * torch.empty(N, 1).uniform_(0.5, 2.0, generator=g)
    mapping = torch.zeros(N, 1, 4)
    mapping[:, 0, :2] = 0.5
    mapping[:, 0, 2] = torch.log(1.0 / (6.0 * spec.scales[:, :2].mean(-1)))
    mapping[:, 0, 3] = torch.empty(N).uniform_(-3.0, 3.0, generator=g)
    raw_opacity = torch.logit(spec.opacity.reshape(-1).clamp(1e-4, 1 - 1e-4))
    return raw_scales, raw_quats, mapping, raw_opacity


def test_raw_parameter_step_matches_preprocess_then_step(setup):
    """The training step from raw parameters (activation fused into the
    projection, its adjoint into the gradient finalize) against the two-kernel
    path: the standalone preprocess kernel, the step on the activated scene,
    and the preprocess adjoint on the activated gradients.  Same loss and raw
    gradients up to float rounding; the activated parameters it wrote equal
    the preprocess kernel's to a few ulp of the largest entry."""
    from gstex_cuda_gb300 import batch as B
    from gstex_cuda_gb300.preprocess import preprocess
    spec, cams, r, scene, _ = setup
    rs, rq, mp, ro = (x.to(DEV) for x in _raw_from(spec))
    raw = B.RawScene(means=scene.means, raw_scales=rs.contiguous(), raw_quats=rq.contiguous(),
                     mapping=mp.contiguous(), raw_opacity=ro.contiguous(), sh_coeffs=scene.sh_coeffs, sh_degree=3,
                     texture_dims=scene.texture_dims, texture=scene.texture)
    gen = torch.Generator().manual_seed(1)
    tgt_img = torch.rand(r.total_pixels, 3, generator=gen).to(DEV)
    tgt_tex = torch.rand(r.total_pixels, 3, generator=gen).to(DEV)
    l_raw = float(r.step_raw(raw, tgt_img, tgt_tex).item())
    g_raw = {k: v.clone() for k, v in r.raw_grads.items()}
    act = {k: getattr(r.activated(raw), k).clone() for k in ("scales", "quats", "uv0", "umap", "vmap", "opacity")}
    # two-kernel path
    leaves = [t.clone().requires_grad_(True) for t in (rs, rq, mp, ro)]
    sc, qu, u0, um, vm, op = preprocess(*leaves)
    for k, v in zip(("scales", "quats", "uv0", "umap", "vmap", "opacity"), (sc, qu, u0, um, vm, op)):
        ref = v.detach().reshape(act[k].shape)
        # fused and standalone kernels differ in multiply-add contraction only
        assert float((act[k] - ref).abs().max()) <= 2e-6 * float(ref.abs().max()), k
    s2 = B.Scene(means=scene.means, scales=sc.detach().contiguous(), quats=qu.detach().contiguous(),
                 opacity=op.detach().contiguous(), sh_coeffs=scene.sh_coeffs, sh_degree=3,
                 uv0=u0.detach().contiguous(), umap=um.detach().contiguous(), vmap=vm.detach().contiguous(),
                 texture_dims=scene.texture_dims, texture=scene.texture)
    l2 = float(r.step(s2, tgt_img, tgt_tex).item())
    g2 = r.grads
    torch.autograd.backward([sc, qu, u0, um, vm, op], [g2["scales"], g2["quats"], g2["uv0"], g2["umap"], g2["vmap"],
                                                       g2["opacity"]])
    assert abs(l_raw - l2) <= 1e-5 * abs(l2)
    refs = dict(raw_scales=leaves[0].grad, raw_quats=leaves[1].grad, mapping=leaves[2].grad,
                raw_opacity=leaves[3].grad, means=g2["means"], texture=g2["texture"], sh_coeffs=g2["sh_coeffs"])
    for k, ref in refs.items():
        got = g_raw[k].reshape(ref.shape)
        if k == "raw_scales":
            got, ref = got[:, :2], ref[:, :2]
        err = float((got - ref).abs().max() / (ref.abs().max() + 1e-12))
        assert err < 1e-3, (k, err)
