"""The headline batched path at its benchmarked size against the reference's
own kernels, view by view.

Scenes: the multi-view workload (32 cameras of 512^2 / 800^2 / 1280x720 /
1920x1080 on an r=8 sphere, 500k Gaussians, 16M bf16 texels, bf16 SH of
degree 3) and the stress workload (8 cameras at 1920x1080, 1M Gaussians in 64
clusters of sigma 0.3, 32M bf16 texels).  ``BatchRenderer.step`` renders all
views in one persistent launch per stage (depth-first 32-bit binning, global
tile queue, heaviest tiles first); the reference's kernels (cubins built from
its sources, oracle/refkern) render the same views one after another with the
bf16-rounded texels and SH coefficients widened to fp32, which are the values
the batched path computes with.

Compared per view: the tile counts, tile ranges and Gaussian order of every
tile bit for bit against the CPU oracle's restatement of the reference's
binning (its AABB, tile counter, emission and sort in IEEE fp32); the tile
counts against the reference's own AABB kernel, which is built with fast
math, so that a splat whose +-3 sigma box edge lies within rounding of a tile
boundary can get one tile more or less (at most 1e-4 of the Gaussians of a
view).  The reference's compositor kernels then run on the batched path's
binning of the view (so that a box flip does not move a splat between
tiles), and the nine forward outputs must agree within the per-view bars of
tests/test_gpu_refkern.py (1e-4, threshold flips excepted), as must the
per-view colour gradients.  The backward of both gets the same upstream
gradients (the batched path's image-loss gradients), and the per-Gaussian and
per-texel gradients summed over views are compared row by row.
"""
import numpy as np
import pytest
import torch

import oracle
from gpu_helpers import close_frac, np_
from test_gpu_refkern import _compare, _edge_on

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


@pytest.fixture(scope="module", autouse=True)
def _require():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import refkern
    if not refkern.available():
        pytest.skip("reference cubins absent (oracle/refkern/build_ref.py builds them where the reference is)")


def _tile_local(idx, bins, W, H, bw=16):
    """Position of each pixel's index inside its tile's [start, end) range of
    the sorted list, -1 where it lies outside (no contributor)."""
    tx = (W + bw - 1) // bw
    ii, jj = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    tile = (ii // bw) * tx + (jj // bw)
    start, end = bins[tile, 0], bins[tile, 1]
    idx = np.asarray(idx).reshape(H, W).astype(np.int64)
    return np.where((idx >= start) & (idx < end), idx - start, -1)


def _workload(which):
    from gstex_cuda_gb300 import synthetic
    if which == "multiview_32x_500k_16M":
        return synthetic.batched(seed=3, n=500_000, texels=16_000_000, views=32)
    return synthetic.stress(seed=4, n=1_000_000, texels=32_000_000, views=8)


# (scene, tile width, backward lanes per walk, backward CTAs per SM, Gaussians per batch):
# the reference's 16x16 tiles, and the configurations the autotuner picks
@pytest.mark.parametrize("which,bw,gs,ctas,nb", [("multiview_32x_500k_16M", 16, 8, 0, 0),
                                                ("multiview_32x_500k_16M", 8, 8, 10, 0),
                                                ("stress_8x1080p_1M_32M", 16, 8, 0, 0),
                                                ("stress_8x1080p_1M_32M", 8, 32, 10, 48)])
def test_batched_step_at_full_size_vs_reference_kernels(which, bw, gs, ctas, nb):
    """Tile widths 16 (the reference's) and 8 (the autotuner's choice on both
    scenes, with the backward variant it picks): the reference's kernels run
    with the same width."""
    from gstex_cuda_gb300 import batch as B
    from oracle import refkern as R
    spec = _workload(which)
    stress = which.startswith("stress")
    cams = spec.cameras
    # the stored values of the batched path: bf16 texels [T, 4] and bf16 SH
    t16 = torch.zeros(spec.texture.shape[0], 4, dtype=torch.bfloat16)
    t16[:, :3] = spec.texture.to(torch.bfloat16)
    sh16 = spec.sh_coeffs.to(torch.bfloat16)
    d = lambda x: x.contiguous().to(DEV)  # noqa: E731
    scene = B.Scene(means=d(spec.means), scales=d(spec.scales), quats=d(spec.quats), opacity=d(spec.opacity),
                    sh_coeffs=d(sh16), sh_degree=spec.sh_degree, uv0=d(spec.uv0), umap=d(spec.umap),
                    vmap=d(spec.vmap), texture_dims=d(spec.texture_dims), texture=d(t16))
    bcams = [B.Camera(c.viewmat, c.fx, c.fy, c.cx, c.cy, c.width, c.height) for c in cams]
    r = B.BatchRenderer(bcams, spec.num_points, texture_dtype=torch.bfloat16, device=DEV, block_width=bw,
                        bwd_group=gs, bwd_ctas=ctas, bwd_batch=nb)
    gen = torch.Generator().manual_seed(11)
    tgt_img = torch.rand(r.total_pixels, 3, generator=gen).to(DEV)
    tgt_tex = torch.rand(r.total_pixels, 3, generator=gen).to(DEV)
    r.step(scene, tgt_img, tgt_tex)
    torch.cuda.synchronize()
    while not r.check_capacity():  # the capacity grows like the benchmark's sizing step
        r.grow(1.25)
        r.step(scene, tgt_img, tgt_tex)
        torch.cuda.synchronize()
    assert r.intersections() > (30_000_000 if not stress else 25_000_000)

    t = dict(means=scene.means, scales=scene.scales, quats=scene.quats, opacity=scene.opacity, uv0=scene.uv0,
             umap=scene.umap, vmap=scene.vmap, dims=scene.texture_dims,
             texture=t16[:, :3].float().contiguous().to(DEV), sh=sh16.float().contiguous().to(DEV))
    gids_b = r.gids_sorted.cpu().numpy()
    bins_b = r.bins.cpu().numpy()
    counts_b = r.counts.cpu().numpy().reshape(r.V, r.N)
    count_flips = 0
    vcol_b = r.grads["vcolors"][..., :3]
    off = toff = 0
    tot = None
    edge = np.zeros(spec.num_points, bool)
    cap = (25 if stress else 10) * 2e-3
    for v, cam in enumerate(cams):
        # binning bit for bit against the oracle's restatement
        c, e = oracle.get_aabb_2d(spec.means.numpy(), spec.scales.numpy(), 1.0, spec.quats.numpy(),
                                  cam.viewmat.numpy(), cam.fx, cam.fy, cam.cx, cam.cy)
        cnt = oracle.num_tiles_hit(c, e, cam.height, cam.width, bw)
        np.testing.assert_array_equal(counts_b[v], cnt, err_msg=f"tile counts of view {v}")
        ob = oracle.bin_and_sort(c, e, oracle.camera_depths(spec.means.numpy(), cam.viewmat.numpy()), cnt,
                                 cam.height, cam.width, bw)
        n = ob["n_isect"]
        obins = ob["tile_bins"].reshape(-1, 2)
        nt = obins.shape[0]
        nonempty = (obins[:, 1] > obins[:, 0])[:, None]
        np.testing.assert_array_equal(bins_b[toff:toff + nt], np.where(nonempty, obins + off, 0),
                                      err_msg=f"tile ranges of view {v}")
        np.testing.assert_array_equal(gids_b[off:off + n], ob["gaussian_ids_sorted"],
                                      err_msg=f"Gaussian order of view {v}")
        # the reference's fast-math AABB kernel: tile counts equal but for
        # boxes within rounding of a tile boundary
        rc = np_(R.num_tiles_hit(*R.get_aabb_2d(t["means"], t["scales"], 1.0, t["quats"],
                                                cam.viewmat.contiguous().to(DEV), cam.fx, cam.fy, cam.cx, cam.cy),
                                 cam.height, cam.width, bw))
        flips = int((rc != cnt).sum())
        count_flips += flips
        assert flips <= max(2, 1e-4 * spec.num_points), (v, flips)
        # the reference's kernels on this view's binning (local ranges)
        local = np.ascontiguousarray(np.where(nonempty, obins, 0).astype(np.int32))
        vg = torch.from_numpy(np.ascontiguousarray(gids_b[off:off + n])).to(DEV)
        vb = torch.from_numpy(local).to(DEV)
        f = R.view_forward(t, cam, spec.sh_degree, block_width=bw, binning=(vg, vb))
        # SH colours of the view from the same (bf16-rounded) coefficients
        np.testing.assert_allclose(np_(r.colors[v]), np_(f["colors"]), atol=2e-6, rtol=2e-5)
        got = {k: r.view_output(k, v) for k in ("img", "depth", "reg", "texture", "normal", "final_T", "final_idx",
                                               "depth_idx", "reg_s")}
        # final_idx / depth_idx index a sorted list (ours: all views', the
        # reference's: the view's own): compare them as positions inside the
        # pixel's tile range
        refo = dict(f["out"])
        for k in ("final_idx", "depth_idx"):
            got[k] = _tile_local(np_(got[k]), bins_b[toff:toff + nt], cam.width, cam.height, bw)
            refo[k] = _tile_local(np_(refo[k]), local, cam.width, cam.height, bw)
        # the outlier cap is 5e-2 here (1e-2 in the single-view tests): over
        # 32 random viewpoints some splats are seen almost edge-on, which
        # this path solves in double and the reference in fast-math fp32, so
        # a pixel's alpha can move by more than one threshold flip
        # the stress scene's 64 dense clusters put more pairs near the
        # thresholds: up to 0.7% of a view's pixels flip (0.5% for one view in
        # the single-view stress test)
        _compare(refo, got, {}, {}, 1e-4, 7e-3 if stress else 3e-3, 2e-3, out_cap=5e-2)
        # backward with identical upstream gradients
        a, b = r.pix_offsets_host[v], r.pix_offsets_host[v + 1]
        H, W = cam.height, cam.width
        ups = {k: r.ups[k][a:b].reshape(H, W, *r.ups[k].shape[1:]) for k in ("img", "texture", "normal", "reg")}
        g = R.view_backward(t, cam, spec.sh_degree, f, ups, block_width=bw)
        cref = np_(g["colors"])
        crow = np.abs(np_(vcol_b[v]) - cref).max(-1) / (np.abs(cref).max() + 1e-12)
        assert (crow > 2e-3).mean() <= 1e-3 and crow.max() < cap, ("colors", v, float(crow.max()))
        edge |= _edge_on(spec, cam)
        cur = {k: g[k] for k in ("opacity", "means", "scales", "quats", "uv0", "umap", "vmap", "texture",
                                 "sh_coeffs")}
        tot = cur if tot is None else {k: tot[k] + cur[k] for k in tot}
        off += n
        toff += nt
        del f, g, got, ups
    assert off == int(r.count.item())
    print(which, "tile-count differences against the reference's fast-math AABB kernel:", count_flips)
    G = r.grads
    for k, ref in tot.items():
        ref = np_(ref).reshape(np_(ref).shape[0], -1)
        got = np_(G[k]).reshape(ref.shape[0], -1)[:, :ref.shape[1]]
        row = np.abs(got - ref).max(-1) / (np.abs(ref).max() + 1e-12)
        frac = float((row > 2e-3).mean())
        print(which, k, "rows beyond 2e-3:", frac, "largest row error:", float(row.max()))
        # summed over 32 views, each view's texel-edge flips (at most 0.1% of
        # its rows) add up: 0.3% of the rows here
        assert frac <= (3e-3 if not stress else 1e-3), (k, frac, float(row.max()))
        if row.shape[0] == edge.shape[0]:
            row = row[~edge]
        # uv gradients jump where a hit crosses a texel edge (bilinear
        # interpolation has no derivative there and each implementation takes
        # one neighbouring cell); summed over 32 views a row can collect
        # several such jumps
        assert row.max() < (5 * cap if k in ("uv0", "umap", "vmap") else cap), (k, float(row.max()))
    close_frac(np_(G["sh_coeffs"]).reshape(-1), np_(tot["sh_coeffs"]).reshape(-1), 2e-3 * float(
        np.abs(np_(tot["sh_coeffs"])).max()), 1e-3, "sh_coeffs", cap=np.inf)
