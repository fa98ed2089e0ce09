"""CUDA path vs the reference's own CUDA kernels on the same GPU.

The reference kernels are compiled from the reference's sources into cubins
(oracle/refkern/build_ref.py) and launched with the reference's host-side
grid, block and argument lists (oracle/refkern).  Both sides get identical
inputs.  Integer work (tile counts, keys, per-slot ids, tile ranges) must
match bit for bit; floating-point outputs within the tolerances stated per
test.  The reference kernels are built with --use_fast_math (approximate
exp, division and square root), so their floats differ from exact IEEE
arithmetic by a few ulp.
"""
import numpy as np
import pytest
import torch

from gpu_helpers import Case, close_frac, np_, small_scene, upstream

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


@pytest.fixture(scope="module", autouse=True)
def _require():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import refkern
    if not refkern.available():
        pytest.skip("reference cubins absent (oracle/refkern/build_ref.py builds them where the reference is)")
    import gstex_cuda_gb300  # noqa: F401


def _R():
    from oracle import refkern
    return refkern


def _G():
    import gstex_cuda_gb300 as G
    return G


# --------------------------------------------------------------------------
# SH, AABB, sampling
# --------------------------------------------------------------------------
@pytest.mark.parametrize("degree", [0, 1, 2, 3, 4])
def test_sh_vs_reference_kernels(degree):
    R, G = _R(), _G()
    g = torch.Generator().manual_seed(degree)
    n = 3000
    nb = (degree + 1) ** 2
    dirs = torch.randn(n, 3, generator=g).to(DEV)
    co = (0.3 * torch.randn(n, nb, 3, generator=g)).to(DEV)
    vcol = torch.randn(n, 3, generator=g).to(DEV)
    for use in range(degree + 1):
        ref = R.compute_sh_forward(n, degree, use, dirs, co)
        got = G.cuda.compute_sh_forward(n, degree, use, dirs, co)
        np.testing.assert_allclose(np_(got), np_(ref), atol=2e-6, rtol=2e-5)
        rv = R.compute_sh_backward(n, degree, use, dirs, vcol)
        gv = G.cuda.compute_sh_backward(n, degree, use, dirs, vcol)
        np.testing.assert_allclose(np_(gv), np_(rv), atol=2e-6, rtol=2e-5)


@pytest.mark.parametrize("which", ["small", "untextured", "behind"])
def test_aabb_vs_reference_kernels(which):
    R, G = _R(), _G()
    if which == "small":
        spec = small_scene(n=500, width=96, height=64, seed=3)
        vm = spec.cameras[0].viewmat
    else:
        from gstex_cuda_gb300 import synthetic
        spec = synthetic.untextured(seed=1, n=20_000, size=800)
        vm = spec.cameras[0].viewmat.clone()
        if which == "behind":  # move the camera into the cloud: some means behind it, some at the plane
            vm[2, 3] = 0.0
    cam = spec.cameras[0]
    args = [t.contiguous().to(DEV) for t in (spec.means, spec.scales)]
    q = spec.quats.contiguous().to(DEV)
    vmd = vm.contiguous().to(DEV)
    rc, re_ = R.get_aabb_2d(args[0], args[1], 1.0, q, vmd, cam.fx, cam.fy, cam.cx, cam.cy)
    gc, ge = G.cuda.get_aabb_2d(args[0], args[1], 1.0, q, vmd, cam.fx, cam.fy, cam.cx, cam.cy)
    rc, re_, gc, ge = np_(rc), np_(re_), np_(gc), np_(ge)
    # clipped Gaussians (mean z <= 0.01) get extent 0 on both sides
    np.testing.assert_array_equal(re_ == 0, ge == 0)
    np.testing.assert_allclose(gc, rc, atol=1e-3, rtol=2e-5)
    np.testing.assert_allclose(ge, re_, atol=1e-3, rtol=2e-5)


def test_texture_sample_vs_reference_kernels():
    R, G = _R(), _G()
    g = torch.Generator().manual_seed(11)
    Q, C = 4000, 5
    hw = torch.randint(1, 9, (Q, 2), generator=g).to(torch.int32)
    dims = torch.zeros(Q, 3, dtype=torch.int32)
    dims[:, :2] = hw
    sizes = hw[:, 0].long() * hw[:, 1].long()
    dims[:, 2] = (torch.cumsum(sizes, 0) - sizes).to(torch.int32)
    tex = torch.rand(int(sizes.sum()), C, generator=g)
    # the reference kernel indexes out of range for uv < 0, so the queries stay
    # in [0, 1] (both edges included); its backward is not compared: it reads
    # the upstream gradient from its own output array
    uvs = torch.rand(Q, 2, generator=g)
    uvs[:200] = torch.tensor([0.0, 1.0])
    uvs[200:400] = torch.tensor([1.0, 0.0])
    d, t, u = (x.contiguous().to(DEV) for x in (dims, tex, uvs))
    info = (Q, 1, C)
    ref = R.texture_sample_forward(info, d, u, t)
    got = G.cuda.texture_sample_forward(info, d, u, t)
    np.testing.assert_allclose(np_(got), np_(ref), atol=2e-6, rtol=2e-6)


# --------------------------------------------------------------------------
# binning: bit-exact
# --------------------------------------------------------------------------
def _ref_binning(case, bw):
    """The reference pipeline end to end: its AABB kernel, its tile counts,
    cumsum, its emission kernel, torch.sort, its bin-edge kernel."""
    R = _R()
    t, cam = case.t, case.cam
    c, e = R.get_aabb_2d(t["means"], t["scales"], case.spec.glob_scale, t["quats"], t["viewmat"], *case.intr)
    vm = t["viewmat"]
    depths = (t["means"] @ vm.T[:3, :3] + vm.T[3:, :3])[:, 2].contiguous()
    counts = R.num_tiles_hit(c, e, cam.height, cam.width, bw)
    tb = ((cam.width + bw - 1) // bw, (cam.height + bw - 1) // bw, 1)
    n, isect_sorted, gids_sorted, bins = R.bin_and_sort(case.spec.num_points, c, e, depths, counts, tb, bw)
    return dict(centers=c, extents=e, depths=depths, counts=counts, n=n, isect_sorted=isect_sorted,
                gids_sorted=gids_sorted, bins=bins, tile_bounds=tb)


def _runs_equal(keys, a, b):
    """Ids sorted by key are equal up to the order inside runs of equal keys."""
    keys, a, b = np_(keys).astype(np.int64), np_(a), np_(b)
    if keys.size == 0:
        return
    cut = np.flatnonzero(np.diff(keys)) + 1
    for ra, rb in zip(np.split(a, cut), np.split(b, cut)):
        np.testing.assert_array_equal(np.sort(ra), np.sort(rb))


@pytest.mark.parametrize("which,bw", [("small", 16), ("small", 8), ("untextured", 16), ("tex1080", 16)])
def test_binning_bit_exact_vs_reference_kernels(which, bw):
    R, G = _R(), _G()
    from gstex_cuda_gb300 import synthetic
    spec = {"small": lambda: small_scene(n=800, width=160, height=96, seed=2),
            "untextured": lambda: synthetic.untextured(seed=1, n=30_000, size=800),
            "tex1080": lambda: synthetic.textured_1080p(seed=2, n=4000, texels=100_000)}[which]()
    case = Case(spec, colors=np.zeros((spec.num_points, 3), np.float32))
    r = _ref_binning(case, bw)
    cam = case.cam
    # the same centers / extents / depths into both pipelines
    counts = G.cuda.num_tiles_hit(r["centers"], r["extents"], cam.height, cam.width, bw)
    np.testing.assert_array_equal(np_(counts), np_(r["counts"]))
    cum = torch.cumsum(counts, 0, dtype=torch.int32)
    n = int(cum[-1].item())
    assert n == r["n"]
    isect, gids = G.cuda.map_gaussian_to_intersects(spec.num_points, n, r["centers"], r["extents"], r["depths"], cum,
                                                    r["tile_bounds"], bw, False)
    risect, rgids = R.map_gaussian_to_intersects(spec.num_points, n, r["centers"], r["extents"], r["depths"], cum,
                                                 r["tile_bounds"], bw)
    np.testing.assert_array_equal(isect.cpu().numpy(), risect.cpu().numpy())
    np.testing.assert_array_equal(gids.cpu().numpy(), rgids.cpu().numpy())
    keys, order = G.cuda.sort_pairs(isect, gids)
    np.testing.assert_array_equal(keys.cpu().numpy(), r["isect_sorted"].cpu().numpy())
    _runs_equal(r["isect_sorted"].cpu(), order.cpu(), r["gids_sorted"].cpu())
    bins = G.cuda.get_tile_bin_edges(n, keys, r["tile_bounds"])
    np.testing.assert_array_equal(bins.cpu().numpy(), r["bins"].cpu().numpy())


# --------------------------------------------------------------------------
# compositor forward / backward
# --------------------------------------------------------------------------
OUT_NAMES = ("img", "depth", "reg", "texture", "normal", "final_T", "final_idx", "depth_idx", "reg_s")
GRAD_NAMES = ("colors", "opacity", "means", "scales", "quats", "uv0", "umap", "vmap", "texture")


def _scene(which):
    from gstex_cuda_gb300 import synthetic
    return {"tiny": lambda: synthetic.tiny(0),
            "small": lambda: small_scene(n=600, width=160, height=96, seed=4),
            "untextured": lambda: synthetic.untextured(seed=1, n=30_000, size=800),
            "tex1080": lambda: synthetic.textured_1080p(seed=2, n=6000, texels=400_000)}[which]()


def _both(case, bw, settings, bg):
    """Forward and backward through the reference kernels and through the
    package, on the reference's binning and identical upstream gradients."""
    R, G = _R(), _G()
    r = _ref_binning(case, bw)
    t, cam, sp = case.t, case.cam, case.spec
    C = sp.texture.shape[1]
    info = (sp.num_points, 1, C)
    bgt = torch.tensor(bg, dtype=torch.float32, device=DEV)
    tb = r["tile_bounds"]
    common = (info, t["dims"], r["gids_sorted"], r["bins"], t["colors"], t["opacity"], t["means"], t["scales"],
              sp.glob_scale, t["quats"], t["uv0"], t["umap"], t["vmap"], t["texture"], t["viewmat"], t["c2w"],
              *case.intr, settings, bgt)
    fr = dict(zip(OUT_NAMES, R.texture_forward(tb, (bw, bw, 1), (cam.width, cam.height, 1), *common)))
    fg = dict(zip(OUT_NAMES, G.cuda.texture_forward(tb, (bw, bw, 1), (cam.width, cam.height, 1), *common)))
    ups = {k: torch.as_tensor(v, dtype=torch.float32).contiguous().to(DEV)
           for k, v in upstream(cam.height, cam.width, C).items()}
    tail = lambda f: (f["final_T"], f["final_idx"], f["depth_idx"].clone(), f["reg_s"], ups["img"], ups["depth"],  # noqa
                      ups["reg"], ups["alpha"], ups["texture"], ups["normal"])
    gr = dict(zip(GRAD_NAMES, R.texture_backward(cam.height, cam.width, bw, *common, *tail(fr))))
    gg = dict(zip(GRAD_NAMES, G.cuda.texture_backward(cam.height, cam.width, bw, *common, *tail(fg))))
    torch.cuda.synchronize()
    return r, fr, fg, gr, gg


def _edge_on(spec, cam, cut=0.05):
    """Splats seen almost edge-on (|n . mu| / |mu| < cut in camera space): their
    mean and rotation gradients carry 1/|n.r| and are compared against fp64
    in test_edge_on_splats_vs_fp64_oracle instead of the reference's fp32."""
    q = spec.quats.double()
    w, x, y, z = q.unbind(-1)
    n = torch.stack([2 * (x * z + w * y), 2 * (y * z - w * x), 1 - 2 * (x * x + y * y)], -1)
    vm = cam.viewmat.double()
    mc = spec.means.double() @ vm[:3, :3].T + vm[:3, 3]
    nc = n @ vm[:3, :3].T
    return ((nc * mc).sum(-1).abs() / mc.norm(dim=-1) < cut).numpy()


def _compare(fr, fg, gr, gg, tol, frac, rtol_grad, rows_frac=0.0, one_texel=False, edge_on=None, row_cap=10.0,
             out_cap=1e-2):
    """Outputs within tol except a fraction frac of threshold flips.  Each
    gradient row (one Gaussian, or one texel) within rtol_grad of the
    reference kernels' largest entry, except a fraction rows_frac of rows,
    which must stay within 10x that: a hit whose texture coordinate lies
    within rounding of a texel edge takes the uv-gradient of either
    neighbouring cell (bilinear interpolation is not differentiable there),
    and a grazing splat multiplies that difference by 1/|n.r| in its mean and
    rotation gradients.  With 1x1 charts the uv-gradients are zero in exact
    arithmetic and both kernels return rounding noise, so they are skipped."""
    for k in ("img", "texture", "normal", "final_T"):
        close_frac(np_(fg[k]), np_(fr[k]), tol, frac, k, cap=out_cap * (1 + np.abs(np_(fr[k]))))
    ref_s = np_(fr["reg_s"])
    tmax = float(np.abs(ref_s[..., 1]).max() / max(float(ref_s[..., 0].max()), 1e-6)) + 1.0
    close_frac(np_(fg["reg_s"]), ref_s, tol * (1 + np.abs(ref_s)), frac, "reg_s",
               cap=(1 + tmax + tmax * tmax) / 255 + 1e-2 * np.abs(ref_s))
    # a flip moves reg by up to (alpha = 1/255) x (t - mean t)^2 x ...: the same bound as reg_s
    rr = np_(fr["reg"])
    close_frac(np_(fg["reg"]), rr, tol * 10 + tol * np.abs(rr), frac, "reg",
               cap=(1 + tmax + tmax * tmax) / 255 + 1e-2 * np.abs(rr))
    same = np_(fg["depth_idx"]) == np_(fr["depth_idx"])
    assert same.mean() >= 1 - frac, ("depth_idx", float(same.mean()))
    # the same depth Gaussian can still give a different depth where the ray
    # runs almost inside a splat whose plane passes almost through the camera
    # centre: t = n.(mu - o) / n.r is then a ratio of two rounding-level terms
    dr = np_(fr["depth"])[same]
    close_frac(np_(fg["depth"])[same], dr, tol * 10 + tol * np.abs(dr), frac, "depth", cap=np.inf)
    assert (np_(fg["final_idx"]) == np_(fr["final_idx"])).mean() >= 1 - frac
    for k in GRAD_NAMES:
        if k not in gr or (one_texel and k in ("uv0", "umap", "vmap")):
            continue
        ref = np_(gr[k])
        got = np_(gg[k])
        if ref.size == 0:
            continue
        ref = ref.reshape(ref.shape[0], -1)
        got = got.reshape(ref.shape[0], -1)[:, :ref.shape[1]]
        row = np.abs(got - ref).max(-1) / (np.abs(ref).max() + 1e-12)
        assert (row > rtol_grad).mean() <= rows_frac, (k, float((row > rtol_grad).mean()), float(row.max()))
        if edge_on is not None and row.shape[0] == edge_on.shape[0]:
            row = row[~edge_on]
        assert row.max() < row_cap * rtol_grad, (k, float(row.max()))


@pytest.mark.parametrize("settings", [1 << 8, 0, (1 << 8) | (1 << 9), (1 << 8) | (1 << 10), (1 << 8) | (1 << 2)])
def test_raster_tiny_vs_reference_kernels(settings):
    case = Case(_scene("tiny"))
    _, fr, fg, gr, gg = _both(case, 16, settings, [0.2, 0.5, 0.7])
    _compare(fr, fg, gr, gg, 2e-5, 0.0, 1e-3)


def test_raster_flip_normals_forward_vs_reference_kernels():
    """Bit 15 (normals flipped towards the camera) is a forward-only setting."""
    case = Case(_scene("small"))
    _, fr, fg, _, _ = _both(case, 16, (1 << 8) | (1 << 15), [0.0, 0.0, 0.0])
    close_frac(np_(fg["normal"]), np_(fr["normal"]), 1e-4, 1e-3, "normal")
    close_frac(np_(fg["img"]), np_(fr["img"]), 1e-4, 1e-3, "img")


@pytest.mark.parametrize("which,bw", [("small", 16), ("small", 8), ("untextured", 16), ("tex1080", 16)])
def test_raster_vs_reference_kernels(which, bw):
    """Threshold flips between two fp32 kernels (the reference's built with
    fast-math exp) stay below 0.3% of the pixels, and texel-edge flips below
    0.1% of the gradient rows, at these sizes."""
    case = Case(_scene(which))
    r, fr, fg, gr, gg = _both(case, bw, 1 << 8, [0.0, 0.0, 0.0])
    _compare(fr, fg, gr, gg, 1e-4, 3e-3, 2e-3, rows_frac=1e-3, one_texel=which == "untextured")


@pytest.mark.parametrize("which", ["untextured_800_100k", "textured_1080p_200k", "stress_1080p_1M"])
def test_full_size_vs_reference_kernels(which):
    """The single-view workloads at full size against the reference kernels:
    800x800 with 100k untextured (1x1-chart) Gaussians and SH degree 3
    colours; 1920x1080 with 200k Gaussians and 8M fp32 texels; and one
    1920x1080 view of the stress scene (1M Gaussians in 64 clusters, 32M fp32
    texels, heavy per-tile overlap).  The tile counts, keys and ranges are
    compared bit for bit on the way."""
    from gstex_cuda_gb300 import synthetic
    spec = {"untextured_800_100k": lambda: synthetic.untextured(seed=1),
            "textured_1080p_200k": lambda: synthetic.textured_1080p(seed=2),
            "stress_1080p_1M": lambda: synthetic.stress(seed=4, views=1)}[which]()
    case = Case(spec)
    bw = 16
    r, fr, fg, gr, gg = _both(case, bw, 1 << 8, [0.0, 0.0, 0.0])
    G = _G()
    cam = case.cam
    counts = G.cuda.num_tiles_hit(r["centers"], r["extents"], cam.height, cam.width, bw)
    assert torch.equal(counts, r["counts"])
    cum = torch.cumsum(counts, 0, dtype=torch.int32)
    isect, gids = G.cuda.map_gaussian_to_intersects(spec.num_points, r["n"], r["centers"], r["extents"], r["depths"],
                                                    cum, r["tile_bounds"], bw, False)
    keys, _ = G.cuda.sort_pairs(isect, gids, G.cuda.sort_end_bit(r["bins"].shape[0]))
    assert torch.equal(keys, r["isect_sorted"])
    assert torch.equal(G.cuda.get_tile_bin_edges(r["n"], keys, r["tile_bounds"]), r["bins"])
    # The stress scene's 64 dense clusters put more pairs near the thresholds,
    # and its smallest splats (s = 0.005) have uv maps of 1/(6 s) = 33 per unit,
    # which carry a texel-edge flip of the uv gradient into the mean gradient
    # 33 times over: its rare outlier rows get a cap of 5% of the largest entry.
    stress = which.startswith("stress")
    _compare(fr, fg, gr, gg, 1e-4, 5e-3 if stress else 3e-3, 2e-3, rows_frac=1e-3,
             one_texel=which.startswith("untextured"), edge_on=_edge_on(spec, case.cam),
             row_cap=25.0 if stress else 10.0)


def test_edge_on_splats_vs_fp64_oracle():
    """A scene of splats seen almost edge-on (|n.d| from 1e-4 to 5e-2 at the
    mean), where the ray-plane solve is ill-conditioned: the gradients of this
    package (records solved in double for these splats) and of the reference
    kernels (fp32, fast math) against the fp64 oracle.  Both are within a few
    1e-3 of the largest entry; ours must be within twice the reference's error
    or 5e-3."""
    import oracle
    g = torch.Generator().manual_seed(31)
    spec = small_scene(n=120, width=96, height=64, seed=31, f=96.0)
    # rotate every splat so that its normal is nearly perpendicular to the view ray
    mc = spec.means.double()
    d = mc / mc.norm(dim=-1, keepdim=True)
    t = torch.cross(d, torch.randn(mc.shape, generator=g, dtype=torch.float64), dim=-1)
    t = t / t.norm(dim=-1, keepdim=True)
    eps = torch.exp(torch.empty(mc.shape[0], 1, dtype=torch.float64).uniform_(np.log(1e-4), np.log(5e-2),
                                                                              generator=g))
    n = t + eps * d
    n = n / n.norm(dim=-1, keepdim=True)
    a1 = torch.cross(n, torch.randn(mc.shape, generator=g, dtype=torch.float64), dim=-1)
    a1 = a1 / a1.norm(dim=-1, keepdim=True)
    a2 = torch.cross(n, a1, dim=-1)
    Rm = torch.stack([a1, a2, n], -1)  # columns = axes
    # rotation matrix -> quaternion (w, x, y, z), trace method with a safe branch
    qs = []
    for R in Rm:
        tr = R.trace()
        if tr > 0:
            sq = torch.sqrt(tr + 1.0) * 2
            qs.append(torch.stack([0.25 * sq, (R[2, 1] - R[1, 2]) / sq, (R[0, 2] - R[2, 0]) / sq,
                                   (R[1, 0] - R[0, 1]) / sq]))
        else:
            i = int(torch.argmax(torch.diagonal(R)))
            j, k = (i + 1) % 3, (i + 2) % 3
            sq = torch.sqrt(1.0 + R[i, i] - R[j, j] - R[k, k]) * 2
            q = torch.zeros(4, dtype=torch.float64)
            q[0] = (R[k, j] - R[j, k]) / sq
            q[1 + i] = 0.25 * sq
            q[1 + j] = (R[j, i] + R[i, j]) / sq
            q[1 + k] = (R[k, i] + R[i, k]) / sq
            qs.append(q)
    spec.quats.copy_(torch.stack(qs).float())
    spec.umap.copy_((a1 / (6 * spec.scales[:, :1].double()))[:, None].float())
    spec.vmap.copy_((a2 / (6 * spec.scales[:, 1:2].double()))[:, None].float())
    case = Case(spec)
    assert _edge_on(spec, case.cam).all()
    bg = [0.0, 0.0, 0.0]
    r, fr, fg, gr, gg = _both(case, 16, 1 << 8, bg)
    C = spec.texture.shape[1]
    ups = upstream(case.cam.height, case.cam.width, C)
    gids, bins = r["gids_sorted"].cpu().numpy(), r["bins"].cpu().numpy()
    fwd = oracle.texture_forward(case.scene_np, case.cam_np, gids, bins, 16, 1 << 8, np.asarray(bg), prec="f64")
    go = oracle.texture_backward(case.scene_np, case.cam_np, gids, bins, 16, 1 << 8, np.asarray(bg), fwd,
                                 ups["img"], ups["depth"], ups["reg"], ups["alpha"], ups["texture"], ups["normal"],
                                 prec="f64")
    for k in ("means", "quats", "scales", "opacity", "colors", "uv0", "umap", "vmap"):
        truth = np.asarray(go[k]).reshape(spec.num_points, -1)
        scale = np.abs(truth).max() + 1e-12
        e_ours = np.abs(np_(gg[k]).reshape(spec.num_points, -1) - truth).max() / scale
        e_ref = np.abs(np_(gr[k]).reshape(spec.num_points, -1) - truth).max() / scale
        assert e_ours <= max(2 * e_ref, 5e-3), (k, float(e_ours), float(e_ref))


def test_alpha_visualisation_forward_vs_reference_kernels():
    """Settings bits 16, 17-21, 24-29 against the reference's forward kernel."""
    case = Case(_scene("small"))
    settings = (1 << 16) | (10 << 17) | (4 << 26) | (1 << 24)
    R, G = _R(), _G()
    r = _ref_binning(case, 16)
    t, cam, sp = case.t, case.cam, case.spec
    info = (sp.num_points, 1, sp.texture.shape[1])
    bgt = torch.tensor([0.2, 0.3, 0.4], dtype=torch.float32, device=DEV)
    common = (info, t["dims"], r["gids_sorted"], r["bins"], t["colors"], t["opacity"], t["means"], t["scales"],
              sp.glob_scale, t["quats"], t["uv0"], t["umap"], t["vmap"], t["texture"], t["viewmat"], t["c2w"],
              *case.intr, settings, bgt)
    tb = r["tile_bounds"]
    fr = dict(zip(OUT_NAMES, R.texture_forward(tb, (16, 16, 1), (cam.width, cam.height, 1), *common)))
    fg = dict(zip(OUT_NAMES, G.cuda.texture_forward(tb, (16, 16, 1), (cam.width, cam.height, 1), *common)))
    for k in ("img", "texture", "normal", "final_T"):
        close_frac(np_(fg[k]), np_(fr[k]), 1e-4, 1e-2, k)
