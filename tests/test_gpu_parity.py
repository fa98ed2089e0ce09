"""CUDA path vs the CPU oracle and the reference's golden vectors.

Integer work (tile counts, keys, sort order, tile ranges) must match bit for
bit; floating-point outputs within the tolerances stated per test.  Every
call goes through the package's public functions and the C ABI.
"""
import os

import numpy as np
import pytest
import torch

import oracle
from gpu_helpers import Case, close_frac as _close, np_, small_scene, upstream

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DEV = "cuda:0"


@pytest.fixture(scope="module", autouse=True)
def _require_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import gstex_cuda_gb300  # noqa: F401  (builds/loads the library)


# --------------------------------------------------------------------------
# projection, SH, sampling
# --------------------------------------------------------------------------
def test_sh_matches_golden():
    import gstex_cuda_gb300 as G
    d = np.load(os.path.join(GOLDEN, "sh.npz"))
    for deg in range(5):
        dirs = torch.tensor(d[f"d{deg}_dirs"], dtype=torch.float32, device=DEV)
        co = torch.tensor(d[f"d{deg}_coeffs"], dtype=torch.float32, device=DEV, requires_grad=True)
        col = G.sh.spherical_harmonics(deg, dirs, co)
        np.testing.assert_allclose(np_(col), d[f"d{deg}_colors"], atol=2e-6, rtol=2e-6)
        col.backward(torch.tensor(d[f"d{deg}_v_colors"], dtype=torch.float32, device=DEV))
        np.testing.assert_allclose(np_(co.grad), d[f"d{deg}_v_coeffs"], atol=2e-6, rtol=2e-6)


def test_texture_sample_matches_golden():
    import gstex_cuda_gb300 as G
    d = np.load(os.path.join(GOLDEN, "sample.npz"))
    tex = torch.tensor(d["texture"], dtype=torch.float32, device=DEV, requires_grad=True)
    uvs = torch.tensor(d["uvs"], dtype=torch.float32, device=DEV, requires_grad=True)
    dims = torch.tensor(d["dims"], device=DEV)
    out = G.texture_sample.texture_sample((7, 1, tex.shape[1]), dims, tex, uvs)
    np.testing.assert_allclose(np_(out), d["out"], atol=2e-6, rtol=2e-6)
    out.backward(torch.tensor(d["v_out"], dtype=torch.float32, device=DEV))
    np.testing.assert_allclose(np_(tex.grad), d["v_texture"], atol=1e-5, rtol=1e-5)
    np.testing.assert_allclose(np_(uvs.grad), d["v_uvs"], atol=2e-4, rtol=1e-4)


def test_num_tiles_hit_matches_golden_bit_exact():
    import gstex_cuda_gb300 as G
    d = np.load(os.path.join(GOLDEN, "tiles.npz"))
    for case in "abc":
        H, W, bw = (int(x) for x in d[f"{case}_hwbw"])
        c = torch.tensor(d[f"{case}_centers"], device=DEV)
        e = torch.tensor(d[f"{case}_extents"], device=DEV)
        got = np_(G.get_aabb_2d.get_num_tiles_hit_2d(c, e, H, W, bw)).astype(np.int32)
        np.testing.assert_array_equal(got, d[f"{case}_counts"])


@pytest.mark.parametrize("seed", [0, 1])
def test_aabb_bit_exact_vs_oracle(seed):
    import gstex_cuda_gb300 as G
    from gstex_cuda_gb300 import synthetic
    spec = synthetic.untextured(seed=seed, n=20000, size=800)
    cam = spec.cameras[0]
    c, e = G.get_aabb_2d.get_aabb_2d(spec.means.to(DEV), spec.scales.to(DEV), 1.0, spec.quats.to(DEV),
                                     cam.viewmat.to(DEV), (cam.fx, cam.fy, cam.cx, cam.cy))
    oc, oe = oracle.get_aabb_2d(spec.means.numpy(), spec.scales.numpy(), 1.0, spec.quats.numpy(),
                                cam.viewmat.numpy(), cam.fx, cam.fy, cam.cx, cam.cy)
    np.testing.assert_array_equal(np_(c), oc)
    np.testing.assert_array_equal(np_(e), oe)


# --------------------------------------------------------------------------
# binning: bit-exact
# --------------------------------------------------------------------------
def _assert_binning_equal(got, ref):
    assert got["n_isect"] == ref["n_isect"]
    np.testing.assert_array_equal(np_(got["counts"]).astype(np.int32), ref["counts"] if "counts" in ref else None)
    np.testing.assert_array_equal(got["isect_ids"].cpu().numpy(), ref["isect_ids"])
    np.testing.assert_array_equal(got["gaussian_ids"].cpu().numpy(), ref["gaussian_ids"])
    np.testing.assert_array_equal(got["isect_ids_sorted"].cpu().numpy(), ref["isect_ids_sorted"])
    np.testing.assert_array_equal(got["gaussian_ids_sorted"].cpu().numpy(), ref["gaussian_ids_sorted"])
    np.testing.assert_array_equal(got["tile_bins"].cpu().numpy(), ref["tile_bins"])


@pytest.mark.parametrize("which", ["tiny", "small", "untextured"])
def test_binning_bit_exact(which):
    from gstex_cuda_gb300 import synthetic
    if which == "tiny":
        spec = synthetic.tiny(0)
    elif which == "small":
        spec = small_scene(n=2000, width=256, height=192, seed=3)
    else:
        spec = synthetic.untextured(seed=1, n=100_000, size=800)
    case = Case(spec, colors=np.zeros((spec.num_points, 3)))
    _assert_binning_equal(case.binning_cuda(), case.binning_np())


@pytest.mark.parametrize("n,dup", [(1, 1), (1000, 3), (300_000, 50), (2_000_003, 1000)])
def test_sort_pairs_stable(n, dup):
    import gstex_cuda_gb300 as G
    rng = np.random.default_rng(n)
    keys = (rng.integers(0, 8160, n).astype(np.int64) << 32) | rng.integers(0, dup, n).astype(np.int64) * 1000
    vals = np.arange(n, dtype=np.int32)
    ko, vo = G.cuda.sort_pairs(torch.from_numpy(keys).to(DEV), torch.from_numpy(vals).to(DEV), end_bit=45)
    order = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(ko.cpu().numpy(), keys[order])
    np.testing.assert_array_equal(vo.cpu().numpy(), vals[order])


def test_phantom_slots_of_clipped_gaussians():
    """A Gaussian behind the near plane has zero extent but the torch tile
    counter still gives it one tile: its slot stays key 0 / id 0 and lands in
    tile 0, exactly as in the reference."""
    spec = small_scene(n=50, width=64, height=64, seed=11)
    spec.means[3] = torch.tensor([0.0, 0.0, -1.0])  # behind the camera; projects inside the image
    case = Case(spec, colors=np.zeros((50, 3)))
    ref = case.binning_np()
    got = case.binning_cuda()
    assert ref["counts"][3] == 1 and ref["extents"][3].max() == 0
    _assert_binning_equal(got, ref)
    assert (ref["isect_ids_sorted"] == 0).sum() >= 1


# --------------------------------------------------------------------------
# compositor forward / backward vs oracle
# --------------------------------------------------------------------------
def _compare_forward(case, bw, settings, bg, tol_img, texture=None, prec="f64", frac=0.0):
    b = case.binning_cuda(bw)
    ref = oracle.texture_forward(case.scene_np, case.cam_np, b["gaussian_ids_sorted"].cpu().numpy(),
                                 b["tile_bins"].cpu().numpy(), bw, settings, bg, prec=prec)
    out, bgt = case.forward_cuda(b["gaussian_ids_sorted"], b["tile_bins"], bw, settings, bg, texture=texture)
    for k in ("img", "texture", "normal", "final_T"):
        _close(np_(out[k]), ref[k], tol_img, frac, k)
    # one flip of alpha >= 1/255 moves the sums (S0, S1, S2) by up to (1, t, t^2) / 255
    tmax = float(np.abs(ref["reg_s"][..., 1]).max() / max(float(ref["reg_s"][..., 0].max()), 1e-6)) + 1.0
    _close(np_(out["reg_s"]), ref["reg_s"], tol_img * (1 + np.abs(ref["reg_s"])), frac, "reg_s",
           cap=(1 + tmax + tmax * tmax) / 255 + 1e-2 * np.abs(ref["reg_s"]))
    _close(np_(out["reg"]), ref["reg"], tol_img * 10 + tol_img * np.abs(ref["reg"]), frac, "reg")
    same_depth = np_(out["depth_idx"]) == ref["depth_idx"]
    assert same_depth.mean() > 0.999
    np.testing.assert_allclose(np_(out["depth"])[same_depth], ref["depth"][same_depth], atol=tol_img * 10,
                               rtol=tol_img, err_msg="depth")
    assert (np_(out["final_idx"]) == ref["final_idx"]).mean() > 0.999
    return b, out, bgt, ref


def _compare_backward(case, b, out, bgt, ref, bw, settings, bg, rtol, texture=None, prec="f64"):
    C = case.spec.texture.shape[1]
    ups = upstream(case.cam.height, case.cam.width, C)
    gref = oracle.texture_backward(case.scene_np, case.cam_np, b["gaussian_ids_sorted"].cpu().numpy(),
                                   b["tile_bins"].cpu().numpy(), bw, settings, bg, ref, ups["img"], ups["depth"],
                                   ups["reg"], ups["alpha"], ups["texture"], ups["normal"], prec=prec)
    g = case.backward_cuda(out, b["gaussian_ids_sorted"], b["tile_bins"], ups, bw, settings, bgt, texture=texture)
    for k in ("colors", "opacity", "means", "scales", "quats", "uv0", "umap", "vmap", "texture"):
        r = gref[k].reshape(-1)
        x = np_(g[k]).reshape(-1)
        if k == "texture" and x.size != r.size:  # bf16 layout [T,4]
            x = np_(g[k])[:, :3].reshape(-1)
        if r.size == 0:
            continue
        scale = np.abs(r).max() + 1e-12
        err = np.abs(x - r).max() / scale
        assert err < rtol, (k, err)


@pytest.mark.parametrize("settings", [1 << 8, 0, (1 << 8) | (1 << 9), (1 << 8) | (1 << 10), (1 << 8) | (1 << 2),
                                      (1 << 8) | (1 << 15)])
def test_raster_tiny_matches_oracle(settings):
    from gstex_cuda_gb300 import synthetic
    case = Case(synthetic.tiny(0))
    bg = np.array([0.2, 0.5, 0.7])
    b, out, bgt, ref = _compare_forward(case, 16, settings, bg, 2e-5)
    if not settings & (1 << 15):
        _compare_backward(case, b, out, bgt, ref, 16, settings, bg, 2e-4)


def test_raster_tiny_matches_reference_golden():
    """Forward and gradients against the reference's own torch rasteriser."""
    d = np.load(os.path.join(GOLDEN, "raster_tiny.npz"))
    from gstex_cuda_gb300 import synthetic
    spec = synthetic.tiny(0)
    spec.umap = torch.tensor(d["umap"])
    spec.vmap = torch.tensor(d["vmap"])
    case = Case(spec, colors=d["colors"])
    gids = torch.tensor(d["gids_sorted"], device=DEV)
    bins = torch.tensor(d["tile_bins"], device=DEV)
    out, bgt = case.forward_cuda(gids, bins, 16, int(d["settings"][0]), d["background"])
    np.testing.assert_allclose(np_(out["img"]), d["f32_out_img"], atol=2e-5)
    np.testing.assert_allclose(1 - np_(out["final_T"]), d["f32_out_alpha"], atol=2e-5)
    np.testing.assert_allclose(np_(out["texture"]), d["f32_out_texture"], atol=2e-5)
    np.testing.assert_allclose(np_(out["normal"]), d["f32_out_normal"], atol=2e-5)
    np.testing.assert_allclose(np_(out["depth"]), d["f32_out_depth"], atol=1e-4)
    np.testing.assert_allclose(np_(out["reg"]), d["f32_out_reg"], atol=1e-5)
    ups = {k: d["up_" + k] for k in ("img", "depth", "reg", "alpha", "texture", "normal")}
    g = case.backward_cuda(out, gids, bins, ups, 16, int(d["settings"][0]), bgt)
    for k in ("means", "scales", "quats", "opacity", "colors", "uv0", "umap", "vmap", "texture"):
        ref = d[f"f32_grad_{k}"]
        got = np_(g[k]).reshape(ref.shape)
        if k == "scales":
            got, ref = got[:, :2], ref[:, :2]
        err = np.abs(got - ref).max() / (np.abs(ref).max() + 1e-12)
        assert err < 2e-4, (k, err)


@pytest.fixture(params=[(1, 32), (2, 32), (1, 16), (1, 8), (1, 4)], ids=["1px", "2px", "1px_g16", "1px_g8", "1px_g4"])
def pixels_per_thread(request):
    """Pixels per thread, and lanes per splat walk of the backward (group
    sizes below 32 apply to block widths that are multiples of 8)."""
    import gstex_cuda_gb300.cuda as C
    old = C.PIXELS_PER_THREAD, C.BACKWARD_GROUP_LANES
    C.PIXELS_PER_THREAD, C.BACKWARD_GROUP_LANES = request.param
    yield request.param[0]
    C.PIXELS_PER_THREAD, C.BACKWARD_GROUP_LANES = old


@pytest.mark.parametrize("w,h,bw", [(64, 64, 16), (48, 32, 16), (70, 45, 8), (33, 29, 5), (40, 30, 10)])
def test_raster_small_matches_oracle(w, h, bw, pixels_per_thread):
    case = Case(small_scene(n=200, width=w, height=h, seed=w + h))
    bg = np.array([1.0, 1.0, 1.0])
    b, out, bgt, ref = _compare_forward(case, bw, 1 << 8, bg, 5e-5)
    _compare_backward(case, b, out, bgt, ref, bw, 1 << 8, bg, 5e-4)


@pytest.mark.parametrize("settings", [1 << 8, (1 << 8) | (1 << 9), (1 << 8) | (1 << 10)])
def test_view_records_match_per_tile_records(settings):
    """texture_forward / texture_backward with the view's splat records built
    once (gstex_view_records, the default) and with every tile deriving the
    records of its Gaussians: both against the oracle, and the same outputs
    and gradients up to float rounding (threshold flips against the fp64
    oracle allowed at the rate of the other parity tests)."""
    import gstex_cuda_gb300.cuda as CU
    case = Case(small_scene(n=400, width=80, height=64, seed=41))
    bg = np.array([0.3, 0.2, 0.1])
    ups = upstream(case.cam.height, case.cam.width, case.spec.texture.shape[1])
    old = CU.PREBUILT_RECORDS
    res = {}
    try:
        for pre in (True, False):
            CU.PREBUILT_RECORDS = pre
            b, out, bgt, ref = _compare_forward(case, 16, settings, bg, 5e-5, frac=1e-3)
            _compare_backward(case, b, out, bgt, ref, 16, settings, bg, 5e-4)
            g = case.backward_cuda(out, b["gaussian_ids_sorted"], b["tile_bins"], ups, 16, settings, bgt)
            res[pre] = (out, g)
    finally:
        CU.PREBUILT_RECORDS = old
    (o1, g1), (o2, g2) = res[True], res[False]
    for k in ("img", "texture", "normal", "final_T", "reg"):
        _close(np_(o1[k]), np_(o2[k]), 1e-5, 1e-3, k)
    assert (np_(o1["final_idx"]) == np_(o2["final_idx"])).mean() > 0.999
    for k in ("colors", "opacity", "means", "scales", "quats", "uv0", "umap", "vmap", "texture"):
        a, r = np_(g1[k]), np_(g2[k])
        assert np.abs(a - r).max() <= 1e-4 * (np.abs(r).max() + 1e-12), k


@pytest.mark.parametrize("C", [0, 1, 5])
def test_raster_generic_channels(C):
    case = Case(small_scene(n=120, width=40, height=40, seed=C, channels=max(C, 1)))
    if C == 0:
        case.spec.texture = case.spec.texture[:, :0]
        case.scene_np.texture = case.scene_np.texture[:, :0]
        case.t["texture"] = case.t["texture"][:, :0].contiguous()
    bg = np.zeros(3)
    b, out, bgt, ref = _compare_forward(case, 16, 1 << 8, bg, 5e-5)
    _compare_backward(case, b, out, bgt, ref, 16, 1 << 8, bg, 5e-4)


def test_raster_bf16_texels(pixels_per_thread):
    """bf16 [T,4] texel storage: compared with the oracle run on the same
    bf16-rounded texel values (all blending in fp32)."""
    case = Case(small_scene(n=300, width=64, height=64, seed=21))
    t16 = torch.zeros(case.spec.texture.shape[0], 4, dtype=torch.bfloat16)
    t16[:, :3] = case.spec.texture.to(torch.bfloat16)
    rounded = t16[:, :3].float().numpy()
    case.scene_np.texture = rounded
    bg = np.zeros(3)
    b, out, bgt, ref = _compare_forward(case, 16, 1 << 8, bg, 5e-5, texture=t16.to(DEV))
    _compare_backward(case, b, out, bgt, ref, 16, 1 << 8, bg, 5e-4, texture=t16.to(DEV))


def test_untextured_800_full_size_vs_oracle():
    """The 800x800, 100k-Gaussian untextured workload against the fp64 oracle."""
    from gstex_cuda_gb300 import synthetic
    spec = synthetic.untextured(seed=1, n=100_000, size=800)
    case = Case(spec)
    bg = np.zeros(3)
    b, out, bgt, ref = _compare_forward(case, 16, 1 << 8, bg, 1e-4, frac=1e-3)


VIS = (1 << 16) | (10 << 17) | (4 << 26)  # alpha-visualisation, alpha_bound 1.25, outline 1 px


@pytest.mark.parametrize("extra", [0, 1 << 24, (1 << 24) | (1 << 25), 1 << 8])
def test_alpha_visualisation_forward_vs_oracle(extra):
    """Settings bits 16-29 (texture.cu:58-63, 201-241): alpha 0.99 inside
    sigma <= alpha_bound^2/2, outline pixels black or white (bit 24),
    low-opacity splats hidden (bit 25).  Forward only: the backward refuses
    the mode."""
    import gstex_cuda_gb300 as G
    case = Case(small_scene(n=150, width=64, height=48, seed=8))
    bw = 16
    settings = VIS | extra
    bg = np.array([0.2, 0.3, 0.4])
    b = case.binning_cuda(bw)
    ref = oracle.texture_forward(case.scene_np, case.cam_np, b["gaussian_ids_sorted"].cpu().numpy(),
                                 b["tile_bins"].cpu().numpy(), bw, settings, bg, prec="f64")
    out, bgt = case.forward_cuda(b["gaussian_ids_sorted"], b["tile_bins"], bw, settings, bg)
    # the outline distance compares sigma at neighbouring pixels with a threshold,
    # so a rounding difference may flip a pixel
    for k in ("img", "texture", "normal", "final_T"):
        _close(np_(out[k]), ref[k], 1e-4, 1e-3, k)
    with pytest.raises(Exception):
        ups = upstream(case.cam.height, case.cam.width, case.spec.texture.shape[1])
        case.backward_cuda(out, b["gaussian_ids_sorted"], b["tile_bins"], ups, bw, settings, bgt)

