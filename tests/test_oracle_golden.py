"""Pin the CPU oracle to golden vectors produced by the reference's own Python.

The fixtures under tests/golden were made by tests/golden/make_golden.py from
gstex_cuda/_torch_impl.py and gstex_cuda/get_aabb_2d.py of the reference.
"""
import os

import numpy as np
import pytest

import oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return np.load(os.path.join(GOLDEN, name))


@pytest.mark.parametrize("deg", range(5))
@pytest.mark.parametrize("prec,tol", [("f64", 1e-12), ("f32", 2e-6)])
def test_sh_matches_reference_torch(deg, prec, tol):
    d = _load("sh.npz")
    dirs, coeffs = d[f"d{deg}_dirs"], d[f"d{deg}_coeffs"]
    col = oracle.sh_forward(deg, deg, dirs, coeffs, prec=prec)
    np.testing.assert_allclose(col, d[f"d{deg}_colors"], atol=tol * 10, rtol=tol)
    vc = oracle.sh_backward(deg, deg, dirs, d[f"d{deg}_v_colors"], prec=prec)
    np.testing.assert_allclose(vc, d[f"d{deg}_v_coeffs"], atol=tol * 10, rtol=tol)


def test_sh_degrees_to_use_below_degree():
    d = _load("sh.npz")
    dirs, coeffs = d["d4_dirs"], d["d4_coeffs"]
    for use in range(4):
        nb = (use + 1) ** 2
        col = oracle.sh_forward(4, use, dirs, coeffs, prec="f64")
        ref = (oracle.sh_forward(use, use, dirs, np.ascontiguousarray(coeffs[:, :nb]), prec="f64"))
        np.testing.assert_allclose(col, ref, atol=1e-12)
        vc = oracle.sh_backward(4, use, dirs, d["d4_v_colors"], prec="f64")
        assert np.all(vc[:, nb:] == 0)


@pytest.mark.parametrize("prec,tol", [("f64", 1e-12), ("f32", 2e-6)])
def test_texture_sample_matches_reference_torch(prec, tol):
    d = _load("sample.npz")
    out = oracle.texture_sample_forward(d["dims"], d["uvs"], d["texture"], prec=prec)
    np.testing.assert_allclose(out, d["out"], atol=tol, rtol=tol)
    vt, vu = oracle.texture_sample_backward(d["dims"], d["uvs"], d["texture"], d["v_out"], prec=prec)
    np.testing.assert_allclose(vt, d["v_texture"], atol=tol * 10, rtol=tol * 10)
    np.testing.assert_allclose(vu, d["v_uvs"], atol=tol * 100, rtol=tol * 10)


@pytest.mark.parametrize("case", ["a", "b", "c"])
def test_num_tiles_hit_bit_exact(case):
    d = _load("tiles.npz")
    H, W, bw = (int(x) for x in d[f"{case}_hwbw"])
    got = oracle.num_tiles_hit(d[f"{case}_centers"], d[f"{case}_extents"], H, W, bw)
    np.testing.assert_array_equal(got, d[f"{case}_counts"])


def test_project_points_matches_reference_torch():
    d = _load("tiles.npz")
    pix, depth = oracle.project_points(d["pp_means"], d["pp_viewmat"], 500.0, 480.0, 320.0, 240.0)
    np.testing.assert_allclose(depth, d["pp_depths"], rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(pix, d["pp_pix"], rtol=1e-6, atol=1e-4)


@pytest.mark.parametrize("case", ["a", "b"])
def test_emission_count_matches_reference_counter(case):
    """With a power-of-two tile width the kernel's emission loop produces exactly
    the per-Gaussian counts of the reference's torch tile counter, so every slot
    is written (except for Gaussians skipped for a tiny extent)."""
    d = _load("tiles.npz")
    H, W, bw = (int(x) for x in d[f"{case}_hwbw"])
    c, e = d[f"{case}_centers"], d[f"{case}_extents"]
    counts = d[f"{case}_counts"]
    depths = np.linspace(1.0, 2.0, c.shape[0]).astype(np.float32)
    b = oracle.bin_and_sort(c, e, depths, counts, H, W, bw)
    keys, gids = b["isect_ids"], b["gaussian_ids"]
    skipped = (e[:, 0] <= 1e-4) & (e[:, 1] <= 1e-4)
    emitted = np.bincount(gids[keys != 0], minlength=c.shape[0])
    np.testing.assert_array_equal(emitted[~skipped], counts[~skipped])
    # sortedness and range consistency
    ks = b["isect_ids_sorted"]
    assert np.all(np.diff(ks) >= 0)
    bins = b["tile_bins"]
    for t in np.unique(ks >> 32):
        lo, hi = bins[t]
        assert np.all((ks[lo:hi] >> 32) == t)


def _raster_inputs(d):
    scene = oracle.Scene(means=d["means"], scales=d["scales"], quats=d["quats"], opacity=d["opacity"],
                         colors=d["colors"], uv0=d["uv0"], umap=d["umap"], vmap=d["vmap"],
                         texture_dims=d["texture_dims"], texture=d["texture_vals"], glob_scale=1.0)
    fx, fy, cx, cy = (float(x) for x in d["intrins"])
    H, W = (int(x) for x in d["hw"])
    cam = oracle.Camera(d["viewmat"], d["c2w"], fx, fy, cx, cy, H, W)
    return scene, cam


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_raster_forward_matches_reference_torch(prec):
    d = _load("raster_tiny.npz")
    scene, cam = _raster_inputs(d)
    out = oracle.texture_forward(scene, cam, d["gids_sorted"], d["tile_bins"], 16, int(d["settings"][0]),
                                 d["background"], prec=prec)
    for k in ("img", "depth", "reg", "alpha", "texture", "normal"):
        np.testing.assert_allclose(out[k], d[f"f32_out_{k}"], atol=2e-6, rtol=2e-5, err_msg=k)


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_raster_backward_matches_reference_autograd(prec):
    d = _load("raster_tiny.npz")
    scene, cam = _raster_inputs(d)
    st = int(d["settings"][0])
    fwd = oracle.texture_forward(scene, cam, d["gids_sorted"], d["tile_bins"], 16, st, d["background"], prec=prec)
    g = oracle.texture_backward(scene, cam, d["gids_sorted"], d["tile_bins"], 16, st, d["background"], fwd,
                                d["up_img"], d["up_depth"], d["up_reg"], d["up_alpha"], d["up_texture"],
                                d["up_normal"], prec=prec)
    for k in ("means", "scales", "quats", "opacity", "colors", "uv0", "umap", "vmap", "texture"):
        ref = d[f"f32_grad_{k}"]
        got = g[k].reshape(ref.shape)
        scale = np.abs(ref).max() + 1e-12
        if k == "scales":  # the reference never differentiates the unused third scale axis
            got, ref = got[:, :2], ref[:, :2]
        err = np.abs(got - ref).max() / scale
        assert err < 5e-5, (k, err)
