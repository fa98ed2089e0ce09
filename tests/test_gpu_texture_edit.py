"""texture_edit (csrc/texture_edit.cu) against the reference's own kernel and
the fp64 oracle, on identical inputs and the same binning.

Each texel row holds sums of bilinear splats; a float rounding difference can
flip one of the reference's thresholds (alpha >= 1/255, T <= 1e-4, the depth
range) for a (pixel, splat) pair, which moves that pair's splat (total weight
1 over four texels) in or out.  So all but a 0.2% fraction of rows must agree
to 1e-4 (relative to the row's size), and the rest within 1 per channel.
"""
import numpy as np
import pytest
import torch

import oracle
from gpu_helpers import Case, np_, small_scene

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


@pytest.fixture(scope="module", autouse=True)
def _require():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import gstex_cuda_gb300  # noqa: F401


def _scene(which):
    from gstex_cuda_gb300 import synthetic
    return {"tiny": lambda: synthetic.tiny(0),
            "small": lambda: small_scene(n=600, width=160, height=96, seed=4),
            "tex1080": lambda: synthetic.textured_1080p(seed=2, n=6000, texels=400_000)}[which]()


def _edit_inputs(H, W, seed=2):
    g = np.random.default_rng(seed)
    img = g.uniform(0, 1, (H, W, 3))
    alpha = g.uniform(0, 1, (H, W)) * (g.uniform(0, 1, (H, W)) > 0.3)
    lo = g.uniform(0.0, 2.8, (H, W))
    hi = lo + g.uniform(0.3, 2.0, (H, W))
    return img, alpha, lo, hi


def _rows_close(got, ref, name, frac=2e-3):
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    err = np.abs(got - ref).max(-1)
    bad = err > 1e-4 * (1 + np.abs(ref).max(-1))
    assert bad.mean() <= frac, (name, float(bad.mean()), float(err.max()))
    assert err.max() <= 1.0 + 1e-3, (name, float(err.max()))


def _run(which, settings, bw=16):
    import gstex_cuda_gb300 as G
    spec = _scene(which)
    case = Case(spec, colors=np.zeros((spec.num_points, 3), np.float32))
    b = case.binning_cuda(bw)
    cam, t = case.cam, case.t
    H, W = cam.height, cam.width
    img, alpha, lo, hi = _edit_inputs(H, W)
    f = lambda x: torch.as_tensor(x, dtype=torch.float32).contiguous().to(DEV)  # noqa: E731
    T = spec.texture.shape[0]
    info = (spec.num_points, 1, 5)
    args = ((b["tile_bounds"][0], b["tile_bounds"][1], 1), (bw, bw, 1), (W, H, 1), info, T, t["dims"], f(img),
            f(alpha), f(lo), f(hi), b["gaussian_ids_sorted"], b["tile_bins"], t["opacity"], t["means"], t["scales"],
            spec.glob_scale, t["quats"], t["uv0"], t["umap"], t["vmap"], t["viewmat"], t["c2w"], *case.intr, settings,
            torch.zeros(3, device=DEV))
    got = np_(G.cuda.texture_edit(*args))
    gids, bins = b["gaussian_ids_sorted"].cpu().numpy(), b["tile_bins"].cpu().numpy()
    ora = oracle.texture_edit(case.scene_np, case.cam_np, gids, bins, bw, settings, img, alpha, lo, hi, T, prec="f64")
    ref = None
    from oracle import refkern
    if refkern.available():
        ref = np_(refkern.texture_edit(*args))
    return got, ora, ref


@pytest.mark.parametrize("which", ["tiny", "small", "tex1080"])
@pytest.mark.parametrize("settings", [0, 1])
def test_texture_edit_matches_oracle_and_reference_kernel(which, settings):
    got, ora, ref = _run(which, settings)
    assert got.shape == ora.shape and ora[:, 4].sum() > 0
    _rows_close(got, ora, "vs oracle")
    if ref is not None:
        _rows_close(got, ref, "vs reference kernel")
        _rows_close(ref, ora, "reference kernel vs oracle")


def test_texture_edit_python_surface():
    """gstex_cuda_gb300.texture_edit.texture_edit with the reference's
    signature, binning included, against the oracle on the same binning."""
    import gstex_cuda_gb300 as G
    spec = _scene("small")
    case = Case(spec, colors=np.zeros((spec.num_points, 3), np.float32))
    cam, t = case.cam, case.t
    H, W = cam.height, cam.width
    img, alpha, lo, hi = _edit_inputs(H, W, seed=5)
    f = lambda x: torch.as_tensor(x, dtype=torch.float32).contiguous().to(DEV)  # noqa: E731
    c, e = G.get_aabb_2d.get_aabb_2d(t["means"], t["scales"], 1.0, t["quats"], t["viewmat"], case.intr)
    _, depths = G.get_aabb_2d.project_points(t["means"], t["viewmat"], case.intr)
    nt = G.get_aabb_2d.get_num_tiles_hit_2d(c, e, H, W, 16)
    out = G.texture_edit.texture_edit((spec.num_points, 1, 5), t["dims"], f(img), f(alpha[..., None]), f(lo), f(hi),
                                      c, e, depths.contiguous(), nt, t["opacity"], t["means"], t["scales"], 1.0,
                                      t["quats"], t["uv0"], t["umap"], t["vmap"], t["viewmat"], t["c2w"], *case.intr,
                                      H, W, 16, 0)
    b = case.binning_np(16)
    ora = oracle.texture_edit(case.scene_np, case.cam_np, b["gaussian_ids_sorted"], b["tile_bins"], 16, 0, img, alpha,
                              lo, hi, spec.texture.shape[0], prec="f64")
    _rows_close(np_(out), ora, "python surface vs oracle")
    with pytest.raises(Exception):
        G.texture_edit.texture_edit((spec.num_points, 1, 3), t["dims"], f(img), f(alpha), f(lo), f(hi), c, e,
                                    depths.contiguous(), nt, t["opacity"], t["means"], t["scales"], 1.0, t["quats"],
                                    t["uv0"], t["umap"], t["vmap"], t["viewmat"], t["c2w"], *case.intr, H, W, 16, 0)
