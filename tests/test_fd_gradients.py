"""Central finite differences against the adjoint.

The fp64 oracle's backward (a restatement of the reference's hand-written
adjoint, csrc/texture.cu:331-760) is checked against central differences of
its own forward on a 64x64 crop with 200 Gaussians for every differentiable
parameter: step 1e-3 for colours, texels and opacities, 1e-5 for the
geometry (means, scales, rotations) and chart (uv0, umap, vmap) parameters,
whose 1e-3 differences almost always straddle a pixel crossing the
alpha >= 1/255 edge or a texel edge (fp64 keeps the smaller step exact).
The binning is held fixed (the adjoint treats it as fixed).  Samples where the loss has a kink or jump inside [x - h, x + h]
(a pair crossing alpha >= 1/255, a pixel reaching T <= 1e-4, a new depth
splat) are recognised by disagreeing one-sided slopes and not used.  Charts
span +-6 sigma so that no texture coordinate is clamped (the reference does
not differentiate the clamp), and opacities stay below the 0.99 alpha clamp.

The GPU test compares the CUDA adjoint (through the C ABI) with the same
differences.
"""
import numpy as np
import pytest
import torch

import oracle
from gpu_helpers import Case, np_, small_scene

STEP = dict(colors=1e-3, texture=1e-3, opacity=1e-3, means=1e-5, scales=1e-5, quats=1e-5, uv0=1e-5, umap=1e-5,
            vmap=1e-5)
PARAMS = ("means", "scales", "quats", "opacity", "colors", "uv0", "umap", "vmap", "texture")


def _scene():
    spec = small_scene(n=200, width=64, height=64, seed=21, f=96.0, chart=(3, 6))
    spec.umap.mul_(0.5)
    spec.vmap.mul_(0.5)
    spec.opacity.clamp_(max=0.95)
    return spec


def _weights(H, W, C, seed=3):
    g = np.random.default_rng(seed)
    return dict(img=g.standard_normal((H, W, 3)), depth=g.standard_normal((H, W)), reg=g.standard_normal((H, W)),
                alpha=g.standard_normal((H, W)), texture=g.standard_normal((H, W, C)),
                normal=g.standard_normal((H, W, 3)))


class _Problem:
    def __init__(self, spec, settings=1 << 8):
        self.case = Case(spec, colors=np.random.default_rng(5).uniform(0, 1, (spec.num_points, 3)), dev="cpu")
        self.settings = settings
        self.bg = np.array([0.1, 0.2, 0.3])
        self.b = self.case.binning_np(16)
        cam = self.case.cam
        self.w = _weights(cam.height, cam.width, spec.texture.shape[1])
        sc = self.case.scene_np
        self.base = {k: np.array(getattr(sc, k), np.float64) for k in PARAMS}

    def _scene(self, vals):
        sc = self.case.scene_np
        return oracle.Scene(means=vals["means"], scales=vals["scales"], quats=vals["quats"],
                            opacity=vals["opacity"], colors=vals["colors"], uv0=vals["uv0"], umap=vals["umap"],
                            vmap=vals["vmap"], texture_dims=sc.texture_dims, texture=vals["texture"])

    def forward(self, vals):
        return oracle.texture_forward(self._scene(vals), self.case.cam_np, self.b["gaussian_ids_sorted"],
                                      self.b["tile_bins"], 16, self.settings, self.bg, prec="f64")

    def loss(self, vals):
        f = self.forward(vals)
        return float(sum((self.w[k] * f[k]).sum() for k in self.w))

    def analytic(self):
        f = self.forward(self.base)
        w = self.w
        return oracle.texture_backward(self._scene(self.base), self.case.cam_np, self.b["gaussian_ids_sorted"],
                                       self.b["tile_bins"], 16, self.settings, self.bg, f, w["img"], w["depth"],
                                       w["reg"], w["alpha"], w["texture"], w["normal"], prec="f64")

    def central(self, name, index):
        """Central difference, or None when the one-sided slopes disagree."""
        h = STEP[name]
        vals = {k: v.copy() for k, v in self.base.items()}
        l0 = self.loss(vals)
        vals[name][index] += h
        lp = self.loss(vals)
        vals[name][index] -= 2 * h
        lm = self.loss(vals)
        sp, sm = (lp - l0) / h, (l0 - lm) / h
        # smooth at this scale: the one-sided slopes differ by O(h) relative
        if abs(sp - sm) > max(2e-4, 20 * h) * max(abs(sp), abs(sm)) + 1e-9:
            return None
        return (lp - lm) / (2 * h)


def _samples(prob, an, name, k, rng):
    """Up to k indices of `name` with a clearly non-zero analytic gradient."""
    g = an[name]
    flat = np.abs(g).reshape(-1)
    if name == "scales":  # the third scale has no gradient in the reference
        flat = flat.reshape(-1, 3).copy()
        flat[:, 2] = 0
        flat = flat.reshape(-1)
    cand = np.flatnonzero(flat > 1e-2 * flat.max())
    rng.shuffle(cand)
    return [np.unravel_index(i, g.shape) for i in cand[:k]]


@pytest.fixture(scope="module")
def problem():
    oracle.build()
    prob = _Problem(_scene())
    an = prob.analytic()
    rng = np.random.default_rng(9)
    fd = {}
    for name in PARAMS:
        idx = _samples(prob, an, name, 12, rng)
        fd[name] = [(i, prob.central(name, i)) for i in idx]
    return prob, an, fd


@pytest.mark.parametrize("name", PARAMS)
def test_oracle_adjoint_matches_central_differences(problem, name):
    prob, an, fd = problem
    used = [(i, d) for i, d in fd[name] if d is not None]
    assert len(used) >= 4, (name, len(used))
    scale = np.abs(an[name]).max()
    for i, d in used:
        a = float(an[name][i])
        assert abs(a - d) <= 1e-3 * abs(d) + 1e-5 * scale, (name, i, a, d)


@pytest.mark.gpu
def test_cuda_adjoint_matches_central_differences(problem):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import gstex_cuda_gb300 as G
    prob, an, fd = problem
    spec = _scene()
    case = Case(spec, colors=prob.case.colors_np, dev="cuda:0")
    gids = torch.from_numpy(prob.b["gaussian_ids_sorted"]).to("cuda:0")
    bins = torch.from_numpy(prob.b["tile_bins"]).to("cuda:0")
    out, bgt = case.forward_cuda(gids, bins, 16, prob.settings, prob.bg)
    ups = {k: v for k, v in prob.w.items()}
    g = case.backward_cuda(out, gids, bins, ups, 16, prob.settings, bgt)
    for name in PARAMS:
        cg = np_(g[name]).astype(np.float64)
        scale = np.abs(an[name]).max()
        for i, d in fd[name]:
            if d is None:
                continue
            assert abs(cg[i] - d) <= 1e-2 * abs(d) + 1e-3 * scale, (name, i, float(cg[i]), d)
