"""Generate golden vectors from the reference's own Python code.

Run where the reference checkout is present (``GSTEX_REFERENCE``, else a
directory named ``reference`` beside this repository's root):

    python tests/golden/make_golden.py

The reference package imports ``jaxtyping`` only for annotations; a
five-line stand-in is written to a temporary directory and put on the path.
Its CUDA extension is never touched: every function called here is pure
PyTorch (gstex_cuda/_torch_impl.py, gstex_cuda/get_aabb_2d.py).  The
rasteriser golden uses the oracle's restated binning as input, because the
reference's torch rasteriser takes the sorted ids and tile ranges as inputs.

Outputs (small .npz files next to this script):
  sh.npz              compute_sh_color + autograd, degrees 0..4 (float64)
  sample.npz          sample_texture + autograd (float64)
  tiles.npz           get_num_tiles_hit_2d + project_points (float32)
  raster_tiny.npz     _torch_impl.texture_forward + autograd on the 32x32
                      10-Gaussian scene (float32: the only precision it runs in)
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("GSTEX_REFERENCE", os.path.join(os.path.dirname(REPO), "reference"))


def _import_reference():
    stub = tempfile.mkdtemp()
    os.makedirs(os.path.join(stub, "jaxtyping"))
    with open(os.path.join(stub, "jaxtyping", "__init__.py"), "w") as f:
        f.write("class _S:\n    def __getitem__(self, k):\n        return object\nFloat = _S()\nInt = _S()\n")
    sys.path[:0] = [stub, REF]
    import gstex_cuda._torch_impl as T  # noqa: E402
    import gstex_cuda.get_aabb_2d as G  # noqa: E402
    return T, G


def make_sh(T):
    g = torch.Generator().manual_seed(100)
    out = {}
    for deg in range(5):
        nb = (deg + 1) ** 2
        n = 32
        d = torch.randn(n, 3, generator=g, dtype=torch.float64)
        d = d / d.norm(dim=-1, keepdim=True)
        c = torch.rand(n, nb, 3, generator=g, dtype=torch.float64).requires_grad_(True)
        v = torch.randn(n, 3, generator=g, dtype=torch.float64)
        col = T.compute_sh_color(d, c)
        (col * v).sum().backward()
        out[f"d{deg}_dirs"] = d.numpy()
        out[f"d{deg}_coeffs"] = c.detach().numpy()
        out[f"d{deg}_colors"] = col.detach().numpy()
        out[f"d{deg}_v_colors"] = v.numpy()
        out[f"d{deg}_v_coeffs"] = c.grad.numpy()
    np.savez_compressed(os.path.join(HERE, "sh.npz"), **out)


def make_sample(T):
    g = torch.Generator().manual_seed(101)
    sz, C, nq = 7, 10, 300
    dims = torch.stack([torch.randint(6, (sz,), generator=g) + 2, torch.randint(7, (sz,), generator=g) + 2,
                        torch.zeros(sz, dtype=torch.long)], -1).to(torch.int32)
    hw = dims[:, 0] * dims[:, 1]
    dims[:, 2] = (torch.cumsum(hw, 0) - hw).to(torch.int32)
    tex = torch.rand(int(hw.sum()), C, generator=g, dtype=torch.float64).requires_grad_(True)
    # uvs inside [0,1] plus a band outside it and the exact edges (clamped by the reference)
    uvs = torch.rand(nq, 2, generator=g, dtype=torch.float64) * 1.4 - 0.2
    uvs[:8] = torch.tensor([[0.0, 0.0], [1.0, 1.0], [0.0, 1.0], [1.0, 0.0], [0.5, 1.0], [1.0, 0.5],
                            [0.25, 0.0], [0.0, 0.75]], dtype=torch.float64)
    uvs.requires_grad_(True)
    ids = torch.randint(sz, (nq,), generator=g)
    qd = dims[ids]
    out = T.sample_texture(qd, tex, uvs)
    v = torch.randn(nq, C, generator=g, dtype=torch.float64)
    (out * v).sum().backward()
    np.savez_compressed(os.path.join(HERE, "sample.npz"), dims=qd.numpy(), texture=tex.detach().numpy(),
                        uvs=uvs.detach().numpy(), out=out.detach().numpy(), v_out=v.numpy(),
                        v_texture=tex.grad.numpy(), v_uvs=uvs.grad.numpy())


def make_tiles(G):
    g = torch.Generator().manual_seed(102)
    res = {}
    for name, (H, W, bw) in dict(a=(1080, 1920, 16), b=(37, 53, 16), c=(64, 64, 8)).items():
        n = 1500
        c = torch.rand(n, 2, generator=g) * torch.tensor([W * 1.4, H * 1.4]) - torch.tensor([W * 0.2, H * 0.2])
        e = torch.exp(torch.rand(n, 2, generator=g) * 8 - 4)
        # exact tile-boundary and degenerate cases
        c[:16] = torch.tensor([[16.0 * k, 16.0 * k] for k in range(16)])
        e[:16] = torch.tensor([[8.0 * k, 0.0] for k in range(16)])
        e[16:32] = 0.0
        c[32:40] = torch.tensor([[-5.0, -5.0], [W + 5.0, H + 5.0], [0.0, 0.0], [W, H], [W - 0.5, H - 0.5],
                                 [-16.0, 3.0], [3.0, -16.0], [bw * 2.0, bw * 3.0]])
        counts = G.get_num_tiles_hit_2d(c, e, H, W, bw)
        res[f"{name}_hwbw"] = np.array([H, W, bw], np.int32)
        res[f"{name}_centers"] = c.numpy()
        res[f"{name}_extents"] = e.numpy()
        res[f"{name}_counts"] = counts.to(torch.int32).numpy()
    m = torch.randn(500, 3, generator=g) * 2
    m[:, 2] += 6
    vm = torch.eye(4)
    vm[:3, 3] = torch.tensor([0.1, -0.2, 0.3])
    pix, depths = G.project_points(m, vm[:3, :], (500.0, 480.0, 320.0, 240.0))
    res.update(pp_means=m.numpy(), pp_viewmat=vm.numpy(), pp_pix=pix.numpy(), pp_depths=depths.numpy())
    np.savez_compressed(os.path.join(HERE, "tiles.npz"), **res)


def make_raster(T):
    sys.path.insert(0, REPO)
    import oracle  # noqa: E402
    from gstex_cuda_gb300 import synthetic  # noqa: E402

    spec = synthetic.tiny(seed=0)
    cam = spec.cameras[0]
    colors = (0.28209479177387814 * spec.sh_coeffs[:, 0, :]).float()
    # chart spans +-6 sigma so no contributing pixel clamps uv (the reference
    # kernel and its torch restatement differ only at clamped uv)
    umap = spec.umap * 0.5
    vmap = spec.vmap * 0.5
    c, e = oracle.get_aabb_2d(spec.means.numpy(), spec.scales.numpy(), 1.0, spec.quats.numpy(),
                              cam.viewmat.numpy(), cam.fx, cam.fy, cam.cx, cam.cy)
    depths = oracle.project_depths(spec.means.numpy(), cam.viewmat.numpy())
    nt = oracle.num_tiles_hit(c, e, cam.height, cam.width, 16)
    b = oracle.bin_and_sort(c, e, depths, nt, cam.height, cam.width, 16)
    g = torch.Generator().manual_seed(103)
    H, W = cam.height, cam.width
    ups = dict(img=torch.randn(H, W, 3, generator=g), depth=torch.randn(H, W, generator=g),
               reg=torch.randn(H, W, generator=g), alpha=torch.randn(H, W, generator=g),
               texture=torch.randn(H, W, 3, generator=g), normal=torch.randn(H, W, 3, generator=g))
    out = dict(means=spec.means.numpy(), scales=spec.scales.numpy(), quats=spec.quats.numpy(),
               opacity=spec.opacity.numpy(), colors=colors.numpy(), uv0=spec.uv0.numpy(), umap=umap.numpy(),
               vmap=vmap.numpy(), texture_dims=spec.texture_dims.numpy(), texture_vals=spec.texture.numpy(),
               viewmat=cam.viewmat.numpy(), c2w=cam.c2w.numpy(),
               intrins=np.array([cam.fx, cam.fy, cam.cx, cam.cy], np.float64),
               hw=np.array([H, W], np.int32), gids_sorted=b["gaussian_ids_sorted"], tile_bins=b["tile_bins"],
               settings=np.array([1 << 8], np.int32), background=np.zeros(3, np.float32))
    for k, v in ups.items():
        out["up_" + k] = v.numpy()
    # the reference torch rasteriser only runs in float32 (its outputs are
    # allocated as float32, gstex_cuda/_torch_impl.py:227-250)
    for tag, dtype in (("f32", torch.float32),):
        old = torch.get_default_dtype()
        torch.set_default_dtype(dtype)
        try:
            P = {k: torch.tensor(out[k], dtype=dtype, requires_grad=True)
                 for k in ("means", "scales", "quats", "opacity", "colors", "uv0", "umap", "vmap")}
            P["texture"] = torch.tensor(out["texture_vals"], dtype=dtype, requires_grad=True)
            tb = oracle.tile_bounds(H, W, 16)
            res = T.texture_forward(
                tb, (16, 16, 1), (W, H, 1), (10, 1, 3), torch.tensor(out["texture_dims"]),
                torch.tensor(b["gaussian_ids_sorted"]).long(), torch.tensor(b["tile_bins"]),
                P["colors"], P["opacity"], P["means"], P["scales"], 1.0, P["quats"], P["uv0"], P["umap"],
                P["vmap"], P["texture"], torch.tensor(out["viewmat"], dtype=dtype),
                torch.tensor(out["c2w"], dtype=dtype), cam.fx, cam.fy, cam.cx, cam.cy, 1 << 8,
                torch.zeros(3, dtype=dtype))
            img, depth, reg, tex, normal, final_T, _ = res
            alpha = 1 - final_T
            loss = ((img * ups["img"]).sum() + (depth * ups["depth"]).sum() + (reg * ups["reg"]).sum()
                    + (alpha * ups["alpha"]).sum() + (tex * ups["texture"]).sum()
                    + (normal * ups["normal"]).sum())
            loss.backward()
            for k, v in dict(img=img, depth=depth, reg=reg, alpha=alpha, texture=tex, normal=normal).items():
                out[f"{tag}_out_{k}"] = v.detach().double().numpy()
            for k, v in P.items():
                out[f"{tag}_grad_{k}"] = v.grad.double().numpy()
        finally:
            torch.set_default_dtype(old)
    np.savez_compressed(os.path.join(HERE, "raster_tiny.npz"), **out)


def main():
    T, G = _import_reference()
    make_sh(T)
    make_sample(T)
    make_tiles(G)
    make_raster(T)
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
