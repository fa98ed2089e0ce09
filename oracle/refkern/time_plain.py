"""Times the reference's own kernels on the multi-view training workload.

TEST INFRASTRUCTURE ONLY (a measurement of the reference, not of this
package).  One step renders every camera of the 32-view, 500k-Gaussian,
16M-texel scene the way a caller of the reference does, one view after
another in fp32: SH colours, AABBs, tile counts, the host-synchronising
intersection count, emission, ``torch.sort``, tile ranges, texture_forward,
the image losses (w_img MSE + w_tex MSE + w_reg mean(reg) + w_normal normal
loss, gradients by elementwise torch), texture_backward and the SH adjoint.
All kernels on that path are the reference's, from the cubins in oracle/_ref.

    python oracle/refkern/time_plain.py [--views 32] [--steps 3] [--warmup 1]

Prints one JSON line: frames/s and the per-stage milliseconds of one step.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--views", type=int, default=32)
    ap.add_argument("--points", type=int, default=500_000)
    ap.add_argument("--texels", type=int, default=16_000_000)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=1)
    args = ap.parse_args()

    import torch
    from gstex_cuda_gb300 import synthetic
    from oracle import refkern as R

    dev = torch.device("cuda:0")
    spec = synthetic.batched(seed=3, n=args.points, texels=args.texels, views=args.views)
    t = lambda x: x.contiguous().to(dev)  # noqa: E731
    means, scales, quats, opac = t(spec.means), t(spec.scales), t(spec.quats), t(spec.opacity)
    uv0, umap, vmap, dims, tex = t(spec.uv0), t(spec.umap), t(spec.vmap), t(spec.texture_dims), t(spec.texture.float())
    sh = t(spec.sh_coeffs.float())
    N, deg = spec.num_points, spec.sh_degree
    lw = dict(img=1.0, texture=1.0, reg=100.0, normal=0.05)
    gen = torch.Generator().manual_seed(11)
    cams = spec.cameras
    tgts = [(torch.rand(c.height, c.width, 3, generator=gen).to(dev), torch.rand(c.height, c.width, 3, generator=gen)
             .to(dev)) for c in cams]
    bg = torch.zeros(3, device=dev)
    bw = 16
    stages = {}

    def mark(name, e0):
        e1 = torch.cuda.Event(enable_timing=True)
        e1.record()
        stages.setdefault(name, []).append((e0, e1))
        return e1

    def step(record):
        ev = torch.cuda.Event(enable_timing=True)
        ev.record()
        for v, cam in enumerate(cams):
            H, W = cam.height, cam.width
            vm = t(cam.viewmat)
            c2w = t(cam.c2w)
            campos = c2w[:3, 3]
            dirs = (means - campos[None]).contiguous()
            colors = R.compute_sh_forward(N, deg, deg, dirs, sh)
            ev = mark("sh", ev) if record else ev
            centers, extents = R.get_aabb_2d(means, scales, 1.0, quats, vm, cam.fx, cam.fy, cam.cx, cam.cy)
            depths = (means @ vm.T[:3, :3] + vm.T[3:, :3])[:, 2].contiguous()
            ev = mark("aabb", ev) if record else ev
            counts = R.num_tiles_hit(centers, extents, H, W, bw)
            tb = ((W + bw - 1) // bw, (H + bw - 1) // bw, 1)
            n, _, gids, bins = R.bin_and_sort(N, centers, extents, depths, counts, tb, bw)
            ev = mark("binning", ev) if record else ev
            info = (N, 1, 3)
            common = (info, dims, gids, bins, colors, opac, means, scales, 1.0, quats, uv0, umap, vmap, tex, vm, c2w,
                      cam.fx, cam.fy, cam.cx, cam.cy, 1 << 8, bg)
            img, depth, reg, otex, normal, fT, fidx, didx, reg_s = R.texture_forward(tb, (bw, bw, 1), (W, H, 1),
                                                                                     *common)
            ev = mark("forward", ev) if record else ev
            ti, tt = tgts[v]
            inv = 1.0 / (H * W)
            v_img = (2 * lw["img"] * inv / 3) * (img - ti)
            v_tex = (2 * lw["texture"] * inv / 3) * (otex - tt)
            v_reg = torch.full_like(reg, lw["reg"] * inv)
            v_normal = (2 * lw["normal"] * inv) * (normal - torch.tensor([0.0, 0.0, 1.0], device=dev))
            zeros = torch.zeros_like(reg)
            ev = mark("loss", ev) if record else ev
            g = R.texture_backward(H, W, bw, *common, fT, fidx, didx, reg_s, v_img.contiguous(), zeros,
                                   v_reg, zeros, v_tex.contiguous(), v_normal.contiguous())
            ev = mark("backward", ev) if record else ev
            R.compute_sh_backward(N, deg, deg, dirs, g[0])
            ev = mark("sh_backward", ev) if record else ev

    for _ in range(args.warmup):
        step(False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step(True)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    ms = {k: sum(a.elapsed_time(b) for a, b in v) / args.steps for k, v in stages.items()}
    print(json.dumps({"workload": f"{args.views} views, {args.points} Gaussians, {args.texels} fp32 texels",
                      "reference_kernels_plain_fp32_frames_per_s": args.views * args.steps / el,
                      "ms_per_step": 1000 * el / args.steps, "stage_ms_per_step": ms}))


if __name__ == "__main__":
    main()
