"""The depth-first order of the batched binning, restated in numpy on the CPU
oracle's per-view emission: sorting the (view, Gaussian) pairs by the bits of
their camera depth (stable), emitting each pair's slots in that order and
stable-sorting by (global tile << 1 | real) reproduces the reference's sort
by (tile << 32 | depth bits) with ties in emission order, view by view.  The
scenes include depth ties and clipped Gaussians whose slots keep the
reference's zero entry (tile 0, Gaussian 0).  The CUDA pipeline is checked
against the same oracle in tests/test_gpu_batch.py."""
import numpy as np
import pytest

import oracle


def _views(seed, n=300, views=3):
    rng = np.random.default_rng(seed)
    means = rng.uniform(-2, 2, (n, 3)).astype(np.float32)
    means[: n // 10, 2] = rng.uniform(-1.0, 0.005, n // 10)      # behind / at the near plane of view 0
    means[n // 10: n // 10 + 20] = means[n // 10]                # identical depths in every view
    scales = np.exp(rng.uniform(np.log(0.02), np.log(0.3), (n, 3))).astype(np.float32)
    quats = rng.normal(size=(n, 4)).astype(np.float32)
    quats /= np.linalg.norm(quats, axis=1, keepdims=True)
    cams = [(np.eye(4, dtype=np.float32), 64, 48)]
    for _ in range(views - 1):
        vm = np.eye(4, dtype=np.float32)
        vm[2, 3] = rng.uniform(3, 5)
        vm[0, 3] = rng.uniform(-0.5, 0.5)
        cams.append((vm, int(rng.choice([48, 64, 80])), int(rng.choice([32, 48, 64]))))
    return means, scales, quats, cams


@pytest.fixture(scope="module", autouse=True)
def _build():
    oracle.build()


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_depth_first_order_equals_64bit_sort(seed):
    means, scales, quats, cams = _views(seed)
    n = means.shape[0]
    ref_gids, ref_tiles, pairs = [], [], []
    toff = 0
    phantoms = 0
    for v, (vm, w, h) in enumerate(cams):
        f = float(w)
        c, e = oracle.get_aabb_2d(means, scales, 1.0, quats, vm, f, f, w / 2, h / 2)
        nt = oracle.num_tiles_hit(c, e, h, w, 16)
        d = oracle.camera_depths(means, vm)
        b = oracle.bin_and_sort(c, e, d, nt, h, w, 16)
        ref_gids.append(b["gaussian_ids_sorted"])
        ref_tiles.append((b["isect_ids_sorted"] >> 32) + toff)
        # the pair's emitted slots, in emission order (filler slots: key 0)
        cum = b["cum"]
        for i in range(n):
            lo = int(cum[i - 1]) if i else 0
            hi = int(cum[i])
            if hi == lo:
                continue
            keys, gids = b["isect_ids"][lo:hi], b["gaussian_ids"][lo:hi]
            real = keys != 0
            phantoms += int((~real).sum())
            dkey = np.float32(d[i]).view(np.uint32)
            pairs.append((dkey, v * n + i, toff + (keys >> 32), real, gids))
        toff += b["tile_bounds"][0] * b["tile_bounds"][1]
    assert phantoms > 0
    # 1. pairs by depth bits, stable in (view, Gaussian) order
    order = sorted(range(len(pairs)), key=lambda p: (int(pairs[p][0]), pairs[p][1]))
    # 2. emission in that order, 3. stable sort by (global tile << 1 | real)
    tiles = np.concatenate([pairs[p][2] for p in order])
    real = np.concatenate([pairs[p][3] for p in order])
    gids = np.concatenate([pairs[p][4] for p in order])
    # filler slots emit the view's first tile with Gaussian 0
    key = (tiles.astype(np.int64) << 1) | real.astype(np.int64)
    perm = np.argsort(key, kind="stable")
    np.testing.assert_array_equal(gids[perm], np.concatenate(ref_gids))
    np.testing.assert_array_equal(key[perm] >> 1, np.concatenate(ref_tiles))
