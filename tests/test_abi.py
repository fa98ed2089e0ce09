"""The C-ABI library builds, loads and exports every symbol its header declares
(no GPU needed: nothing is launched)."""
import os
import re

import pytest

from gstex_cuda_gb300 import _lib, build

HEADER_DIR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


def declared_functions():
    names = []
    for f in sorted(os.listdir(HEADER_DIR)):
        if f.endswith(".h"):
            src = open(os.path.join(HEADER_DIR, f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"\b(gstex_\w+)\s*\(", src)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "gstex_texture_forward" in names and "gstex_texture_backward" in names
    assert len(names) >= 15


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_status_strings_and_workspace_queries():
    L = _lib.lib()
    assert L.gstex_status_string(0) == b"ok"
    assert L.gstex_status_string(2) == b"buffer too small"
    assert L.gstex_version().decode().count(".") == 2
    assert L.gstex_sort_workspace_bytes(1000) >= 1000 * 12
    assert L.gstex_backward_workspace_bytes(10) >= 10 * 24 * 4
    assert L.gstex_scan_workspace_bytes(1) > 0
    # 224-byte record per Gaussian, then the deferred-record count and list
    assert L.gstex_view_records_bytes(1000) == 1000 * 224 + 16 + 1000 * 4
    assert L.gstex_view_records_bytes(0) == 16


def test_invalid_arguments_rejected_without_gpu():
    """Host-side validation runs before any launch."""
    L = _lib.lib()
    assert L.gstex_get_aabb_2d(-1, None, None, 1.0, None, None, 1.0, 1.0, 0.0, 0.0, None, None, None) == 1
    assert L.gstex_sort_pairs(10, 70, None, None, None, None, None, 0, None) == 1
    # SH: the degree in use above the stored degree, and degrees above 4
    assert L.gstex_compute_sh_forward(1, 2, 3, 16, 16, 16, None) == 1
    assert L.gstex_compute_sh_backward(1, 5, 5, 16, 16, 16, None) == 3
    ri = _lib.RasterInputs()
    ri.num_points, ri.img_width, ri.img_height, ri.block_width, ri.channels = 1, 8, 8, 16, 65
    import ctypes
    fo = _lib.ForwardOutputs()
    # block width 16 is fine, 65 channels is not
    ri.tile_bins = ri.viewmat = ri.background = 1
    assert L.gstex_texture_forward(ctypes.byref(ri), ctypes.byref(fo), None) == 3
    ri.channels, ri.block_width = 3, 17
    assert L.gstex_texture_forward(ctypes.byref(ri), ctypes.byref(fo), None) == 1
    # texture_edit writes five channels: any other texture_info[2] is refused
    eio = _lib.EditIO()
    ri.block_width = 16
    assert L.gstex_texture_edit(ctypes.byref(ri), ctypes.byref(eio), None) == 3
    # records: a buffer that is too small, and a misaligned one, are refused
    ri.channels = 3
    ri.colors = ri.opacities = ri.means = ri.scales = ri.quats = ri.uv0 = ri.umap = ri.vmap = 16
    ri.texture = ri.texture_dims = 16
    assert L.gstex_view_records(ctypes.byref(ri), 16, L.gstex_view_records_bytes(1) - 1, None) == 2
    assert L.gstex_view_records(ctypes.byref(ri), 8, L.gstex_view_records_bytes(1), None) == 1
    ri.records = 8
    assert L.gstex_texture_forward(ctypes.byref(ri), ctypes.byref(fo), None) == 1


def test_cpu_tensors_fail_loudly():
    torch = pytest.importorskip("torch")
    import gstex_cuda_gb300 as G
    with pytest.raises(RuntimeError):
        G.cuda.compute_sh_forward(1, 0, 0, torch.zeros(1, 3), torch.zeros(1, 1, 3))


def test_build_is_incremental():
    assert os.path.exists(build.build())
    assert not build._stale()


def test_batch_layout_and_workspace_sizes_on_host():
    """Host-only entry points of the batched path: the tile/pixel layout of a
    camera set and the sizes of the caller-provided buffers."""
    import ctypes
    from gstex_cuda_gb300 import batch as B
    L = B._L()
    descs = (B.ViewDesc * 3)()
    for d, (w, h) in zip(descs, [(1920, 1080), (512, 512), (33, 17)]):
        d.width, d.height, d.fx, d.fy = w, h, w / 2.0, w / 2.0
    tiles, pix = ctypes.c_int(0), ctypes.c_longlong(0)
    assert L.gstex_batch_layout(3, descs, 16, ctypes.byref(tiles), ctypes.byref(pix)) == 0
    assert tiles.value == 120 * 68 + 32 * 32 + 3 * 2
    assert pix.value == 1920 * 1080 + 512 * 512 + 33 * 17
    assert L.gstex_batch_layout(3, descs, 1, ctypes.byref(tiles), ctypes.byref(pix)) == 1  # block width < 2
    descs[2].width = 0
    assert L.gstex_batch_layout(3, descs, 16, ctypes.byref(tiles), ctypes.byref(pix)) == 1
    # records: 224 bytes per (view, Gaussian); sorts: room for alternate keys and values
    assert L.gstex_batch_records_bytes(1000, 4) == 1000 * 4 * 224
    assert L.gstex_sort32_workspace_bytes(1 << 20) >= (1 << 20) * 8
    assert L.gstex_sort_workspace_bytes(1 << 20) >= (1 << 20) * 12
    assert L.gstex_batch_tile_order_workspace_bytes(96464) >= 96464 * 24 + L.gstex_sort32_workspace_bytes(96464)


def test_static_scratch_sort_rejects_bad_arguments_without_gpu():
    """gstex_sort_pairs_static checks its arguments before touching the GPU:
    a negative count or end_bit outside [0, 64] is an invalid argument, more
    pairs than its fixed scratch array holds is a capacity error."""
    import ctypes
    L = _lib.lib()
    f = L.gstex_sort_pairs_static
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 5
    assert f(-1, 45, None, None, None, None, None) == 1
    assert f(10, 65, None, None, None, None, None) == 1
    assert f(10, -1, None, None, None, None, None) == 1
    assert f((1 << 20) + 1, 45, None, None, None, None, None) == 2


def test_batch_knobs_and_tile_order_rejected_without_gpu():
    """The batched entry points check the launch knobs and the queue-order
    arguments before any device work: a negative Gaussians-per-batch or
    resident-CTA count, a tile-order group outside [1, 64], a group above 1
    without the views, or a short workspace."""
    import ctypes
    from gstex_cuda_gb300 import batch as B
    L = B._L()
    bi = B.BatchInputs()
    bi.num_points, bi.num_views, bi.total_tiles, bi.block_width, bi.channels = 10, 1, 4, 8, 3
    dummy = ctypes.c_void_p(16)
    bi.views = bi.tile_view = bi.tile_bins = bi.background = bi.queue = dummy
    bi.gaussian_ids_sorted = bi.colors = bi.texture_dims = bi.opacities = bi.means = dummy
    bi.scales = bi.quats = bi.uv0 = bi.umap = bi.vmap = dummy
    fwd = L.gstex_batch_forward
    for field, value in (("batch_size", -1), ("resident_ctas", -1)):
        setattr(bi, field, value)
        assert fwd(ctypes.byref(bi), None, None) == 1, field
        setattr(bi, field, 0)
    order = L.gstex_batch_tile_order
    ws = L.gstex_batch_tile_order_workspace_bytes(100)
    assert order(100, dummy, dummy, dummy, 0, dummy, dummy, ws, None) == 1
    assert order(100, dummy, dummy, dummy, 65, dummy, dummy, ws, None) == 1
    assert order(100, dummy, None, None, 4, dummy, dummy, ws, None) == 1
    assert order(100, dummy, dummy, dummy, 4, dummy, dummy, ws - 1, None) == 2
    assert order(0, None, None, None, 4, None, None, 0, None) == 0


def test_autotune_cache_key_and_file(tmp_path):
    """The autotuner's cache key is the multiset of view resolutions (order
    free), the Gaussian count, texel layout, settings, tile width and GPU;
    tunings round-trip through the cache file."""
    from gstex_cuda_gb300 import batch as B
    k1 = B.autotune_key([(1080, 1920), (512, 512), (1080, 1920)], 500000, 3, 1, 256, 8, "GB300")
    k2 = B.autotune_key([(512, 512), (1080, 1920), (1080, 1920)], 500000, 3, 1, 256, 8, "GB300")
    assert k1 == k2 and "1920x1080*2" in k1 and "512x512*1" in k1
    assert B.autotune_key([(1080, 1920)], 500000, 3, 1, 256, 16, "GB300") != \
        B.autotune_key([(1080, 1920)], 500000, 3, 1, 256, 8, "GB300")
    path = str(tmp_path / "tune.json")
    knobs = dict(fwd_ppt=1, fwd_batch=0, bwd_ppt=1, bwd_group=8, bwd_ctas=10, bwd_batch=0, extra=5)
    B.autotune_cache_store(k1, knobs, path=path)
    B._tune_cache.clear()
    got = B.autotune_cache_load(path)
    assert got[k1] == {k: knobs[k] for k in B.TUNED_KNOBS}
    B._tune_cache.clear()
