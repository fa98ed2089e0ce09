"""Batched multi-view rendering on the GB300 library.

The reference renders one camera per ``texture_gaussians`` call and reads the
intersection count back to the host every time (gstex_cuda/utils.py:57-58).
``BatchRenderer`` renders a fixed set of cameras of one scene with one launch
per stage, keeps every size on the device (intersection buffers are sized by
capacity, an overflow flag reports a too-small capacity), and can capture a
whole forward + backward step in a CUDA graph.

Stages of ``step``: projection of all (view, Gaussian) pairs with SH colours,
depth keys and tile rectangles -> (side stream) splat records -> stable sort
of the pairs by depth -> inclusive scan of their tile counts in that order ->
emission of (global tile << 1 | real) keys -> stable sort by tile -> tile
ranges -> persistent forward over a global tile queue -> image losses and
their gradients -> persistent backward -> SH adjoint over views.
"""
from __future__ import annotations

import ctypes
import json
import os
from collections import Counter
from dataclasses import dataclass
from typing import List, Optional, Sequence

import torch

from . import _lib
from ._lib import check, ptr

_P = ctypes.c_void_p
_I = ctypes.c_int
_F = ctypes.c_float
_LL = ctypes.c_longlong


class ViewDesc(ctypes.Structure):
    _fields_ = [("viewmat", _F * 16), ("fx", _F), ("fy", _F), ("cx", _F), ("cy", _F), ("width", _I),
                ("height", _I)]


class BatchInputs(ctypes.Structure):
    _fields_ = [("num_points", _I), ("num_views", _I), ("block_width", _I), ("channels", _I), ("num_texels", _I),
                ("texture_dtype", _I), ("settings", _I), ("total_tiles", _I),
                ("views", _P), ("tile_view", _P), ("tile_order", _P), ("gaussian_ids_sorted", _P), ("tile_bins", _P),
                ("colors", _P), ("opacities", _P), ("means", _P), ("scales", _P), ("glob_scale", _F), ("quats", _P),
                ("uv0", _P), ("umap", _P), ("vmap", _P), ("texture_dims", _P), ("texture", _P), ("background", _P),
                ("queue", _P), ("grid", _I), ("pixels_per_thread", _I), ("records", _P), ("group_lanes", _I),
                ("batch_size", _I), ("resident_ctas", _I)]


class RawGrads(ctypes.Structure):
    _fields_ = [("raw_quats", _P), ("v_raw_scales", _P), ("v_raw_quats", _P), ("v_mapping", _P),
                ("v_raw_opacity", _P)]


_BATCH_SIGS = {
    "gstex_batch_layout": (_I, [_I, ctypes.POINTER(ViewDesc), _I, ctypes.POINTER(_I), ctypes.POINTER(_LL)]),
    "gstex_batch_views_bytes": (ctypes.c_size_t, [_I]),
    "gstex_batch_prepare": (_I, [_I, ctypes.POINTER(ViewDesc), _I, _P, _P, _P, _P]),
    "gstex_batch_project": (_I, [_I, _I, _P, _P, _P, _F, _P, _P, _I, _I, _I, _P, _P, _P]),
    "gstex_batch_project_keys": (_I, [_I, _I, _P, _P, _P, _F, _P, _P, _I, _I, _I, _P, _P, _P, _P, _P, _P]),
    "gstex_batch_project_keys_raw": (_I, [_I, _I, _P, _P, _P, _P, _P, _P, _F, _P, _I, _I, _I] + [_P] * 11),
    "gstex_batch_backward_raw": (_I, [ctypes.POINTER(BatchInputs), ctypes.POINTER(_lib.BackwardIO),
                                      ctypes.POINTER(RawGrads), _P]),
    "gstex_batch_gather_counts": (_I, [_I, _P, _P, _P, _P]),
    "gstex_batch_emit_sorted": (_I, [_I, _I, _P, _P, _P, _P, _P, _LL, _P, _P, _P, _P, _P]),
    "gstex_sort32_workspace_bytes": (ctypes.c_size_t, [_I]),
    "gstex_sort_pairs32": (_I, [_I, _P, _I, _P, _P, _P, _P, _P, ctypes.c_size_t, _P]),
    "gstex_get_tile_bin_edges32_dyn": (_I, [_I, _P, _P, _I, _I, _P, _P]),
    "gstex_batch_tile_order_workspace_bytes": (ctypes.c_size_t, [_I]),
    "gstex_batch_tile_order": (_I, [_I, _P, _P, _P, _I, _P, _P, ctypes.c_size_t, _P]),
    "gstex_batch_emit": (_I, [_I, _I, _P, _P, _P, _F, _P, _I, _P, _P, _LL, _P, _P, _P, _P, _P]),
    "gstex_sort_pairs_dyn": (_I, [_I, _P, _I, _P, _P, _P, _P, _P, ctypes.c_size_t, _P]),
    "gstex_get_tile_bin_edges_dyn": (_I, [_I, _P, _P, _I, _P, _P]),
    "gstex_batch_records_bytes": (ctypes.c_size_t, [_I, _I]),
    "gstex_batch_records_workspace_bytes": (ctypes.c_size_t, [_I, _I]),
    "gstex_batch_records": (_I, [ctypes.POINTER(BatchInputs), _P, _P, _P, ctypes.c_size_t, _P]),
    "gstex_batch_forward": (_I, [ctypes.POINTER(BatchInputs), ctypes.POINTER(_lib.ForwardOutputs), _P]),
    "gstex_batch_backward_workspace_bytes": (ctypes.c_size_t, [_I]),
    "gstex_batch_backward": (_I, [ctypes.POINTER(BatchInputs), ctypes.POINTER(_lib.BackwardIO), _P]),
    "gstex_batch_sh_backward": (_I, [_I, _I, _P, _P, _I, _P, _P, _P]),
    "gstex_batch_image_loss": (_I, [_LL, _I, _P, _I, _P, _P, _P, _P, _P, _P, _F, _F, _F, _F, _P, _P, _P, _P, _P,
                                    _P]),
}


def _L():
    L = _lib.lib()
    if not getattr(L, "_batch_sigs", False):
        for name, (res, args) in _BATCH_SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        L._batch_sigs = True
    return L


@dataclass
class Camera:
    viewmat: torch.Tensor  # [4,4] world->camera
    fx: float
    fy: float
    cx: float
    cy: float
    width: int
    height: int


@dataclass
class Scene:
    """Device tensors of one scene.  ``texture`` is float32 [T, C] or bfloat16
    [T, 4] (3 channels padded); ``sh_coeffs`` is float32 or bfloat16 [N, B, 3]."""
    means: torch.Tensor
    scales: torch.Tensor
    quats: torch.Tensor
    opacity: torch.Tensor
    sh_coeffs: torch.Tensor
    sh_degree: int
    uv0: torch.Tensor
    umap: torch.Tensor
    vmap: torch.Tensor
    texture_dims: torch.Tensor
    texture: torch.Tensor
    channels: int = 3
    glob_scale: float = 1.0


@dataclass
class RawScene:
    """A scene as a GStex trainer holds it (example.py:126-143, 155-171 of the
    reference): means [N,3]; raw_scales [N,3] log-scales (first two used);
    raw_quats [N,4] wxyz of any norm; mapping [N,1,4] (uv0 x, uv0 y, log
    uv-scale, theta); raw_opacity [N] logits; SH coefficients and texels as in
    Scene.  BatchRenderer.step_raw activates them on the device inside the
    projection and returns gradients w.r.t. these raw tensors."""
    means: torch.Tensor
    raw_scales: torch.Tensor
    raw_quats: torch.Tensor
    mapping: torch.Tensor
    raw_opacity: torch.Tensor
    sh_coeffs: torch.Tensor
    sh_degree: int
    texture_dims: torch.Tensor
    texture: torch.Tensor
    channels: int = 3
    glob_scale: float = 1.0


LOSS_WEIGHTS = dict(img=1.0, texture=1.0, reg=100.0, normal=0.05)

# Settings bits the backward reads (bilinear off, uv-gradient propagation,
# blur, NDC depth) and the value the kernels compiled for fixed settings
# serve (the library's kFixedBwdMask / kFixedBwdSettings).
FIXED_BWD_MASK = (1 << 2) | (1 << 8) | (1 << 9) | (1 << 10)
FIXED_BWD_SETTINGS = 1 << 8

# Launch knobs the autotuner chooses, and its cache: in this process, and in
# the JSON file named by GSTEX_AUTOTUNE_CACHE when that is set.
TUNED_KNOBS = ("fwd_ppt", "fwd_batch", "bwd_ppt", "bwd_group", "bwd_ctas", "bwd_batch")
_tune_cache: dict = {}


def autotune_key(sizes, num_points, channels, texmode, settings, block_width, device_name) -> str:
    """Cache key of a tuning: the multiset of view resolutions, the Gaussian
    count, the texel layout, the settings word, the tile width and the GPU."""
    mix = ",".join(f"{w}x{h}*{n}" for (h, w), n in sorted(Counter(sizes).items()))
    return (f"views={mix};N={num_points};C={channels};tex={texmode};settings={settings};bw={block_width};"
            f"gpu={device_name}")


def autotune_cache_load(path: Optional[str] = None) -> dict:
    """Tunings in the cache file (and remembered in this process)."""
    path = path if path is not None else os.environ.get("GSTEX_AUTOTUNE_CACHE")
    if path and os.path.exists(path):
        with open(path) as f:
            for k, v in json.load(f).items():
                _tune_cache.setdefault(k, v)
    return _tune_cache


def autotune_cache_store(key: str, knobs: dict, path: Optional[str] = None) -> None:
    """Remember a tuning in this process and, if a cache file is named, in it
    (read, merged and rewritten whole)."""
    _tune_cache[key] = {k: int(knobs[k]) for k in TUNED_KNOBS}
    path = path if path is not None else os.environ.get("GSTEX_AUTOTUNE_CACHE")
    if path:
        data = {}
        if os.path.exists(path):
            with open(path) as f:
                data = json.load(f)
        data[key] = _tune_cache[key]
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)


class BatchRenderer:
    """Fixed cameras, fixed scene size; reusable buffers for repeated steps."""

    def __init__(self, cameras: Sequence[Camera], num_points: int, *, channels: int = 3, texture_dtype=torch.float32,
                 block_width: int = 16, settings: int = 1 << 8, background=(0.0, 0.0, 0.0), capacity: int = 0,
                 device="cuda:0", grid: int = 0, loss_weights: Optional[dict] = None, fwd_ppt: int = 1,
                 bwd_ppt: int = 1, bwd_group: int = 8, fwd_batch: int = 0, bwd_batch: int = 0,
                 bwd_ctas: int = 0,
                 prebuilt_records: bool = True, heavy_first: bool = True, order_group: int = 4):
        self.dev = torch.device(device)
        self.N = int(num_points)
        self.V = len(cameras)
        self.bw = int(block_width)
        self.C = int(channels)
        self.settings = int(settings)
        self.texmode = 1 if texture_dtype == torch.bfloat16 else 0
        self.grid = int(grid)
        self.fwd_ppt, self.bwd_ppt = int(fwd_ppt), int(bwd_ppt)
        self.bwd_group = int(bwd_group)
        self.fwd_batch, self.bwd_batch = int(fwd_batch), int(bwd_batch)
        self.bwd_ctas = int(bwd_ctas)
        self.order_group = int(order_group)  # heaviest-first groups of order_group^2 tiles (forward)
        self.lw = dict(LOSS_WEIGHTS if loss_weights is None else loss_weights)
        L = _L()
        descs = (ViewDesc * self.V)()
        for v, cam in enumerate(cameras):
            vm = cam.viewmat.detach().double().cpu().reshape(-1).tolist()
            for k in range(16):
                descs[v].viewmat[k] = vm[k]
            descs[v].fx, descs[v].fy, descs[v].cx, descs[v].cy = cam.fx, cam.fy, cam.cx, cam.cy
            descs[v].width, descs[v].height = cam.width, cam.height
        self.descs = descs
        tt, tp = _I(0), _LL(0)
        check(L.gstex_batch_layout(self.V, descs, self.bw, ctypes.byref(tt), ctypes.byref(tp)), "batch_layout")
        self.total_tiles, self.total_pixels = tt.value, tp.value
        self.sizes = [(c.height, c.width) for c in cameras]
        dev = self.dev
        u8 = dict(dtype=torch.uint8, device=dev)
        f32 = dict(dtype=torch.float32, device=dev)
        i32 = dict(dtype=torch.int32, device=dev)
        i64 = dict(dtype=torch.int64, device=dev)
        self.views_dev = torch.empty(L.gstex_batch_views_bytes(self.V), **u8)
        self.tile_view = torch.empty(self.total_tiles, **i32)
        self.pix_offsets = torch.empty(self.V + 1, **i64)
        stream = torch.cuda.current_stream(dev).cuda_stream
        check(L.gstex_batch_prepare(self.V, descs, self.bw, ptr(self.views_dev), ptr(self.tile_view),
                                    ptr(self.pix_offsets), stream), "batch_prepare")
        self.pix_offsets_host = self.pix_offsets.cpu().tolist()
        # per-(view, Gaussian) buffers
        VN = self.V * self.N
        self.colors = torch.empty((self.V, self.N, 3), **f32)
        self.counts = torch.empty(VN, **i32)
        self.cum = torch.empty(VN, **i32)
        self.total = torch.zeros(1, **i64)
        self.scan_ws = torch.empty(L.gstex_scan_workspace_bytes(VN), **u8)
        # depth-first binning: per-pair depth keys, ids and tile rectangles,
        # their depth order, and the counts / offsets in that order
        self.dkeys = torch.empty(VN, **i32)
        self.pair_ids = torch.empty(VN, **i32)
        self.rects = torch.empty((VN, 2), **i32)
        self.dkeys_sorted = torch.empty(VN, **i32)
        self.order = torch.empty(VN, **i32)
        self.scounts = torch.empty(VN, **i32)
        self.dsort_ws = torch.empty(L.gstex_sort32_workspace_bytes(VN), **u8)
        # splat records of every (view, Gaussian), built once per step by bin()
        self.records = (torch.empty(L.gstex_batch_records_bytes(self.N, self.V), **u8) if prebuilt_records
                        else None)
        self.records_ws = (torch.empty(L.gstex_batch_records_workspace_bytes(self.N, self.V), **u8)
                           if prebuilt_records else None)
        # intersections (capacity-sized)
        self.capacity = int(capacity) if capacity else max(1 << 20, 4 * VN)
        self._alloc_isect()
        self.count = torch.zeros(1, **i64)
        self.overflow = torch.zeros(1, **i32)
        self.bins = torch.empty((self.total_tiles, 2), **i32)
        # forward queue order: heaviest tiles first (the backward keeps tile order)
        self.tile_order = torch.empty(self.total_tiles, **i32) if heavy_first else None
        self.order_ws = (torch.empty(L.gstex_batch_tile_order_workspace_bytes(self.total_tiles), **u8)
                         if heavy_first else None)
        self.queue = torch.zeros(1, **i32)
        self.bg = torch.tensor(list(background), **f32)
        # per-pixel outputs of all views
        P = self.total_pixels
        self.out = dict(img=torch.empty((P, 3), **f32), depth=torch.empty(P, **f32), reg=torch.empty(P, **f32),
                        texture=torch.empty((P, self.C), **f32), normal=torch.empty((P, 3), **f32),
                        final_T=torch.empty(P, **f32), final_idx=torch.empty(P, **i32),
                        depth_idx=torch.empty(P, **i32), reg_s=torch.empty((P, 3), **f32))
        self.ups = dict(img=torch.zeros((P, 3), **f32), texture=torch.zeros((P, self.C), **f32),
                        normal=torch.zeros((P, 3), **f32), reg=torch.zeros(P, **f32))
        self.loss = torch.zeros(1, **f32)
        self.moments = torch.empty(L.gstex_batch_backward_workspace_bytes(self.N), **u8)
        self.grads = None
        self.graph = None
        # the splat records are built on a side stream, concurrently with the
        # scan / emission / sort chain, and joined before the forward
        self.side = torch.cuda.Stream(dev)
        self.ev_fork = torch.cuda.Event()
        self.ev_join = torch.cuda.Event()

    def _alloc_isect(self):
        L = _L()
        cap = self.capacity
        dev = self.dev
        # (global tile << 1 | real) keys of the intersections and their Gaussians
        self.keys = torch.empty(cap, dtype=torch.int32, device=dev)
        self.vals = torch.empty(cap, dtype=torch.int32, device=dev)
        self.keys_sorted = torch.empty(cap, dtype=torch.int32, device=dev)
        self.gids_sorted = torch.empty(cap, dtype=torch.int32, device=dev)
        self.sort_ws = torch.empty(L.gstex_sort32_workspace_bytes(cap), dtype=torch.uint8, device=dev)

    def end_bit(self):
        return 1 + max(1, int(self.total_tiles).bit_length())

    # ------------------------------------------------------------------
    def _inputs(self, s: Scene, backward: bool = False) -> BatchInputs:
        bi = BatchInputs()
        bi.num_points, bi.num_views, bi.block_width = self.N, self.V, self.bw
        bi.channels, bi.num_texels, bi.texture_dtype, bi.settings = self.C, s.texture.shape[0], self.texmode, \
            self.settings
        bi.total_tiles = self.total_tiles
        bi.views, bi.tile_view = ptr(self.views_dev), ptr(self.tile_view)
        bi.tile_order = ptr(self.tile_order) if (self.tile_order is not None and not backward) else None
        bi.gaussian_ids_sorted, bi.tile_bins = ptr(self.gids_sorted), ptr(self.bins)
        bi.colors, bi.opacities, bi.means, bi.scales = ptr(self.colors), ptr(s.opacity), ptr(s.means), ptr(s.scales)
        bi.glob_scale = float(s.glob_scale)
        bi.quats, bi.uv0, bi.umap, bi.vmap = ptr(s.quats), ptr(s.uv0), ptr(s.umap), ptr(s.vmap)
        bi.texture_dims, bi.texture, bi.background = ptr(s.texture_dims), ptr(s.texture), ptr(self.bg)
        bi.queue, bi.grid = ptr(self.queue), self.grid
        bi.pixels_per_thread = self.bwd_ppt if backward else self.fwd_ppt
        bi.group_lanes = self.bwd_group if backward else 32
        bi.batch_size = self.bwd_batch if backward else self.fwd_batch
        bi.resident_ctas = self.bwd_ctas if backward else 0
        bi.records = ptr(self.records) if self.records is not None else None
        return bi

    def bin(self, s: Scene):
        """Projection, SH colours, splat records and binning of all views (device
        only)."""
        L = _L()
        st = torch.cuda.current_stream(self.dev).cuda_stream
        sh_dtype = 1 if s.sh_coeffs.dtype == torch.bfloat16 else 0
        check(L.gstex_batch_project_keys(self.N, self.V, ptr(self.views_dev), ptr(s.means), ptr(s.scales),
                                         float(s.glob_scale), ptr(s.quats), ptr(s.sh_coeffs), sh_dtype, s.sh_degree,
                                         self.bw, ptr(self.colors), ptr(self.counts), ptr(self.dkeys),
                                         ptr(self.pair_ids), ptr(self.rects), st), "batch_project_keys")
        self._bin_rest(s)

    def activated(self, raw: RawScene) -> Scene:
        """The device buffers that bin_raw fills with the activated parameters
        of `raw` (allocated once; the texels, SH coefficients and means are
        raw's own tensors)."""
        if getattr(self, "_act", None) is None or self._act.means is not raw.means:
            f32 = dict(dtype=torch.float32, device=self.dev)
            N = self.N
            self._act = Scene(means=raw.means, scales=torch.empty((N, 3), **f32), quats=torch.empty((N, 4), **f32),
                              opacity=torch.empty((N, 1), **f32), sh_coeffs=raw.sh_coeffs, sh_degree=raw.sh_degree,
                              uv0=torch.empty((N, 1, 2), **f32), umap=torch.empty((N, 1, 3), **f32),
                              vmap=torch.empty((N, 1, 3), **f32), texture_dims=raw.texture_dims,
                              texture=raw.texture, channels=raw.channels, glob_scale=raw.glob_scale)
        return self._act

    def bin_raw(self, raw: RawScene) -> Scene:
        """bin() from the trainer's raw parameters: the projection activates
        every Gaussian (writing the activated parameters into activated(raw))
        and the rest of binning reads those.  Returns the activated Scene."""
        L = _L()
        st = torch.cuda.current_stream(self.dev).cuda_stream
        a = self.activated(raw)
        sh_dtype = 1 if raw.sh_coeffs.dtype == torch.bfloat16 else 0
        check(L.gstex_batch_project_keys_raw(self.N, self.V, ptr(self.views_dev), ptr(raw.means),
                                             ptr(raw.raw_scales), ptr(raw.raw_quats), ptr(raw.mapping),
                                             ptr(raw.raw_opacity), float(raw.glob_scale), ptr(raw.sh_coeffs),
                                             sh_dtype, raw.sh_degree, self.bw, ptr(a.scales), ptr(a.quats),
                                             ptr(a.uv0), ptr(a.umap), ptr(a.vmap), ptr(a.opacity), ptr(self.colors),
                                             ptr(self.counts), ptr(self.dkeys), ptr(self.pair_ids), ptr(self.rects),
                                             st), "batch_project_keys_raw")
        self._bin_rest(a)
        return a

    def _bin_rest(self, s: Scene):
        L = _L()
        st = torch.cuda.current_stream(self.dev).cuda_stream
        VN = self.V * self.N
        main = torch.cuda.current_stream(self.dev)
        if self.records is not None:
            self.ev_fork.record(main)
            self.side.wait_event(self.ev_fork)
            check(L.gstex_batch_records(ctypes.byref(self._inputs(s)), ptr(self.counts), ptr(self.records),
                                        ptr(self.records_ws), self.records_ws.numel(), self.side.cuda_stream),
                  "batch_records")
            self.ev_join.record(self.side)
        # pairs in depth order, then their tiles in that order, then one stable
        # sort by (global tile << 1 | real)
        check(L.gstex_sort_pairs32(VN, None, 32, ptr(self.dkeys), ptr(self.pair_ids), ptr(self.dkeys_sorted),
                                   ptr(self.order), ptr(self.dsort_ws), self.dsort_ws.numel(), st), "sort_pairs32")
        check(L.gstex_batch_gather_counts(VN, ptr(self.order), ptr(self.counts), ptr(self.scounts), st),
              "batch_gather_counts")
        check(L.gstex_inclusive_scan_i32(VN, ptr(self.scounts), ptr(self.cum), ptr(self.total), ptr(self.scan_ws),
                                         self.scan_ws.numel(), st), "scan")
        check(L.gstex_batch_emit_sorted(self.N, self.V, ptr(self.views_dev), ptr(self.order), ptr(self.cum),
                                        ptr(self.rects), ptr(self.total), self.capacity, ptr(self.keys),
                                        ptr(self.vals), ptr(self.count), ptr(self.overflow), st), "batch_emit_sorted")
        check(L.gstex_sort_pairs32(self.capacity, ptr(self.count), self.end_bit(), ptr(self.keys), ptr(self.vals),
                                   ptr(self.keys_sorted), ptr(self.gids_sorted), ptr(self.sort_ws),
                                   self.sort_ws.numel(), st), "sort_pairs32")
        check(L.gstex_get_tile_bin_edges32_dyn(self.capacity, ptr(self.count), ptr(self.keys_sorted), 1,
                                               self.total_tiles, ptr(self.bins), st), "tile_bin_edges32_dyn")
        if self.tile_order is not None:
            check(L.gstex_batch_tile_order(self.total_tiles, ptr(self.bins), ptr(self.tile_view), ptr(self.views_dev),
                                           self.order_group, ptr(self.tile_order), ptr(self.order_ws),
                                           self.order_ws.numel(), st), "batch_tile_order")
        if self.records is not None:
            main.wait_event(self.ev_join)

    def forward(self, s: Scene):
        L = _L()
        st = torch.cuda.current_stream(self.dev).cuda_stream
        bi = self._inputs(s)
        o = self.out
        fo = _lib.ForwardOutputs(ptr(o["img"]), ptr(o["depth"]), ptr(o["reg"]), ptr(o["texture"]), ptr(o["normal"]),
                                 ptr(o["final_T"]), ptr(o["final_idx"]), ptr(o["depth_idx"]), ptr(o["reg_s"]))
        check(L.gstex_batch_forward(ctypes.byref(bi), ctypes.byref(fo), st), "batch_forward")
        return o

    def image_loss(self, tgt_img, tgt_tex):
        L = _L()
        st = torch.cuda.current_stream(self.dev).cuda_stream
        o, u, w = self.out, self.ups, self.lw
        check(L.gstex_batch_image_loss(self.total_pixels, self.V, ptr(self.pix_offsets), self.C, ptr(o["img"]),
                                       ptr(o["texture"]), ptr(o["normal"]), ptr(o["reg"]), ptr(tgt_img),
                                       ptr(tgt_tex), w["img"], w["texture"], w["reg"], w["normal"], ptr(u["img"]),
                                       ptr(u["texture"]), ptr(u["normal"]), ptr(u["reg"]), ptr(self.loss), st),
              "batch_image_loss")
        return self.loss

    def _grad_buffers(self, s: Scene):
        if self.grads is None:
            f32 = dict(dtype=torch.float32, device=self.dev)
            N = self.N
            tex_cols = 4 if self.texmode == 1 else self.C
            nb = s.sh_coeffs.shape[1]
            self.grads = dict(vcolors=torch.empty((self.V, N, 4), **f32), opacity=torch.empty(s.opacity.shape, **f32),
                              means=torch.empty((N, 3), **f32), scales=torch.empty((N, 3), **f32),
                              quats=torch.empty((N, 4), **f32), uv0=torch.empty(s.uv0.shape, **f32),
                              umap=torch.empty(s.umap.shape, **f32), vmap=torch.empty(s.vmap.shape, **f32),
                              texture=torch.zeros((s.texture.shape[0], tex_cols), **f32),
                              sh_coeffs=torch.empty((N, nb, 3), **f32))
        return self.grads

    def backward(self, s: Scene, upstream: Optional[dict] = None):
        """Gradients w.r.t. the scene given upstream pixel gradients (default:
        those written by image_loss).  Returns a dict of gradient tensors."""
        L = _L()
        st = torch.cuda.current_stream(self.dev).cuda_stream
        g = self._grad_buffers(s)
        u = self.ups if upstream is None else upstream
        g["texture"].zero_()
        o = self.out
        bio = _lib.BackwardIO(ptr(o["final_T"]), ptr(o["final_idx"]), ptr(o["depth_idx"]), ptr(o["reg_s"]),
                              ptr(u.get("img")), ptr(u.get("depth")), ptr(u.get("reg")), ptr(u.get("alpha")),
                              ptr(u.get("texture")), ptr(u.get("normal")), ptr(g["vcolors"]), ptr(g["opacity"]),
                              ptr(g["means"]), ptr(g["scales"]), ptr(g["quats"]), ptr(g["uv0"]), ptr(g["umap"]),
                              ptr(g["vmap"]), ptr(g["texture"]), ptr(self.moments), self.moments.numel())
        bi = self._inputs(s, backward=True)
        check(L.gstex_batch_backward(ctypes.byref(bi), ctypes.byref(bio), st), "batch_backward")
        check(L.gstex_batch_sh_backward(self.N, self.V, ptr(self.views_dev), ptr(s.means), s.sh_degree,
                                        ptr(g["vcolors"]), ptr(g["sh_coeffs"]), st), "batch_sh_backward")
        return g

    def step(self, s: Scene, tgt_img, tgt_tex):
        """One forward + backward pass over all views; returns the device loss."""
        self.bin(s)
        self.forward(s)
        loss = self.image_loss(tgt_img, tgt_tex)
        self.backward(s)
        return loss

    def backward_raw(self, raw: RawScene, upstream: Optional[dict] = None):
        """backward() carried on through the parameter activation: gradients
        w.r.t. raw's tensors (keys means, raw_scales, raw_quats, mapping,
        raw_opacity, texture, sh_coeffs; vcolors per view)."""
        L = _L()
        st = torch.cuda.current_stream(self.dev).cuda_stream
        a = self.activated(raw)
        g = self._grad_buffers(a)
        if "raw_scales" not in g:
            f32 = dict(dtype=torch.float32, device=self.dev)
            N = self.N
            g.update(raw_scales=torch.empty((N, 3), **f32), raw_quats=torch.empty((N, 4), **f32),
                     mapping=torch.empty((N, 1, 4), **f32), raw_opacity=torch.empty((N,), **f32))
        u = self.ups if upstream is None else upstream
        g["texture"].zero_()
        o = self.out
        bio = _lib.BackwardIO(ptr(o["final_T"]), ptr(o["final_idx"]), ptr(o["depth_idx"]), ptr(o["reg_s"]),
                              ptr(u.get("img")), ptr(u.get("depth")), ptr(u.get("reg")), ptr(u.get("alpha")),
                              ptr(u.get("texture")), ptr(u.get("normal")), ptr(g["vcolors"]), None,
                              ptr(g["means"]), None, None, None, None, None, ptr(g["texture"]), ptr(self.moments),
                              self.moments.numel())
        rg = RawGrads(ptr(raw.raw_quats), ptr(g["raw_scales"]), ptr(g["raw_quats"]), ptr(g["mapping"]),
                      ptr(g["raw_opacity"]) if raw.raw_opacity is not None else None)
        bi = self._inputs(a, backward=True)
        check(L.gstex_batch_backward_raw(ctypes.byref(bi), ctypes.byref(bio), ctypes.byref(rg), st),
              "batch_backward_raw")
        check(L.gstex_batch_sh_backward(self.N, self.V, ptr(self.views_dev), ptr(raw.means), raw.sh_degree,
                                        ptr(g["vcolors"]), ptr(g["sh_coeffs"]), st), "batch_sh_backward")
        return {k: g[k] for k in ("vcolors", "means", "raw_scales", "raw_quats", "mapping", "raw_opacity",
                                  "texture", "sh_coeffs")}

    def step_raw(self, raw: RawScene, tgt_img, tgt_tex):
        """One training step from the trainer's raw parameters: activation
        fused into the projection, forward, image losses, backward carried on
        to the raw parameters.  Returns the device loss; gradients are in
        self.raw_grads."""
        a = self.bin_raw(raw)
        self.forward(a)
        loss = self.image_loss(tgt_img, tgt_tex)
        self.raw_grads = self.backward_raw(raw)
        return loss

    # ------------------------------------------------------------------
    def tune_key(self) -> str:
        return autotune_key(self.sizes, self.N, self.C, self.texmode, self.settings, self.bw,
                            torch.cuda.get_device_name(self.dev))

    def autotune(self, s: Scene, tgt_img, tgt_tex, reps: int = 2, use_cache: bool = True) -> dict:
        """Choose pixels-per-thread and Gaussians per batch (64, 128 or one per
        thread) of the forward kernel, and pixels-per-thread, lanes per splat
        walk (32, 16, 8, 4), the resident-CTA variant and Gaussians per batch
        (48, 64, 128 or one per thread) of the backward kernel, by timing each
        candidate on this scene and these cameras (CUDA events).
        The tile width is fixed per renderer (it sets the binning): to tune
        it, build a renderer per block_width and time whole steps.
        With use_cache, a tuning of the same resolution mix, Gaussian count,
        texel layout, settings, tile width and GPU (this process, or the file
        named by GSTEX_AUTOTUNE_CACHE) is applied without timing; new tunings
        are stored there."""
        key = self.tune_key()
        if use_cache:
            hit = autotune_cache_load().get(key)
            if hit is not None:
                for k in TUNED_KNOBS:
                    setattr(self, k, int(hit[k]))
                self.graph = None
                return dict(hit, cached=True)
        stream = torch.cuda.current_stream(self.dev)
        self.bin(s)

        def timed(fn):
            fn()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                fn()
            e1.record(stream)
            torch.cuda.synchronize(self.dev)
            return e0.elapsed_time(e1) / reps

        result = {}
        best = None
        for ppt in (1, 2):
            self.fwd_ppt, self.fwd_batch = ppt, 0
            ms = timed(lambda: self.forward(s))
            result[f"forward_ppt{ppt}_ms"] = ms
            best = (ms, ppt, 0) if best is None or ms < best[0] else best
        for nb in (64, 128):
            if nb >= self.bw * self.bw:
                continue  # not below one Gaussian per thread
            self.fwd_ppt, self.fwd_batch = 1, nb
            ms = timed(lambda: self.forward(s))
            result[f"forward_ppt1_batch{nb}_ms"] = ms
            best = (ms, 1, nb) if ms < best[0] else best
        self.fwd_ppt, self.fwd_batch = best[1], best[2]
        self.forward(s)
        self.image_loss(tgt_img, tgt_tex)
        best = None
        cands = [(1, 32, 0), (2, 32, 0), (1, 16, 0), (1, 8, 0), (1, 4, 0)]
        # 8x8 tiles with bf16 RGB texels: kernels compiled for 10 resident
        # CTAs per SM (96 registers instead of 124, more warps)
        if self.bw == 8 and self.C == 3 and self.texmode == 1:
            cands += [(1, 8, 10)]
            if (self.settings & FIXED_BWD_MASK) == FIXED_BWD_SETTINGS:
                cands += [(1, 32, 10)]
        for ppt, gs, ctas in cands:
            self.bwd_ppt, self.bwd_group, self.bwd_ctas, self.bwd_batch = ppt, gs, ctas, 0
            ms = timed(lambda: self.backward(s))
            result[f"backward_ppt{ppt}_g{gs}" + (f"_ctas{ctas}" if ctas else "") + "_ms"] = ms
            best = (ms, ppt, gs, ctas, 0) if best is None or ms < best[0] else best
        for nb in (48, 64, 128):
            if nb >= self.bw * self.bw // best[1]:
                continue  # not below one Gaussian per thread
            self.bwd_ppt, self.bwd_group, self.bwd_ctas, self.bwd_batch = best[1], best[2], best[3], nb
            ms = timed(lambda: self.backward(s))
            result[f"backward_ppt{best[1]}_g{best[2]}" + (f"_ctas{best[3]}" if best[3] else "") + f"_batch{nb}_ms"] = ms
            best = (ms, best[1], best[2], best[3], nb) if ms < best[0] else best
        self.bwd_ppt, self.bwd_group, self.bwd_ctas, self.bwd_batch = best[1], best[2], best[3], best[4]
        result.update(fwd_ppt=self.fwd_ppt, fwd_batch=self.fwd_batch or "threads", bwd_ppt=self.bwd_ppt,
                      bwd_group=self.bwd_group, bwd_batch=self.bwd_batch or "threads",
                      bwd_ctas=self.bwd_ctas or "default")
        autotune_cache_store(key, {k: getattr(self, k) for k in TUNED_KNOBS})
        self.graph = None
        return result

    def capture(self, s, tgt_img, tgt_tex):
        """Capture ``step`` (``step_raw`` for a RawScene) for these (static)
        tensors in a CUDA graph."""
        step = self.step_raw if isinstance(s, RawScene) else self.step
        side = torch.cuda.Stream(self.dev)
        side.wait_stream(torch.cuda.current_stream(self.dev))
        with torch.cuda.stream(side):
            for _ in range(2):
                step(s, tgt_img, tgt_tex)
        torch.cuda.current_stream(self.dev).wait_stream(side)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            step(s, tgt_img, tgt_tex)
        self.graph = g
        return g

    def replay(self):
        self.graph.replay()
        return self.loss

    def check_capacity(self) -> bool:
        """True if the last step's intersections fit the capacity (syncs)."""
        return int(self.overflow.item()) == 0

    def intersections(self) -> int:
        return int(self.total.item())

    def grow(self, factor: float = 1.5):
        """Resize the intersection buffers after an overflow (invalidates a captured graph)."""
        need = int(self.total.item())
        self.capacity = max(int(need * factor), self.capacity + 1)
        self._alloc_isect()
        self.overflow.zero_()
        self.graph = None

    # views of the per-pixel outputs -----------------------------------
    def view_output(self, name: str, v: int):
        H, W = self.sizes[v]
        a, b = self.pix_offsets_host[v], self.pix_offsets_host[v + 1]
        t = self.out[name][a:b]
        return t.reshape(H, W, *t.shape[1:])


_SCENE_TENSORS = ("means", "scales", "quats", "opacity", "sh_coeffs", "uv0", "umap", "vmap", "texture_dims",
                  "texture")


class HostInputStepper:
    """Steps of a BatchRenderer whose scene tensors come from host memory each
    step (a trainer that keeps its parameters on the host, or streams scenes).

    Two device copies of the scene alternate: while step k computes on one,
    the inputs of step k + 1 are uploaded into the other on a copy stream, so
    the host-to-device copies overlap the compositor instead of preceding it.
    Host tensors should be pinned for the copies to run asynchronously, and
    must not change until the step that uploads them has been issued and the
    device synchronised or the next step's loss read.

        stepper = HostInputStepper(renderer, like=device_scene)
        stepper.upload(host_scene)                        # inputs of the first step
        for k in range(steps):
            loss = stepper.step(tgt_img, tgt_tex, next_host=host_scene_of(k + 1))
    """

    def __init__(self, renderer: "BatchRenderer", like: Scene):
        self.r = renderer
        self.dev = renderer.dev
        mk = lambda: Scene(**{**like.__dict__, **{k: torch.empty_like(getattr(like, k)) for k in _SCENE_TENSORS}})
        self.bufs = [mk(), mk()]
        self.copy_stream = torch.cuda.Stream(device=self.dev)
        self.ready = [torch.cuda.Event(), torch.cuda.Event()]
        self.free = [torch.cuda.Event(), torch.cuda.Event()]
        self.i = 0
        self.loaded = False

    def _upload(self, host: Scene, slot: int):
        dst = self.bufs[slot]
        with torch.cuda.stream(self.copy_stream):
            self.copy_stream.wait_event(self.free[slot])  # the step that read this buffer is done
            for k in _SCENE_TENSORS:
                getattr(dst, k).copy_(getattr(host, k), non_blocking=True)
            self.ready[slot].record(self.copy_stream)

    def upload(self, host: Scene):
        """Upload the inputs of the next step (the first one, or after a step
        taken without next_host)."""
        self._upload(host, self.i % 2)
        self.loaded = True

    def step(self, tgt_img, tgt_tex, next_host: Optional[Scene] = None):
        """One step on the uploaded inputs; next_host's upload starts at once on
        the copy stream.  Returns the loss tensor (device)."""
        if not self.loaded:
            raise RuntimeError("HostInputStepper.step: no inputs uploaded")
        cur = self.i % 2
        stream = torch.cuda.current_stream(self.dev)
        stream.wait_event(self.ready[cur])
        if next_host is not None:
            self._upload(next_host, 1 - cur)
        loss = self.r.step(self.bufs[cur], tgt_img, tgt_tex)
        self.free[cur].record(stream)
        self.i += 1
        self.loaded = next_host is not None
        return loss


def plain_step(s: Scene, cameras: Sequence[Camera], tgt_img, tgt_tex, pix_offsets, *, block_width=16,
               settings=1 << 8, background=None, loss_weights=None, timers=None):
    """The per-view path a caller of the reference API takes: for every camera,
    SH colours, AABBs, tile counts, the host-synchronising intersection count,
    binning, texture_forward, the image losses, texture_backward and the SH
    adjoint, one view after another (float32 or bfloat16 texels as given).
    Returns (loss, gradient dict); gradients are summed over views."""
    from . import cuda as C
    from .get_aabb_2d import project_points
    from .utils import bin_and_sort_gaussians, compute_cumulative_intersects
    L = _L()
    dev = s.means.device
    lw = dict(LOSS_WEIGHTS if loss_weights is None else loss_weights)
    bg = background if background is not None else torch.zeros(3, device=dev)
    N = s.means.shape[0]
    nb = s.sh_coeffs.shape[1]
    grads = None
    loss_total = torch.zeros((), device=dev)
    st = torch.cuda.current_stream(dev).cuda_stream
    bw = block_width
    # world->camera and camera->world matrices of every camera, as a caller
    # keeps them (example.py:100-109 of the reference): one host inverse, one copy
    vms = torch.stack([c.viewmat.detach().double().cpu().reshape(4, 4) for c in cameras])
    mats = torch.stack([vms, torch.linalg.inv(vms)], 1).float().to(dev)
    for v, cam in enumerate(cameras):
        H, W = cam.height, cam.width
        vm = mats[v, 0].contiguous()
        c2w = mats[v, 1].contiguous()
        campos = c2w[:3, 3]
        dirs = (s.means - campos[None]).contiguous()
        coeffs = s.sh_coeffs if s.sh_coeffs.dtype == torch.float32 else s.sh_coeffs.float()
        colors = C.compute_sh_forward(N, s.sh_degree, s.sh_degree, dirs, coeffs)
        intr = (cam.fx, cam.fy, cam.cx, cam.cy)
        _, depths = project_points(s.means, vm, intr)
        centers, extents = C.get_aabb_2d(s.means, s.scales, s.glob_scale, s.quats, vm, *intr)
        counts = C.num_tiles_hit(centers, extents, H, W, bw)
        n_isect, cum = compute_cumulative_intersects(counts)
        tb = ((W + bw - 1) // bw, (H + bw - 1) // bw, 1)
        _, _, _, gids, bins = bin_and_sort_gaussians(N, n_isect, centers, extents, depths.contiguous(), cum, tb, bw)
        info = (N, 1, s.channels)
        outs = C.texture_forward(tb, (bw, bw, 1), (W, H, 1), info, s.texture_dims, gids, bins, colors, s.opacity,
                                 s.means, s.scales, s.glob_scale, s.quats, s.uv0, s.umap, s.vmap, s.texture, vm, c2w,
                                 *intr, settings, bg)
        img, depth, reg, tex, normal, final_T, final_idx, depth_idx, reg_s = outs
        a, b = pix_offsets[v], pix_offsets[v + 1]
        P = H * W
        off = torch.tensor([0, P], dtype=torch.int64, device=dev)
        v_img = torch.empty_like(img)
        v_tex = torch.empty_like(tex)
        v_normal = torch.empty_like(normal)
        v_reg = torch.empty_like(reg)
        loss = torch.zeros(1, device=dev)
        check(L.gstex_batch_image_loss(P, 1, ptr(off), s.channels, ptr(img), ptr(tex), ptr(normal), ptr(reg),
                                       ptr(tgt_img[a:b]), ptr(tgt_tex[a:b]), lw["img"], lw["texture"], lw["reg"],
                                       lw["normal"], ptr(v_img), ptr(v_tex), ptr(v_normal), ptr(v_reg), ptr(loss), st),
              "image_loss")
        zeros = torch.zeros_like(reg)
        g = C.texture_backward(H, W, bw, info, s.texture_dims, gids, bins, colors, s.opacity, s.means, s.scales,
                               s.glob_scale, s.quats, s.uv0, s.umap, s.vmap, s.texture, vm, c2w, *intr, settings, bg,
                               final_T, final_idx, depth_idx, reg_s, v_img, zeros, v_reg, zeros, v_tex, v_normal)
        v_colors, v_opacity, v_means, v_scales, v_quats, v_uv0, v_umap, v_vmap, v_texture = g
        v_coeffs = C.compute_sh_backward(N, s.sh_degree, s.sh_degree, dirs, v_colors)
        cur = dict(opacity=v_opacity, means=v_means, scales=v_scales, quats=v_quats, uv0=v_uv0, umap=v_umap,
                   vmap=v_vmap, texture=v_texture, sh_coeffs=v_coeffs)
        if grads is None:
            grads = cur
        else:
            for k in grads:
                grads[k].add_(cur[k])
        loss_total = loss_total + loss[0]
    return loss_total, grads
