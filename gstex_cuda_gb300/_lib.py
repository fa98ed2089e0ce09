"""ctypes binding of libgstex_gb300.so (C ABI in include/gstex_gb300.h).

The library is loaded from the package's _build directory; if it is missing
it is compiled with nvcc first.  There is no fallback: without the library
every operator raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

import torch

from . import build as _build

_P = ctypes.c_void_p
_I = ctypes.c_int
_F = ctypes.c_float
_LOCK = threading.Lock()
_LIB = None


class RasterInputs(ctypes.Structure):
    _fields_ = [("num_points", _I), ("img_width", _I), ("img_height", _I), ("block_width", _I),
                ("channels", _I), ("num_texels", _I), ("texture_dtype", _I),
                ("texture_dims", _P), ("gaussian_ids_sorted", _P), ("tile_bins", _P), ("colors", _P),
                ("opacities", _P), ("means", _P), ("scales", _P), ("glob_scale", _F), ("quats", _P),
                ("uv0", _P), ("umap", _P), ("vmap", _P), ("texture", _P), ("viewmat", _P),
                ("fx", _F), ("fy", _F), ("cx", _F), ("cy", _F), ("settings", _I), ("background", _P),
                ("pixels_per_thread", _I), ("records", _P), ("group_lanes", _I)]


class EditIO(ctypes.Structure):
    _fields_ = [("updated_img", _P), ("updated_alpha", _P), ("depth_lower", _P), ("depth_upper", _P),
                ("num_texels", ctypes.c_longlong), ("updated_texture", _P)]


class ForwardOutputs(ctypes.Structure):
    _fields_ = [("img", _P), ("depth", _P), ("reg", _P), ("texture", _P), ("normal", _P), ("final_T", _P),
                ("final_idx", _P), ("depth_idx", _P), ("reg_s", _P)]


class BackwardIO(ctypes.Structure):
    _fields_ = [("final_T", _P), ("final_idx", _P), ("depth_idx", _P), ("reg_s", _P),
                ("v_img", _P), ("v_depth", _P), ("v_reg", _P), ("v_alpha", _P), ("v_texture", _P),
                ("v_normal", _P),
                ("v_colors", _P), ("v_opacity", _P), ("v_means", _P), ("v_scales", _P), ("v_quats", _P),
                ("v_uv0", _P), ("v_umap", _P), ("v_vmap", _P), ("v_tex_grad", _P),
                ("workspace", _P), ("workspace_bytes", ctypes.c_size_t)]


_SIGS = {
    "gstex_status_string": (ctypes.c_char_p, [_I]),
    "gstex_last_cuda_error": (ctypes.c_char_p, []),
    "gstex_version": (ctypes.c_char_p, []),
    "gstex_launch_count": (ctypes.c_ulonglong, []),
    "gstex_get_aabb_2d": (_I, [_I, _P, _P, _F, _P, _P, _F, _F, _F, _F, _P, _P, _P]),
    "gstex_num_tiles_hit": (_I, [_I, _P, _P, _I, _I, _I, _P, _P]),
    "gstex_view_records_bytes": (ctypes.c_size_t, [_I]),
    "gstex_view_records": (_I, [_P, _P, ctypes.c_size_t, _P]),
    "gstex_scan_workspace_bytes": (ctypes.c_size_t, [_I]),
    "gstex_inclusive_scan_i32": (_I, [_I, _P, _P, _P, _P, ctypes.c_size_t, _P]),
    "gstex_compute_sh_forward": (_I, [_I, _I, _I, _P, _P, _P, _P]),
    "gstex_compute_sh_backward": (_I, [_I, _I, _I, _P, _P, _P, _P]),
    "gstex_map_gaussian_to_intersects": (_I, [_I, _I, _P, _P, _P, _P, _I, _I, _I, _I, _P, _P, _P]),
    "gstex_sort_workspace_bytes": (ctypes.c_size_t, [_I]),
    "gstex_sort_pairs": (_I, [_I, _I, _P, _P, _P, _P, _P, ctypes.c_size_t, _P]),
    "gstex_get_tile_bin_edges": (_I, [_I, _P, _I, _P, _P]),
    "gstex_texture_forward": (_I, [ctypes.POINTER(RasterInputs), ctypes.POINTER(ForwardOutputs), _P]),
    "gstex_texture_edit": (_I, [ctypes.POINTER(RasterInputs), ctypes.POINTER(EditIO), _P]),
    "gstex_preprocess_forward": (_I, [_I, _I] + [_P] * 10 + [_P]),
    "gstex_preprocess_backward": (_I, [_I, _I] + [_P] * 14 + [_P]),
    "gstex_backward_workspace_bytes": (ctypes.c_size_t, [_I]),
    "gstex_texture_backward": (_I, [ctypes.POINTER(RasterInputs), ctypes.POINTER(BackwardIO), _P]),
    "gstex_texture_sample_forward": (_I, [_I, _I, _P, _P, _P, _P, _P]),
    "gstex_texture_sample_backward": (_I, [_I, _I, _P, _P, _P, _P, _P, _P, _P]),
}


def library_path() -> str:
    return _build.LIB


def lib():
    """Load (building first if needed) the CUDA library."""
    global _LIB
    if _LIB is None:
        with _LOCK:
            if _LIB is None:
                path = _build.build()
                L = ctypes.CDLL(path)
                for name, (res, args) in _SIGS.items():
                    f = getattr(L, name)
                    f.restype = res
                    f.argtypes = args
                _LIB = L
    return _LIB


class GstexError(RuntimeError):
    pass


def check(rc: int, what: str) -> None:
    if rc != 0:
        L = lib()
        msg = L.gstex_status_string(rc).decode()
        cuda = L.gstex_last_cuda_error().decode()
        raise GstexError(f"{what}: {msg}" + (f" ({cuda})" if rc == 4 and cuda else ""))


def ptr(t) -> int | None:
    if t is None:
        return None
    return t.data_ptr()


def stream_of(t: torch.Tensor):
    """Handle of the current torch stream on t's device."""
    if not t.is_cuda:
        raise GstexError("gstex_cuda_gb300 operators need CUDA tensors (no CPU implementation)")
    return torch.cuda.current_stream(t.device).cuda_stream


def require_cuda(*tensors, names=None):
    for k, t in enumerate(tensors):
        if t is None:
            continue
        if not t.is_cuda:
            n = names[k] if names else f"argument {k}"
            raise GstexError(f"{n} must be a CUDA tensor (gstex_cuda_gb300 has no CPU path)")
