"""GB300-native (sm_103a) textured 2D-Gaussian rasteriser.

Drop-in for the rasteriser path of the reference ``gstex_cuda`` package:
the same module layout and functions (``texture.texture_gaussians``,
``get_aabb_2d.{project_points, get_aabb_2d, get_num_tiles_hit_2d, ...}``,
``utils.bin_and_sort_gaussians`` and friends, ``sh.spherical_harmonics``,
``texture_sample.texture_sample``, ``texture_edit.texture_edit``,
``timer.Timer``) and the
native op surface in ``cuda``,
implemented by hand-written CUDA kernels behind the C ABI of
``include/gstex_gb300.h``.
"""
from . import cuda, get_aabb_2d, sh, texture, texture_edit, texture_sample, timer, utils  # noqa: F401
from ._lib import GstexError, lib, library_path  # noqa: F401
from .get_aabb_2d import get_aabb_2d as get_aabb_2d_fn  # noqa: F401
from .sh import spherical_harmonics  # noqa: F401
from .texture import texture_gaussians  # noqa: F401
from .texture_sample import texture_sample as texture_sample_fn  # noqa: F401

__version__ = "0.1.0"
