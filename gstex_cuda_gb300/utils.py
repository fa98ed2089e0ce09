"""Binning and sorting of Gaussian-tile intersections.

Mirror of gstex_cuda/utils.py (reference): the same functions, arguments and
return values, on the GB300 library.  The sort is this library's stable LSD
radix sort over the key bits that can be non-zero for valid keys.
"""
from __future__ import annotations

from typing import Tuple

import torch
from torch import Tensor

from . import cuda as _C


def get_tile_bin_edges(num_intersects: int, isect_ids_sorted: Tensor, tile_bounds: Tuple[int, int, int]) -> Tensor:
    """Per-tile [start, end) ranges of sorted intersection ids
    (gstex_cuda/utils.py:11-37)."""
    return _C.get_tile_bin_edges(num_intersects, isect_ids_sorted.contiguous(), tile_bounds)


def compute_cumulative_intersects(num_tiles_hit: Tensor) -> Tuple[int, Tensor]:
    """Inclusive int32 cumsum of tiles hit and the total, read back to the host
    (gstex_cuda/utils.py:40-59)."""
    counts = num_tiles_hit.contiguous()
    if counts.dtype != torch.int32:
        counts = counts.to(torch.int32)
    cum, total = _C.inclusive_scan(counts)
    n = int(total.item())
    if n >= 2 ** 31:
        raise OverflowError(f"{n} intersections exceed the int32 range of the reference's cumsum")
    return n, cum


def map_gaussian_to_intersects(num_points: int, num_intersects: int, centers: Tensor, extents: Tensor,
                               depths: Tensor, cum_tiles_hit: Tensor, tile_bounds: Tuple[int, int, int],
                               block_size: int, wrapped: bool = False) -> Tuple[Tensor, Tensor]:
    """(tile << 32 | depth bits) keys and Gaussian ids, one per tile hit
    (gstex_cuda/utils.py:61-104)."""
    return _C.map_gaussian_to_intersects(num_points, num_intersects, centers.contiguous(), extents.contiguous(),
                                         depths.contiguous(), cum_tiles_hit.contiguous(), tile_bounds, block_size,
                                         wrapped)


def bin_and_sort_gaussians(num_points: int, num_intersects: int, centers: Tensor, extents: Tensor, depths: Tensor,
                           cum_tiles_hit: Tensor, tile_bounds: Tuple[int, int, int], block_size: int,
                           wrapped: bool = False):
    """Returns (isect_ids_unsorted, gaussian_ids_unsorted, isect_ids_sorted,
    gaussian_ids_sorted, tile_bins) (gstex_cuda/utils.py:106-161)."""
    isect_ids, gaussian_ids = map_gaussian_to_intersects(num_points, num_intersects, centers, extents, depths,
                                                         cum_tiles_hit, tile_bounds, block_size, wrapped=wrapped)
    num_tiles = int(tile_bounds[0]) * int(tile_bounds[1])
    isect_sorted, gids_sorted = _C.sort_pairs(isect_ids, gaussian_ids, _C.sort_end_bit(num_tiles))
    tile_bins = get_tile_bin_edges(num_intersects, isect_sorted, tile_bounds)
    return isect_ids, gaussian_ids, isect_sorted, gids_sorted, tile_bins
