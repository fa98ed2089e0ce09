"""gstex_sort_pairs_static: the pair sort for callers that cannot allocate.

Callers such as a host framework that owns every device allocation, or a
plugin that only receives a stream and raw pointers, cannot hand the sort a
workspace.  This entry point keeps its scratch in a fixed device array inside
the library.  The test calls it through the C ABI twice in a row (the second
time at its maximum size, reusing the array the first call left behind) and
requires exactly the output of the workspace-taking gstex_sort_pairs.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

MAX_ITEMS = 1 << 20  # GSTEX_SORT_STATIC_MAX_ITEMS in include/gstex_gb300.h


def _lib():
    from gstex_cuda_gb300 import _lib as L
    lib = L.lib()
    f = lib.gstex_sort_pairs_static
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p]
    return lib


def _pairs(n, seed):
    rng = np.random.default_rng(seed)
    keys = (rng.integers(0, 8160, n).astype(np.int64) << 32) | rng.integers(0, 1 << 20, n).astype(np.int64)
    vals = rng.integers(0, 1 << 30, n).astype(np.int32)
    return torch.from_numpy(keys).cuda(), torch.from_numpy(vals).cuda()


def test_static_scratch_sort_matches_workspace_sort_twice():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import gstex_cuda_gb300 as G
    lib = _lib()
    stream = torch.cuda.current_stream().cuda_stream
    for seed, n in ((1, 300_001), (2, MAX_ITEMS)):
        k, v = _pairs(n, seed)
        ref_k, ref_v = G.cuda.sort_pairs(k, v, end_bit=45)
        ko = torch.empty_like(k)
        vo = torch.empty_like(v)
        rc = lib.gstex_sort_pairs_static(n, 45, k.data_ptr(), v.data_ptr(), ko.data_ptr(), vo.data_ptr(), stream)
        assert rc == 0, lib.gstex_status_string(rc)
        torch.cuda.synchronize()
        assert torch.equal(ko, ref_k)
        assert torch.equal(vo, ref_v)


@pytest.mark.parametrize("n", [0, 1, 2049])
@pytest.mark.parametrize("end_bit", [0, 8, 64])
def test_static_scratch_sort_small_cases(n, end_bit):
    """The branches of the sort through the static entry point: no pairs, one
    pair and end_bit 0 (plain copies), 8 bits (one pass), 64 bits (eight
    passes), each equal to gstex_sort_pairs."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import gstex_cuda_gb300 as G
    lib = _lib()
    stream = torch.cuda.current_stream().cuda_stream
    k, v = _pairs(max(n, 1), 7 + n + end_bit)
    k, v = k[:n].contiguous(), v[:n].contiguous()
    ref_k, ref_v = G.cuda.sort_pairs(k, v, end_bit=end_bit)
    ko = torch.full_like(k, -1)
    vo = torch.full_like(v, -1)
    rc = lib.gstex_sort_pairs_static(n, end_bit, k.data_ptr() if n else None, v.data_ptr() if n else None,
                                     ko.data_ptr() if n else None, vo.data_ptr() if n else None, stream)
    assert rc == 0, lib.gstex_status_string(rc)
    torch.cuda.synchronize()
    assert torch.equal(ko, ref_k) and torch.equal(vo, ref_v)


def test_static_scratch_sort_rejects_sizes_beyond_its_array():
    lib = _lib()
    rc = lib.gstex_sort_pairs_static(MAX_ITEMS + 1, 45, None, None, None, None, None)
    assert rc == 2  # GSTEX_ERR_CAPACITY: more pairs than the fixed scratch holds
