"""Small PyTorch helpers of the reference's public surface.

These are the elementwise helpers callers use for preprocessing
(gstex_cuda/_torch_impl.py:116-147 of the reference, e.g. example.py:130).
The reference's pure-PyTorch rasteriser is not provided: rendering always
runs on the CUDA library.
"""
import torch
import torch.nn.functional as F
from torch import Tensor


def normalized_quat_to_rotmat(quat: Tensor) -> Tensor:
    """Rotation matrices (row-major [..., 3, 3]) of unit quaternions (w, x, y, z)."""
    assert quat.shape[-1] == 4, quat.shape
    w, x, y, z = torch.unbind(quat, dim=-1)
    mat = torch.stack([
        1 - 2 * (y ** 2 + z ** 2), 2 * (x * y - w * z), 2 * (x * z + w * y),
        2 * (x * y + w * z), 1 - 2 * (x ** 2 + z ** 2), 2 * (y * z - w * x),
        2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x ** 2 + y ** 2),
    ], dim=-1)
    return mat.reshape(quat.shape[:-1] + (3, 3))


def quat_to_rotmat(quat: Tensor) -> Tensor:
    assert quat.shape[-1] == 4, quat.shape
    return normalized_quat_to_rotmat(F.normalize(quat, dim=-1))


def project_pix(fxfy, p_view: Tensor, center, eps: float = 1e-6) -> Tensor:
    """Pinhole projection with the reference's 1e-6 depth offset."""
    fx, fy = fxfy
    cx, cy = center
    rw = 1.0 / (p_view[..., 2] + 1e-6)
    return torch.stack([p_view[..., 0] * rw * fx + cx, p_view[..., 1] * rw * fy + cy], dim=-1)
