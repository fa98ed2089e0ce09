"""Device-side parameter activation (gstex_preprocess_forward/backward)
against the demo trainer's PyTorch preprocessing (example.py:126-143 and the
opacity sigmoid), restated here in float64 with autograd."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _torch_preprocess(rs, rq, mp, ro):
    from gstex_cuda_gb300._torch_impl import normalized_quat_to_rotmat
    scales = torch.zeros_like(rs)
    scales[:, :2] = torch.exp(rs[:, :2])
    scales[:, -1] = 1e-5 * torch.mean(scales[:, :-1], dim=-1).detach()
    q = rq / rq.norm(dim=-1, keepdim=True)
    R = normalized_quat_to_rotmat(q)
    ax1, ax2 = R[:, None, :, 0], R[:, None, :, 1]
    us, th = torch.exp(mp[:, :, None, 2]), mp[:, :, None, 3]
    umap = us * (ax1 * torch.cos(th) + ax2 * torch.sin(th))
    vmap = us * (-ax1 * torch.sin(th) + ax2 * torch.cos(th))
    return scales, q, mp[:, :, :2], umap, vmap, torch.sigmoid(ro)


@pytest.mark.parametrize("P", [1, 3])
def test_preprocess_forward_backward_match_torch(P):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from gstex_cuda_gb300.preprocess import preprocess
    g = torch.Generator().manual_seed(P)
    N = 5000
    rs = torch.log(torch.empty(N, 3).uniform_(0.005, 0.5, generator=g))
    rq = torch.randn(N, 4, generator=g) * torch.empty(N, 1).uniform_(0.3, 3.0, generator=g)
    mp = torch.cat([torch.rand(N, P, 2, generator=g), torch.randn(N, P, 1, generator=g),
                    torch.empty(N, P, 1).uniform_(0, 6.3, generator=g)], -1)
    ro = torch.randn(N, 1, generator=g)
    ref_in = [t.double().requires_grad_(True) for t in (rs, rq, mp, ro)]
    ref = _torch_preprocess(*ref_in)
    ours_in = [t.float().to(DEV).requires_grad_(True) for t in (rs, rq, mp, ro)]
    ours = preprocess(*ours_in)
    names = ("scales", "quats", "uv0", "umap", "vmap", "opacity")
    for n, a, b in zip(names, ours, ref):
        np.testing.assert_allclose(a.detach().cpu().double().numpy(), b.detach().numpy(), rtol=2e-6, atol=2e-6,
                                   err_msg=n)
    ups = [torch.randn(b.shape, generator=g, dtype=torch.float64) for b in ref]
    torch.autograd.backward(ref, ups)
    torch.autograd.backward(ours, [u.float().to(DEV) for u in ups])
    for n, a, b in zip(("raw_scales", "raw_quats", "mapping", "raw_opacity"), ours_in, ref_in):
        ga, gb = a.grad.cpu().double().numpy(), b.grad.numpy()
        np.testing.assert_allclose(ga, gb, rtol=1e-4, atol=1e-5 * np.abs(gb).max(), err_msg=n)
