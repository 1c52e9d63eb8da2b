"""The denoiser's tensor-core convolution (ss_dn_conv32, tcgen05) against a
plain PyTorch fp32 reference: conv3d with circular padding on the same
BF16-rounded inputs and weights.

Products of BF16 numbers are exact in FP32, so the kernel differs from the
reference only by FP32 summation order (864 terms): relative error below
1e-4 of the output's scale for the FP32 output, one BF16 rounding (2^-8)
for the BF16 outputs.
"""
import ctypes

import numpy as np
import pytest

from test_gpu_parity import _gpu

pytestmark = pytest.mark.gpu

SHAPES = [(8, 8, 32), (6, 8, 8), (4, 4, 16)]


def _torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _conv_ref(torch, x, w, bias):
    """x (nx, ny, np, 32) fp32; w (27, 32 out, 32 in) -> periodic 3x3x3 conv + bias."""
    import torch.nn.functional as F
    nx, ny, np_, c = x.shape
    wt = w.reshape(3, 3, 3, 32, 32).permute(3, 4, 0, 1, 2).contiguous()  # [out][in][dx][dy][dp]
    xi = x.permute(3, 0, 1, 2)[None]
    y = F.conv3d(F.pad(xi, (1, 1, 1, 1, 1, 1), mode="circular"), wt, bias)
    return y[0].permute(1, 2, 3, 0).contiguous()


def _call(ss, x, w, b, ref, y, shape, mode):
    lib = ss.load_library()
    p = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None
    rc = lib.ss_dn_conv32(p(x), p(w), p(b), p(ref), p(y), *shape, mode, None)
    if rc != 0:
        raise ss.SsError(rc, ss._lib.last_error())


@pytest.mark.parametrize("shape", SHAPES, ids=["8x8x32", "6x8x8", "4x4x16"])
def test_conv32_forward_matches_torch(shape):
    ss = _gpu()
    torch = _torch()
    g = torch.Generator().manual_seed(sum(shape))
    nx, ny, np_ = shape
    x = torch.randn(nx, ny, np_, 32, generator=g).to(torch.bfloat16)
    w = (0.1 * torch.randn(27, 32, 32, generator=g)).to(torch.bfloat16).float()
    b = 0.1 * torch.randn(32, generator=g)
    want = _conv_ref(torch, x.float(), w, b)
    xd, wd, bd = x.cuda(), w.cuda(), b.cuda()
    y32 = torch.empty(nx, ny, np_, 32, device="cuda")
    _call(ss, xd, wd, bd, None, y32, shape, 1)
    got = y32.cpu()
    scale = want.abs().max().item()
    assert (got - want).abs().max().item() <= 1e-4 * scale
    y16 = torch.empty(nx, ny, np_, 32, device="cuda", dtype=torch.bfloat16)
    _call(ss, xd, wd, bd, None, y16, shape, 0)
    relu = torch.relu(want)
    assert (y16.cpu().float() - relu).abs().max().item() <= 2.0 ** -7 * scale


def test_conv32_backward_data_matches_autograd():
    ss = _gpu()
    torch = _torch()
    import torch.nn.functional as F
    shape = (8, 8, 32)
    g = torch.Generator().manual_seed(5)
    nx, ny, np_ = shape
    up = torch.randn(nx, ny, np_, 32, generator=g).to(torch.bfloat16)      # dL/dy
    ref = torch.randn(nx, ny, np_, 32, generator=g).to(torch.bfloat16)     # pre-activation of x
    w = (0.1 * torch.randn(27, 32, 32, generator=g)).to(torch.bfloat16).float()
    x = torch.zeros(nx, ny, np_, 32, requires_grad=True)
    y = _conv_ref(torch, x, w, None)
    (gx,) = torch.autograd.grad(y, x, grad_outputs=up.float())
    want = gx * (ref.float() > 0)
    out = torch.empty(nx, ny, np_, 32, device="cuda", dtype=torch.bfloat16)
    _call(ss, up.cuda(), w.cuda(), None, ref.cuda(), out, shape, 2)
    scale = want.abs().max().item()
    assert (out.cpu().float() - want).abs().max().item() <= 2.0 ** -7 * scale


def test_conv32_rejects_bad_shapes():
    ss = _gpu()
    torch = _torch()
    x = torch.zeros(5, 5, 5, 32, device="cuda", dtype=torch.bfloat16)
    w = torch.zeros(27, 32, 32, device="cuda")
    b = torch.zeros(32, device="cuda")
    with pytest.raises(ss.SsError):
        _call(ss, x, w, b, None, torch.empty_like(x), (5, 5, 5), 0)
