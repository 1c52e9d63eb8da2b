"""The denoiser's tensor-core convolution (ss_dn_conv32, tcgen05) against a
plain PyTorch fp32 reference: conv3d with circular padding on the same
BF16-rounded inputs and weights.  The tests hold activations as
[nx][nphi][ny][32] and pass them to the library in its layout
[nx][nphi][4][ny][8] (ny a multiple of 128).

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

# (nx, ny, nphi); the larger grids give every CTA several tiles, so that the
# line ring is reused along phi and the CTAs' ranges cross segments and x
SHAPES = [(1, 128, 4), (2, 128, 8), (3, 128, 5), (2, 256, 3), (24, 256, 12), (128, 128, 32)]
SHAPE_IDS = ["x".join(map(str, s)) for s in SHAPES]


def _torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _conv_ref(torch, x, w, bias):
    """x (nx, nphi, ny, 32) fp32 (the activation layout); w (27, 32 out, 32 in)
    -> periodic 3x3x3 conv + bias in the same layout (on the device of x,
    in full FP32: no TF32)."""
    import torch.nn.functional as F
    wt = w.reshape(3, 3, 3, 32, 32).permute(3, 4, 0, 1, 2).contiguous()  # [out][in][dx][dy][dp]
    xi = x.permute(3, 0, 2, 1)[None]  # (1, C, nx, ny, nphi)
    tf32 = torch.backends.cudnn.allow_tf32
    torch.backends.cudnn.allow_tf32 = False
    try:
        y = F.conv3d(F.pad(xi, (1, 1, 1, 1, 1, 1), mode="circular"), wt.to(x.device),
                     None if bias is None else bias.to(x.device))
    finally:
        torch.backends.cudnn.allow_tf32 = tf32
    return y[0].permute(1, 3, 2, 0).contiguous()


def planar(a):
    """[nx][nphi][ny][32] -> the library's activation layout [nx][nphi][4][ny][8]."""
    nx, np_, ny, _ = a.shape
    return a.reshape(nx, np_, ny, 4, 8).permute(0, 1, 3, 2, 4).contiguous()


def unplanar(a):
    nx, np_, _, ny, _ = a.shape
    return a.permute(0, 1, 3, 2, 4).reshape(nx, np_, ny, 32)


def _raw(ss, x, w, b, ref, y, shape, mode):
    lib = ss.load_library()
    p = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None
    rc = lib.ss_dn_conv32(p(x), p(w), p(b), p(ref), p(y), *shape, mode, None)
    if rc != 0:
        raise ss.SsError(rc, ss._lib.last_error())


def _call(ss, x, w, b, ref, y, shape, mode):
    """The convolution on x, ref, y given as [nx][nphi][ny][32] (y filled in place)."""
    yp = planar(y)
    _raw(ss, planar(x), w, b, None if ref is None else planar(ref), yp, shape, mode)
    y.copy_(unplanar(yp))


@pytest.mark.parametrize("shape", SHAPES, ids=SHAPE_IDS)
def test_conv32_forward_matches_torch(shape):
    ss = _gpu()
    torch = _torch()
    g = torch.Generator().manual_seed(sum(shape))
    nx, ny, np_ = shape
    x = torch.randn(nx, np_, ny, 32, generator=g).to(torch.bfloat16)
    w = (0.1 * torch.randn(27, 32, 32, generator=g)).to(torch.bfloat16).float()
    b = 0.1 * torch.randn(32, generator=g)
    want = _conv_ref(torch, x.float().cuda(), w, b).cpu()
    xd, wd, bd = x.cuda(), w.cuda(), b.cuda()
    y32 = torch.empty(nx, np_, ny, 32, device="cuda")
    _call(ss, xd, wd, bd, None, y32, shape, 1)
    got = y32.cpu()
    scale = want.abs().max().item()
    assert (got - want).abs().max().item() <= 1e-4 * scale
    y16 = torch.empty(nx, np_, ny, 32, device="cuda", dtype=torch.bfloat16)
    _call(ss, xd, wd, bd, None, y16, shape, 0)
    relu = torch.relu(want)
    assert (y16.cpu().float() - relu).abs().max().item() <= 2.0 ** -7 * scale


@pytest.mark.parametrize("shape", [(3, 128, 4), (24, 256, 12)], ids=["3x128x4", "24x256x12"])
def test_conv32_backward_data_matches_autograd(shape):
    ss = _gpu()
    torch = _torch()
    g = torch.Generator().manual_seed(5)
    nx, ny, np_ = shape
    up = torch.randn(nx, np_, ny, 32, generator=g).to(torch.bfloat16)      # dL/dy
    ref = torch.randn(nx, np_, ny, 32, generator=g).to(torch.bfloat16)     # pre-activation of x
    w = (0.1 * torch.randn(27, 32, 32, generator=g)).to(torch.bfloat16).float()
    x = torch.zeros(nx, np_, ny, 32, requires_grad=True)
    y = _conv_ref(torch, x, w, None)
    (gx,) = torch.autograd.grad(y, x, grad_outputs=up.float())
    want = gx * (ref.float() > 0)
    out = torch.empty(nx, np_, ny, 32, device="cuda", dtype=torch.bfloat16)
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
        _raw(ss, x, w, b, None, torch.empty_like(x), (5, 5, 5), 0)
    # an input that does not start on a 16-byte boundary (its bulk copies need one)
    big = torch.zeros(2 * 128 * 2 * 32 + 1, device="cuda", dtype=torch.bfloat16)
    y = torch.empty(2 * 128 * 2 * 32, device="cuda", dtype=torch.bfloat16)
    with pytest.raises(ss.SsError):
        _raw(ss, big[1:], w, b, None, y, (2, 128, 2), 0)


# ---------------------------------------------------------------- the network
def _ref_net(torch, x, P, ste=False):
    """The denoiser in torch fp32 with the kernel's BF16 roundings (the input
    of the first layer, the weights of every layer, the three activations)."""
    import torch.nn.functional as F
    from stochasticsampling_gb300.denoiser import split_params
    p = {k: torch.as_tensor(v.copy()) for k, v in split_params(P).items()}

    def bf(t):
        r = t.to(torch.bfloat16).float()
        return t + (r - t).detach() if ste else r

    def conv(a, w, b):  # a (in, nx, ny, np); w (27, out, in)
        wt = w.reshape(3, 3, 3, w.shape[1], w.shape[2]).permute(3, 4, 0, 1, 2)
        return F.conv3d(F.pad(a[None], (1, 1, 1, 1, 1, 1), mode="circular"), wt, b)[0]

    a1 = bf(torch.relu(conv(bf(x)[None], bf(p["w_in"])[:, :, None], p["b_in"])))
    a2 = bf(torch.relu(conv(a1, bf(p["w2"]), p["b2"])))
    a3 = bf(torch.relu(conv(a2, bf(p["w3"]), p["b3"])))
    return x + conv(a3, bf(p["w_out"])[:, None, :], p["b_out"])[0], p


def _net(ss, shape, seed=3, out_scale=0.05):
    from stochasticsampling_gb300.denoiser import Denoiser, split_params
    dn = Denoiser(shape, seed=seed)
    P = dn.params
    rng = np.random.default_rng(seed)
    split_params(P)["w_out"][:] = out_scale * rng.standard_normal((27, 32))
    split_params(P)["b_in"][:] = 0.05 * rng.standard_normal(32)
    dn.params = P
    return dn, P


def test_denoiser_forward_matches_torch():
    ss = _gpu()
    torch = _torch()
    shape = (4, 128, 8)
    dn, P = _net(ss, shape)
    g = torch.Generator().manual_seed(1)
    x = 1.0 + 0.3 * torch.randn(*shape, generator=g)
    y = dn.forward(x.cuda()).cpu()
    want, _ = _ref_net(torch, x, P)
    corr, wcorr = y - x, want - x
    assert (corr - wcorr).abs().max().item() <= 1e-2 * wcorr.abs().max().item()
    dn.close()


@pytest.mark.parametrize("shape,w", [((3, 128, 4), 0.0), ((3, 128, 8), 4.0), ((24, 256, 12), 0.0)],
                         ids=["mse", "mse_and_moment", "mse_24x256x12"])
def test_denoiser_gradients_match_torch(shape, w):
    """Parameter gradients and loss against torch autograd of the same
    network and loss: the mean-square error, and with the angular-moment term
    (ss_dn_set_loss) w * sum_cells (c2^2 + s2^2) / V, c2 and s2 the second
    harmonic of the residual over phi."""
    ss = _gpu()
    torch = _torch()
    from stochasticsampling_gb300.denoiser import split_params
    dn, P = _net(ss, shape, seed=4)
    dn.set_loss(w)
    g = torch.Generator().manual_seed(2)
    x = 1.0 + 0.3 * torch.randn(2, *shape, generator=g)
    t = 1.0 + 0.1 * torch.randn(2, *shape, generator=g)
    grads, loss = dn.gradients(x.cuda().contiguous(), t.cuda().contiguous())
    # autograd through the network rebuilt with leaf parameters and
    # straight-through BF16 roundings
    import torch.nn.functional as F
    P_t = {k: torch.as_tensor(v.copy(), dtype=torch.float32).requires_grad_(True)
           for k, v in split_params(P).items()}

    def bf(a):
        return a + (a.to(torch.bfloat16).float() - a).detach()

    def conv(a, w, bias):
        wt = w.reshape(3, 3, 3, w.shape[1], w.shape[2]).permute(3, 4, 0, 1, 2)
        return F.conv3d(F.pad(a[None], (1, 1, 1, 1, 1, 1), mode="circular"), wt, bias)[0]

    lt = 0.0
    for b in range(2):
        a1 = bf(torch.relu(conv(bf(x[b])[None], bf(P_t["w_in"])[:, :, None], P_t["b_in"])))
        a2 = bf(torch.relu(conv(a1, bf(P_t["w2"]), P_t["b2"])))
        a3 = bf(torch.relu(conv(a2, bf(P_t["w3"]), P_t["b3"])))
        yb = x[b] + conv(a3, bf(P_t["w_out"])[:, None, :], P_t["b_out"])[0]
        r = yb - t[b]
        phi2 = 2 * (torch.arange(shape[2], dtype=torch.float64) + 0.5) * 2 * np.pi / shape[2]
        c2 = (r * torch.cos(phi2).float()).sum(-1)
        s2 = (r * torch.sin(phi2).float()).sum(-1)
        lt = lt + ((r ** 2).mean() + w * (c2 ** 2 + s2 ** 2).sum() / r.numel()) / 2
    lt.backward()
    assert abs(loss - lt.item()) <= 1e-3 * lt.item()
    got = split_params(grads)
    for k, v in P_t.items():
        want = v.grad.numpy()
        err = np.linalg.norm(got[k] - want) / max(np.linalg.norm(want), 1e-30)
        assert err < 3e-2, (k, err)
    dn.close()


def test_denoiser_training_reduces_loss():
    ss = _gpu()
    torch = _torch()
    shape = (8, 128, 8)
    from stochasticsampling_gb300.denoiser import Denoiser
    dn = Denoiser(shape, seed=7)
    g = torch.Generator().manual_seed(3)
    X, Y, P_ = torch.meshgrid(torch.arange(8.0), torch.arange(128.0), torch.arange(8.0), indexing="ij")

    def batch(n):
        amp = 0.3 * torch.rand(n, 1, 1, 1, generator=g)
        ph = 6.283 * torch.rand(n, 1, 1, 1, generator=g)
        t = 1.0 + amp * torch.sin(6.283 * Y / 128 + ph) * torch.cos(6.283 * P_ / 8)
        x = t + 0.2 * torch.randn(n, *shape, generator=g)
        return x.cuda().contiguous(), t.cuda().contiguous()

    xv, tv = batch(4)
    l0 = dn.loss(xv, tv)
    for _ in range(150):
        dn.train(*batch(4), lr=2e-3)
    l1 = dn.loss(xv, tv)
    assert np.isfinite(l1) and l1 < 0.5 * l0, (l0, l1)
    dn.close()


def test_sample_histogram_profile():
    _gpu()
    torch = _torch()
    from stochasticsampling_gb300.denoiser import sample_histogram
    shape = (32, 32, 16)  # the sampler takes any grid
    h = sample_histogram(shape, 4_000_000, 0.05, 0.3, 0, seed=11).cpu().numpy()
    assert abs(h.mean() - 1.0) < 1e-5
    prof = h.mean(axis=(1, 2))
    s = (np.arange(32) + 0.5) / 32
    want = 1 + 0.05 * np.sin(2 * np.pi * s + 0.3) * np.sinc(1 / 32)  # bin average of the sine
    assert np.abs(prof - want).max() < 0.02  # ~4 sigma of 4e6 / 32 particles per slab
    hy = sample_histogram(shape, 4_000_000, 0.05, 0.3, 1, seed=12).cpu().numpy()
    assert np.abs(hy.mean(axis=(0, 2)) - want).max() < 0.02


def test_denoised_step_with_identity_network_matches_plain():
    """With w_out = b_out = 0 the network is the identity, so the denoised
    step contracts counts / mean * mean: the plain step up to FP32 rounding."""
    ss = _gpu()
    _torch()
    from stochasticsampling_gb300.denoiser import Denoiser, split_params
    from test_gpu_parity import _particles
    grid, box, n = (8, 128, 1, 8, 1), (2.5, 40.0, 1.0), 200_000
    params = dict(timestep=0.01, trans_diffusion=0.1, rot_diffusion=0.5, stress_active=-1.0)
    p = dict(params, number_of_particles=n, seed=5)
    dn = Denoiser((grid[0], grid[1], grid[3]), seed=1)
    P = dn.params
    split_params(P)["w_out"][:] = 0.0
    split_params(P)["b_out"][:] = 0.0
    dn.params = P
    rng = np.random.default_rng(2)
    rows = _particles(rng, n, box, True)
    a = ss.Simulation(grid=grid, box=box, params=p, quasi2d=True, mixed=True)
    b = ss.Simulation(grid=grid, box=box, params=p, quasi2d=True, mixed=True)
    a.init(rows)
    b.init(rows)
    b.set_denoiser(dn)
    for _ in range(3):
        a.do_timestep()
        b.do_timestep()
        ua, ub = a.get_flow_field(), b.get_flow_field()
        assert np.linalg.norm(ua - ub) <= 1e-5 * np.linalg.norm(ua)
    pa, pb = a.get_particles(), b.get_particles()
    assert np.mean(np.abs(pa[:, 0] - pb[:, 0]) > 1e-6) < 1e-3
    # a non-trivial network changes the contraction (a uniform output
    # weight would only shift the mean, which the flow does not see)
    split_params(P)["w_out"][:] = 0.05 * rng.standard_normal((27, 32))
    dn.params = P
    b.do_timestep()
    a.do_timestep()
    assert np.linalg.norm(a.get_flow_field() - b.get_flow_field()) > 1e-3 * np.linalg.norm(a.get_flow_field())
    b.set_denoiser(None)
    a.close()
    b.close()
    dn.close()
