"""The real-to-complex spectral solve equals the reference's complex one.

The reference transforms each real field with a complex-to-complex FFT,
applies the k-space operators (spectral_solver.rs:133-229,
magnetic_solver.rs:71-135) on the full spectrum and keeps the real part of
the complex inverse (simulation/mod.rs:399-414).  The GPU path transforms
real to complex (half spectrum), applies the operators on the half spectrum
and transforms complex to real.  With X(k) the operator's output on the full
spectrum,

    Re(ifft(X))[n] = sum_k H(k) e^{ikn},  H(k) = (X(k) + conj(X(-k))) / 2,

which is Hermitian, so a complex-to-real transform of H restricted to the
half spectrum gives it.  X(-k) is the operator at the index -k with the
spectrum conj(sigma(k)); its wave vector is -k except along axes where k is
the (negative) Nyquist index of an even n, which is its own mirror.  Without
a Nyquist index conj(X(-k)) = X(k), so H = X there.  The imaginary part
Im(ifft(X)) is the complex-to-real transform of (X(k) - conj(X(-k))) / 2i.

Checked here in numpy for even and odd grids, 2-D and 3-D, flow and dipolar
operators, against the full complex pipeline.
"""
import numpy as np
import pytest


def kvec(n, L):
    """get_k_sampling (src/mesh/fft_helper.rs:26-51): the Nyquist index of an even n is negative."""
    b = n // 2 if n % 2 == 0 else n // 2 + 1
    i = np.arange(n)
    return np.where(i < b, i, i - n) * (2 * np.pi / L)


def flow_op(sig, k, screening, ncell):
    """u_k and G_k = i k_a u_b of the reference for stress spectra sig [3][3][...],
    wave vectors k [3][...] (fft_mean_flow_field, update_gradient)."""
    s = k[0] ** 2 + k[1] ** 2 + k[2] ** 2
    with np.errstate(divide="ignore", invalid="ignore"):
        ik2 = np.where(s == 0, 0.0, 1.0 / s)
        inrm = np.where(s == 0, 0.0, 1.0 / np.sqrt(s))
    kn = k * inrm
    sg = np.einsum("rc...,c...->r...", sig, k)
    ks = np.einsum("r...,r...->...", kn, sg)
    u = 1j * (sg - kn * ks) * (ik2 + screening) / ncell
    G = 1j * k[:, None] * u[None, :]
    return u, G


def mag_op(P, k, ncell):
    """B_k = (P_k - k^(k^ . P_k)) / N with k = 0 kept, grad B_k = i k_a B_b (magnetic_solver.rs:71-135)."""
    s = k[0] ** 2 + k[1] ** 2 + k[2] ** 2
    with np.errstate(divide="ignore", invalid="ignore"):
        inrm = np.where(s == 0, 0.0, 1.0 / np.sqrt(s))
    kn = k * inrm
    d = np.einsum("r...,r...->...", kn, P)
    B = (P - kn * d) / ncell
    return B, 1j * k[:, None] * B[None, :]


def mesh(dims, box):
    ks = [kvec(n, L) for n, L in zip(dims, box)]
    return np.array(np.meshgrid(*ks, indexing="ij"))


def half_pipeline(fields_real, dims, box, op):
    """rfftn -> operator on the half spectrum with the Hermitian part at
    Nyquist bins -> irfftn; returns (real part, imaginary part)."""
    axes = tuple(range(-3, 0))
    spec = np.fft.rfftn(fields_real, axes=axes)
    nz = dims[2]
    kfull = mesh(dims, box)
    k = kfull[..., : nz // 2 + 1]
    # mirrored wave vector: Nyquist components keep their value
    nyq = [np.zeros(d, bool) for d in dims]
    for a, d in enumerate(dims):
        if d % 2 == 0:
            nyq[a][d // 2] = True
    ny_mask = np.array(np.meshgrid(*nyq, indexing="ij"))[..., : nz // 2 + 1]
    kmir = np.where(ny_mask, k, -k)
    X = op(spec, k)
    Xm = op(np.conj(spec), kmir)
    H = [(x + np.conj(xm)) / 2 for x, xm in zip(X, Xm)]
    A = [(x - np.conj(xm)) / 2j for x, xm in zip(X, Xm)]
    real = [np.fft.irfftn(h, s=dims, axes=axes) for h in H]
    imag = [np.fft.irfftn(a, s=dims, axes=axes) for a in A]
    return real, imag, X, H


def full_pipeline(fields_real, dims, box, op):
    axes = tuple(range(-3, 0))
    spec = np.fft.fftn(fields_real.astype(complex), axes=axes)
    X = op(spec, mesh(dims, box))
    return [np.fft.ifftn(x, axes=axes) for x in X]


GRIDS = [(8, 6, 1), (7, 5, 1), (6, 5, 4), (5, 7, 3), (4, 4, 4), (9, 8, 6)]


@pytest.mark.parametrize("dims", GRIDS, ids=["x".join(map(str, g)) for g in GRIDS])
def test_half_spectrum_flow_equals_complex_solve(dims):
    rng = np.random.default_rng(sum(dims))
    box = (3.0, 2.5, 1.7)
    ncell = int(np.prod(dims))
    sig = rng.standard_normal((3, 3, *dims))
    op = lambda s, k: flow_op(s, k, 0.3, ncell)
    real, imag, X, H = half_pipeline(sig, dims, box, op)
    full = full_pipeline(sig, dims, box, op)
    for r, i, f in zip(real, imag, full):
        scale = np.abs(f).max()
        assert np.abs(r - f.real).max() <= 1e-13 * scale
        assert np.abs(i - f.imag).max() <= 1e-13 * scale
    # away from Nyquist bins the operator's output is already Hermitian: H = X bit for bit
    nyq_any = np.zeros(H[0].shape[-3:], bool)
    for a, d in enumerate(dims):
        if d % 2 == 0:
            sl = [slice(None)] * 3
            sl[a] = d // 2
            nyq_any[tuple(sl)] = True
    for x, h in zip(X, H):
        assert np.array_equal(x[..., ~nyq_any], h[..., ~nyq_any])


@pytest.mark.parametrize("dims", GRIDS, ids=["x".join(map(str, g)) for g in GRIDS])
def test_half_spectrum_dipolar_equals_complex_solve(dims):
    rng = np.random.default_rng(7 + sum(dims))
    box = (2.0, 3.0, 2.2)
    ncell = int(np.prod(dims))
    P = rng.standard_normal((3, *dims))
    op = lambda s, k: mag_op(s, k, ncell)
    real, imag, _, _ = half_pipeline(P, dims, box, op)
    full = full_pipeline(P, dims, box, op)
    for r, i, f in zip(real, imag, full):
        scale = np.abs(f).max()
        assert np.abs(r - f.real).max() <= 1e-13 * scale
        assert np.abs(i - f.imag).max() <= 1e-13 * scale


def test_odd_grids_have_no_imaginary_part():
    """Without any even axis there is no Nyquist bin: the reference's complex
    inverse is real up to round-off."""
    dims, box = (7, 5, 3), (1.0, 1.0, 1.0)
    rng = np.random.default_rng(3)
    sig = rng.standard_normal((3, 3, *dims))
    full = full_pipeline(sig, dims, box, lambda s, k: flow_op(s, k, 0.0, 105))
    for f in full:
        assert np.abs(f.imag).max() <= 1e-14 * np.abs(f.real).max()
