"""The two-float arithmetic of the FP64 update (csrc/f32x2.cuh), compiled for
the CPU from the same header (tests/f32x2_host.cpp) and checked against
x86 extended precision (64-bit significand): the double -> pair split,
sin / cos of a double angle and of a pair angle, atan2 of pairs, and the
increments dx, dy, dphi of the canonical quasi-2-D chain.  The GPU parity
tests pin the compiled device code against the oracle."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "stochasticsampling_gb300", "csrc")
LD = np.longdouble

pytestmark = pytest.mark.skipif(np.finfo(np.longdouble).nmant < 63 or shutil.which("g++") is None,
                                reason="needs g++ and a long double with a 64-bit significand")

TERMS = dict(sp=1, conv=2, trans=4, rot=8, ext=16, vort=32, strain=64, float_noise=128)


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = tmp_path_factory.mktemp("xf") / "libxf.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-I", CSRC,
                    os.path.join(HERE, "f32x2_host.cpp"), "-o", str(out)], check=True)
    L = ctypes.CDLL(str(out))
    for name in ("xf_split", "xf_to_double", "xf_sincos_d", "xf_sincos_f2", "xf_atan2", "xf_canon", "xf_full",
                 "xf_helpers"):
        getattr(L, name).restype = None
    return L


def _p(a):
    return np.ascontiguousarray(a).ctypes.data_as(ctypes.c_void_p)


def split(lib, d):
    d = np.ascontiguousarray(d, dtype=np.float64)
    out = np.empty(2 * d.size, np.float32)
    lib.xf_split(len(d), _p(d), _p(out))
    return out.reshape(-1, 2)


def val(pairs):
    """exact value of float pairs (rows h, l) in extended precision"""
    pairs = np.asarray(pairs)
    return pairs[..., 0].astype(LD) + pairs[..., 1].astype(LD)


def rand_pairs(rng, x):
    """pairs (h, l) of arbitrary low parts around x: h = float(x), l a float below ulp(h) / 2"""
    h = np.float32(x)
    l = (rng.random(h.shape) - 0.5) * np.spacing(np.abs(h)).astype(np.float64)
    return np.stack([h, l.astype(np.float32)], axis=-1)


def test_split_is_nearest_pair(lib):
    rng = np.random.default_rng(0)
    d = np.concatenate([rng.normal(size=2000) * 10.0 ** rng.integers(-30, 30, 2000),
                        [0.0, -0.0, 1.0, -1.5, 2.0 ** -126, 3.0 * 2.0 ** -127, 1e-300, np.pi]])
    p = split(lib, d)
    assert np.array_equal(p[:, 0], d.astype(np.float32))
    rest = d - p[:, 0].astype(np.float64)  # exact: h is within half an ulp of float of d
    big = np.abs(d) >= 2.0 ** -90
    assert np.array_equal(p[big, 1], rest[big].astype(np.float32))
    assert np.all(np.abs(p[~big, 1].astype(np.float64) - rest[~big]) <= 2.0 ** -126)
    for bad in (np.inf, -np.inf):
        h, l = split(lib, [bad])[0]
        assert h == bad and l == 0.0
    assert np.isnan(split(lib, [np.nan])[0, 0])


def test_to_double_is_exact(lib):
    """float -> double from the bits: every class of float (zero, subnormal,
    normal, inf, NaN) as the exact conversion gives it"""
    rng = np.random.default_rng(4)
    bits = np.concatenate([rng.integers(0, 2 ** 32, 200000, dtype=np.uint64).astype(np.uint32),
                           np.array([0, 0x80000000, 1, 0x807FFFFF, 0x00800000, 0x7F7FFFFF, 0x7F800000,
                                     0xFF800000, 0x7FC00001], np.uint32)])
    f = bits.view(np.float32)
    out = np.empty(f.size)
    lib.xf_to_double(len(f), _p(f), _p(out))
    with np.errstate(invalid="ignore"):  # signalling NaNs among the random bits
        ref = f.astype(np.float64)
    nan = np.isnan(ref)
    assert np.array_equal(out[~nan].view(np.uint64), ref[~nan].view(np.uint64))
    assert np.all(np.isnan(out[nan]))


def test_sincos_of_double_angles(lib):
    rng = np.random.default_rng(1)
    a = np.concatenate([rng.random(20000) * 2 * np.pi, np.arange(0, 6.3, 1 / 512.0),
                        np.arange(0, 6.3, 1 / 512.0) + 1 / 1024.0, [0.0, 1e-300, 2.0 ** -20, np.pi / 2, np.pi,
                                                                   6.2999999, 6.3, 7.0, 100.0, -0.5]])
    out = np.empty(4 * a.size)
    lib.xf_sincos_d(len(a), _p(a), _p(out))
    out = out.reshape(-1, 4)
    al = a.astype(LD)
    es = np.abs(val(out[:, 0:2]) - np.sin(al))
    ec = np.abs(val(out[:, 2:4]) - np.cos(al))
    # measured: 7.6e-15 (2^-47.1) at most, 6e-16 on average (the pair's own resolution)
    assert es.max() < 2.0 ** -46 and ec.max() < 2.0 ** -46, (float(es.max()), float(ec.max()))


def test_sincos_of_pair_angles(lib):
    rng = np.random.default_rng(2)
    r = rand_pairs(rng, np.concatenate([np.abs(rng.normal(size=20000)) * 0.4, rng.random(2000) * 6.25,
                                        [0.0, 1e-9, 1 / 512.0, 6.2499]]))
    out = np.empty(4 * len(r))
    lib.xf_sincos_f2(len(r), _p(r), _p(out))
    out = out.reshape(-1, 4)
    rl = val(r)
    es = np.abs(val(out[:, 0:2]) - np.sin(rl))
    ec = np.abs(val(out[:, 2:4]) - np.cos(rl))
    assert es.max() < 2.0 ** -46 and ec.max() < 2.0 ** -46, (float(es.max()), float(ec.max()))
    # angles beyond the table go through FP64 sincos
    far = rand_pairs(rng, np.array([6.25, 7.0, 30.0]))
    o2 = np.empty(12)
    lib.xf_sincos_f2(3, _p(far), _p(o2))
    assert np.all(np.abs(val(o2.reshape(-1, 4)[:, 0:2]) - np.sin(val(far))) < 1e-15)


def test_atan2_of_pairs(lib):
    rng = np.random.default_rng(3)
    n = 20000
    ang = np.concatenate([rng.normal(size=n) * 0.2, rng.random(n) * 2 * np.pi - np.pi])
    rad = 0.2 + rng.random(2 * n) * 2
    y, x = rand_pairs(rng, rad * np.sin(ang)), rand_pairs(rng, rad * np.cos(ang))
    out = np.empty(2 * len(y))
    lib.xf_atan2(len(y), _p(y), _p(x), _p(out))
    exact = np.arctan2(val(y), val(x))
    err = np.abs(val(out.reshape(-1, 2)) - exact)
    # about 2^-47 of the table angle a_j and of the result: an angle near 1e-3
    # reached as a_1 - eps (2^-9 - 1e-3) carries ~4e-17 absolute
    assert np.all(err <= 2.0 ** -46 * (np.abs(exact) + 2.0 ** -8)), float(err.max())
    # zero, signed zero, axes, tiny and huge vectors
    cases = [(0.0, 1.0), (-0.0, 1.0), (0.0, -1.0), (-0.0, -1.0), (1.0, 0.0), (-1.0, 0.0), (1e-30, 1.0),
             (1e30, 1e30), (3.0, -4.0), (-3.0, -4.0)]
    yy = np.array([[c[0], 0.0] for c in cases], np.float32)
    xx = np.array([[c[1], 0.0] for c in cases], np.float32)
    o = np.empty(2 * len(cases))
    lib.xf_atan2(len(cases), _p(yy), _p(xx), _p(o))
    o = o.reshape(-1, 2)
    for k, (cy, cx) in enumerate(cases):
        ref = np.arctan2(LD(np.float32(cy)), LD(np.float32(cx)))
        assert abs(val(o[k]) - ref) <= 2.0 ** -46 * abs(ref) + 1e-300, (cy, cx)
        assert np.signbit(o[k, 0]) == np.signbit(ref), (cy, cx)


def _canon_inputs(rng, n, scale_flow=1.0):
    phi = rng.random(n) * 2 * np.pi
    dt, shape_dt, reorient_dt = 0.005, 0.4 * 0.005, 0.8 * 0.005
    u0, u1 = (rng.normal(size=n) * 0.5 * scale_flow * dt for _ in range(2))
    w01 = rng.normal(size=n) * 0.3 * scale_flow * dt
    e00, e01, e11 = (rng.normal(size=n) * 0.3 * scale_flow * shape_dt for _ in range(3))
    diff = np.full(n, np.sqrt(2 * 0.1 * dt))
    ct = np.zeros((n, 8, 2), np.float32)
    for k, v in enumerate([u0, u1, w01, e00, e01, e11, diff]):
        ct[:, k] = rand_pairs(rng, v)
    xi = np.concatenate([rand_pairs(rng, rng.normal(size=n)), rand_pairs(rng, rng.normal(size=n))], axis=1)
    sa = rand_pairs(rng, np.sin(rng.random(n) * 2 * np.pi))
    rot = rand_pairs(rng, 0.1 * np.sqrt(-2 * np.log(1 - rng.random(n))))
    dtp = rand_pairs(rng, np.array([dt]))[0]
    rep = rand_pairs(rng, np.array([reorient_dt]))[0]
    return phi, ct, xi, sa, rot, dtp, rep


def _canon_exact(phi, ct, xi, sa, rot, dtp, rep, terms, float_noise):
    """the chain's increments in extended precision from the same inputs"""
    cp, sp = np.cos(phi.astype(LD)), np.sin(phi.astype(LD))
    u0, u1, w01, e00, e01, e11, diff = (val(ct[:, k]) for k in range(7))
    x0, x1, s_a = (xi[:, 0].astype(LD), xi[:, 2].astype(LD), sa[:, 0].astype(LD)) if float_noise else \
        (val(xi[:, 0:2]), val(xi[:, 2:4]), val(sa))
    dt, re, r = val(dtp), val(rep), val(rot)
    d0 = np.zeros_like(cp)
    d1 = np.zeros_like(cp)
    if terms & TERMS["sp"]:
        d0, d1 = d0 + cp * dt, d1 + sp * dt
    if terms & TERMS["conv"]:
        d0, d1 = d0 + u0, d1 + u1
    if terms & TERMS["trans"]:
        d0, d1 = d0 + x0 * diff, d1 + x1 * diff
    G = np.zeros_like(cp)
    if terms & TERMS["ext"]:
        G = G + re * cp
    if terms & TERMS["vort"]:
        G = G + w01
    if terms & TERMS["strain"]:
        f0, f1 = e00 * cp + e01 * sp, e01 * cp + e11 * sp
        G = G + (cp * f1 - sp * f0)
    C = np.ones_like(cp)
    if terms & TERMS["rot"]:
        G = G - s_a * np.sin(r)
        C = np.cos(r)
    return d0, d1, np.arctan2(G, C)


@pytest.mark.parametrize("terms", [
    TERMS["sp"] | TERMS["conv"] | TERMS["trans"] | TERMS["rot"] | TERMS["vort"],
    TERMS["sp"] | TERMS["conv"] | TERMS["trans"] | TERMS["rot"] | TERMS["vort"] | TERMS["strain"] | TERMS["ext"],
    TERMS["sp"] | TERMS["trans"] | TERMS["rot"] | TERMS["float_noise"],
    TERMS["conv"] | TERMS["vort"] | TERMS["strain"],
    TERMS["sp"] | TERMS["ext"],
    0,
], ids=["c1_terms", "all_terms", "device_noise", "flow_only", "no_noise", "none"])
def test_canonical_increments(lib, terms):
    rng = np.random.default_rng(terms)
    n = 20000
    phi, ct, xi, sa, rot, dtp, rep = _canon_inputs(rng, n)
    out = np.empty(6 * n)
    lib.xf_canon(n, _p(phi), _p(ct), _p(xi), _p(sa), _p(rot), ctypes.c_uint(terms), _p(dtp), _p(rep), _p(out))
    out = out.reshape(n, 3, 2)
    got = [val(out[:, k]) for k in range(3)]
    exact = _canon_exact(phi, ct, xi, sa, rot, dtp, rep, terms, bool(terms & TERMS["float_noise"]))
    for k, (g, e) in enumerate(zip(got, exact)):
        err = np.abs(g - e)
        # a few 2^-48 of the increment's terms: measured at most 7e-16 on dx, dy
        # (terms up to ~0.15) and 4.1e-15 on dphi (up to ~0.5, mostly from
        # sin rot), against ulps of 4.4e-16 (phi near pi) to 7.1e-15 (x near 40)
        # and the 1e-12 bar of the step
        assert np.all(err <= 2.0 ** -45 * np.maximum(np.abs(e), 0.01)), (k, float(err.max()))
        assert float(err.max()) < (1.5e-15, 1.5e-15, 8e-15)[k], (k, float(err.max()))


# ---------------------------------------------------------------- full chain
FULL = dict(sp=1, conv=2, mdd_force=4, ext=8, mdd_rot=16, vort=32, strain=64, step=128, trans=256, rot=512,
            float_noise=1024)
FULL_ALL = sum(v for k, v in FULL.items() if k != "float_noise")


def _full_inputs(rng, n, theta=None):
    phi = rng.random(n) * 2 * np.pi
    theta = np.arccos(1 - 2 * rng.random(n)) if theta is None else theta
    vals = np.zeros((n, 32))
    vals[:, 0:3] = rng.normal(size=(n, 3)) * 0.5          # u
    vals[:, 3:6] = rng.normal(size=(n, 3)) * 0.3          # W01 W02 W12
    vals[:, 6:12] = rng.normal(size=(n, 6)) * 0.3         # E
    vals[:, 12] = np.sqrt(2 * 0.002 * 0.1)                # diffusion length
    vals[:, 13:16] = rng.normal(size=(n, 3)) * 0.5        # B
    vals[:, 16:25] = rng.normal(size=(n, 9)) * 0.5        # grad B
    row = np.zeros((n, 32, 2), np.float32)
    for k in range(25):
        row[:, k] = rand_pairs(rng, vals[:, k])
    xi = np.concatenate([rand_pairs(rng, rng.normal(size=n)) for _ in range(3)], axis=1)
    alpha = rng.random(n) * 2 * np.pi
    sa, ca = rand_pairs(rng, np.sin(alpha)), rand_pairs(rng, np.cos(alpha))
    rot = rand_pairs(rng, 0.063 * np.sqrt(-2 * np.log(1 - rng.random(n))))  # sigma = sqrt(2 Dr dt), Dr 1, dt 0.002
    prm = np.concatenate([rand_pairs(rng, np.array([v]))[0] for v in (0.002, 1.0, 0.6, 0.2)])
    return phi, theta, row, xi, sa, ca, rot, prm


def _full_exact(phi, theta, row, xi, sa, ca, rot, prm, terms):
    """langevin<> (the FP64 chain) in extended precision from the same inputs:
    the new position increments and angles"""
    f = val(row.reshape(len(phi), 32, 2))
    cp, sp, ct, st = np.cos(phi.astype(LD)), np.sin(phi.astype(LD)), np.cos(theta.astype(LD)), np.sin(theta.astype(LD))
    n = [st * cp, st * sp, ct]
    if terms & FULL["float_noise"]:
        x = [xi[:, 2 * k].astype(LD) for k in range(3)]
        s_a = sa[:, 0].astype(LD)
        c_a = np.copysign(np.sqrt(1 - s_a * s_a), ca[:, 0].astype(LD))
    else:
        x = [val(xi[:, 2 * k:2 * k + 2]) for k in range(3)]
        s_a, c_a = val(sa), val(ca)
    dt, re, sh, dr = (val(prm[2 * k:2 * k + 2]) for k in range(4))
    r = val(rot)
    z = np.zeros_like(cp)
    dp, dn = [z.copy(), z.copy(), z.copy()], [z.copy(), z.copy(), z.copy()]
    if terms & FULL["sp"]:
        dp = [n[0].copy(), n[1].copy(), n[2].copy()]
    if terms & FULL["conv"]:
        dp = [dp[k] + f[:, k] for k in range(3)]
    if terms & FULL["mdd_force"]:
        g = f[:, 16:25]
        dp = [dp[a] + (g[:, 3 * a] * n[0] + g[:, 3 * a + 1] * n[1] + g[:, 3 * a + 2] * n[2]) * dr for a in range(3)]
    if terms & FULL["ext"]:
        d = n[1] * re
        dn = [dn[0] - n[0] * d, dn[1] + (re - n[1] * d), dn[2] - n[2] * d]
    if terms & FULL["mdd_rot"]:
        b = [f[:, 13 + k] for k in range(3)]
        d = n[0] * b[0] + n[1] * b[1] + n[2] * b[2]
        dn = [dn[k] + (b[k] - n[k] * d) for k in range(3)]
    if terms & FULL["vort"]:
        w01, w02, w12 = f[:, 3], f[:, 4], f[:, 5]
        fv = [w01 * n[1] + w02 * n[2], -w01 * n[0] + w12 * n[2], -w02 * n[0] - w12 * n[1]]
        dn = [dn[k] - fv[k] for k in range(3)]
    if terms & FULL["strain"]:
        e00, e01, e02, e11, e12, e22 = (f[:, 6 + k] for k in range(6))
        fs = [(e00 * n[0] + e01 * n[1] + e02 * n[2]) * sh, (e01 * n[0] + e11 * n[1] + e12 * n[2]) * sh,
              (e02 * n[0] + e12 * n[1] + e22 * n[2]) * sh]
        fn = fs[0] * n[0] + fs[1] * n[1] + fs[2] * n[2]
        dn = [dn[k] + (fs[k] - n[k] * fn) for k in range(3)]
    if terms & FULL["step"]:
        dp = [v * dt for v in dp]
        dn = [v * dt for v in dn]
    if terms & FULL["trans"]:
        dp = [dp[k] + x[k] * f[:, 12] for k in range(3)]
    if terms & FULL["rot"]:
        ax = [cp * ct * s_a - c_a * sp, c_a * cp + ct * s_a * sp, -s_a * st]
        kx = [ax[1] * n[2] - ax[2] * n[1], ax[2] * n[0] - ax[0] * n[2], ax[0] * n[1] - ax[1] * n[0]]
        dn = [dn[k] + n[k] * (np.cos(r) - 1) + kx[k] * np.sin(r) for k in range(3)]
    v = [n[k] + dn[k] for k in range(3)]
    nphi = np.arctan2(v[1], v[0])
    nth = LD(np.pi) / 2 - np.arctan2(v[2], np.sqrt(v[0] ** 2 + v[1] ** 2))
    return dp, nphi, nth


def _run_full(lib, inputs, terms):
    phi, theta, row, xi, sa, ca, rot, prm = inputs
    n = len(phi)
    out = np.empty(11 * n)
    lib.xf_full(n, _p(phi), _p(theta), _p(row), _p(xi), _p(sa), _p(ca), _p(rot), ctypes.c_uint(terms), _p(prm),
                _p(out))
    return out.reshape(n, 11)


def _wrap(a):
    """angle difference brought to (-pi, pi]"""
    return (a + LD(np.pi)) % (2 * LD(np.pi)) - LD(np.pi)


@pytest.mark.parametrize("terms", [
    FULL_ALL,
    FULL_ALL | FULL["float_noise"],
    FULL["sp"] | FULL["conv"] | FULL["ext"] | FULL["mdd_rot"] | FULL["vort"] | FULL["step"] | FULL["trans"]
    | FULL["rot"] | FULL["float_noise"],
    FULL["step"] | FULL["rot"],
    FULL["sp"] | FULL["step"],
], ids=["all_terms", "all_terms_device_noise", "c2_terms", "rotation_only", "no_rotation"])
def test_full_chain(lib, terms):
    rng = np.random.default_rng(terms)
    inputs = _full_inputs(rng, 20000)
    phi, theta = inputs[0], inputs[1]
    out = _run_full(lib, inputs, terms)
    dp, nphi, nth = _full_exact(*inputs, terms)
    for k in range(3):
        err = np.abs(val(out[:, 2 * k:2 * k + 2]) - dp[k])
        assert float(err.max()) < 2e-18 + 2.0 ** -45 * float(np.abs(dp[k]).max()), (k, float(err.max()))
    inc = out[:, 10] == 0
    gphi = np.where(inc, phi.astype(LD) + val(out[:, 6:8]), val(out[:, 6:8]))
    gth = np.where(inc, theta.astype(LD) + val(out[:, 8:10]), LD(np.pi) / 2 - val(out[:, 8:10]))
    # errors on the sphere: phi's times sin theta (phi is ill-conditioned near a
    # pole in any arithmetic), theta's as they are; the increments carry a few
    # 2^-48 of the orientation change, the direct angles near a pole 2^-46 of pi
    ephi, eth = np.abs(_wrap(gphi - nphi)) * np.sin(nth), np.abs(gth - nth)
    assert float(ephi[inc].max()) < 1e-14 and float(eth[inc].max()) < 1e-14, (float(ephi[inc].max()),
                                                                              float(eth[inc].max()))
    if np.any(~inc):
        assert float(ephi[~inc].max()) < 6e-14 and float(eth[~inc].max()) < 6e-14


def test_full_chain_near_and_at_the_poles(lib):
    rng = np.random.default_rng(7)
    theta = np.concatenate([np.zeros(50), np.full(50, np.pi), rng.random(400) * 2e-3,
                            np.pi - rng.random(400) * 2e-3])
    inputs = _full_inputs(rng, len(theta), theta=theta)
    out = _run_full(lib, inputs, FULL_ALL)
    dp, nphi, nth = _full_exact(*inputs, FULL_ALL)
    inc = out[:, 10] == 0
    assert np.any(inc) and np.any(~inc)
    gphi = np.where(inc, inputs[0].astype(LD) + val(out[:, 6:8]), val(out[:, 6:8]))
    gth = np.where(inc, inputs[1].astype(LD) + val(out[:, 8:10]), LD(np.pi) / 2 - val(out[:, 8:10]))
    assert float((np.abs(_wrap(gphi - nphi)) * np.sin(nth)).max()) < 6e-14
    assert float(np.abs(gth - nth).max()) < 6e-14


def _helpers(lib, op, a, b=None):
    b = a if b is None else b
    out = np.empty(4 * len(a))
    lib.xf_helpers(len(a), op, _p(a), _p(b), _p(out))
    return out.reshape(-1, 4)


def test_pair_sqrt_and_quotient(lib):
    rng = np.random.default_rng(8)
    x = rand_pairs(rng, np.concatenate([rng.random(20000) * 4, 10.0 ** rng.uniform(-20, 20, 2000)]))
    r = val(_helpers(lib, 0, x)[:, 0:2])
    assert np.all(np.abs(r - np.sqrt(val(x))) <= 2.0 ** -45 * np.sqrt(val(x)))
    assert np.all(_helpers(lib, 0, np.zeros((3, 2), np.float32))[:, 0:2] == 0)
    y = rand_pairs(rng, 0.1 + rng.random(len(x)) * 3)
    q = val(_helpers(lib, 1, x, y)[:, 0:2])
    exact = val(x) / val(y)
    assert np.all(np.abs(q - exact) <= 2.0 ** -45 * np.abs(exact))


def test_pair_sin_and_cos_minus_one(lib):
    rng = np.random.default_rng(9)
    r = rand_pairs(rng, np.concatenate([np.abs(rng.normal(size=20000)) * 0.1, rng.random(2000) * 6.2,
                                        [0.0, 1e-8, 1 / 512.0]]))
    o = _helpers(lib, 2, r)
    rl = val(r)
    es = np.abs(val(o[:, 0:2]) - np.sin(rl))
    # cos r - 1 without cancellation: within the table pair's own 2^-49 of C_j plus 2^-47 of the value
    ec = np.abs(val(o[:, 2:4]) - (np.cos(rl) - 1))
    assert float(es.max()) < 2.0 ** -46
    assert np.all(ec <= 2.0 ** -48 + 2.0 ** -46 * np.abs(np.cos(rl) - 1)), float(ec.max())
    far = rand_pairs(rng, np.array([6.3, 9.0]))
    of = _helpers(lib, 2, far)
    assert np.all(np.abs(val(of[:, 2:4]) - (np.cos(val(far)) - 1)) < 1e-15)


def test_axis_cosine_is_the_unit_complement_of_the_sine(lib):
    """sqrt(1 - sa^2) with the sign of the FP32 cosine, as the on-device noise
    defines the rotation axis"""
    rng = np.random.default_rng(10)
    ang = rng.random(20000) * 2 * np.pi
    sa = np.stack([np.sin(ang).astype(np.float32), np.zeros(len(ang), np.float32)], axis=-1)
    ca = np.stack([np.cos(ang).astype(np.float32), np.zeros(len(ang), np.float32)], axis=-1)
    o = val(_helpers(lib, 3, sa, ca)[:, 0:2])
    s = sa[:, 0].astype(LD)
    exact = np.copysign(np.sqrt(1 - s * s), ca[:, 0].astype(LD))
    assert np.all(np.abs(o - exact) <= 2.0 ** -45)
    assert np.all(np.signbit(o.astype(np.float64)) == np.signbit(ca[:, 0]))
