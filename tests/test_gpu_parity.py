"""Parity of the CUDA timestep (through the C ABI) with the CPU oracle.

Bars: integer histograms and the sanitised particle state bit-exact; fields,
velocities and positions within 1e-12 norm-wise relative error of the FP64
oracle (||gpu - oracle||_2 / ||oracle||_2), the tolerance the reference's
FP64 path is held to.  Per-step comparisons start from identical state and
identical noise; trajectories over several steps are compared with the noise
the GPU drew (ss_noise) fed to the oracle.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_l2

pytestmark = pytest.mark.gpu

PI = np.pi
TWOPI = 2 * PI
TOL = 1e-12


def _gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import stochasticsampling_gb300 as ss
    return ss


# configurations: (name, grid, box, params, n, quasi2d)
C0 = ("c0_2d", (32, 32, 1, 16, 1), (10.0, 10.0, 1.0),
      dict(timestep=0.01, trans_diffusion=0.1, rot_diffusion=0.5, stress_active=-1.0), 100_000, True)
SMALL3D = ("small_3d_all_terms", (6, 5, 4, 6, 4), (3.0, 2.5, 2.0),
           dict(timestep=0.01, trans_diffusion=0.3, rot_diffusion=0.7, stress_active=-1.3, stress_magnetic=0.4,
                shape=0.6, magnetic_drag=0.2, hydro_screening=0.1, volume_exclusion=0.05,
                magnetic_reorientation=0.8, magnetic_dipole_dipole=0.5), 20_000, False)
ODD3D = ("odd_3d_magnetic", (9, 7, 5, 5, 3), (4.5, 3.5, 2.5),
         dict(timestep=0.002, trans_diffusion=0.2, rot_diffusion=1.0, stress_active=-2.0,
              magnetic_reorientation=1.0, magnetic_dipole_dipole=0.5), 30_000, False)
EVEN2D = ("even_2d_screened", (16, 12, 1, 8, 1), (8.0, 6.0, 1.0),
          dict(timestep=0.005, trans_diffusion=0.1, rot_diffusion=1.0, stress_active=-2.0, hydro_screening=0.3,
               shape=0.4, volume_exclusion=0.1), 40_000, True)
CONFIGS = [C0, SMALL3D, ODD3D, EVEN2D]


def _particles(rng, n, box, quasi2d):
    th = np.full(n, PI / 2) if quasi2d else np.arccos(1 - 2 * rng.random(n))
    z = np.zeros(n) if quasi2d else box[2] * rng.random(n)
    return np.column_stack([box[0] * rng.random(n), box[1] * rng.random(n), z, TWOPI * rng.random(n), th])


def _noise(rng, n, params):
    sigma = np.sqrt(2 * params.get("rot_diffusion", 0.0) * params.get("timestep", 0.0))
    return np.column_stack([rng.standard_normal((n, 3)), TWOPI * rng.random(n),
                            sigma * np.sqrt(-2 * np.log(1 - rng.random(n)))])


def _pair(oracle, cfg, seed=1, nthreads=None, **gpu_kw):
    ss = _gpu()
    name, grid, box, params, n, q2d = cfg
    p = dict(params, number_of_particles=n, seed=seed)
    g = ss.Simulation(grid=grid, box=box, params=p, quasi2d=q2d, **gpu_kw)
    s = oracle.make_settings(grid, box, timestep=p.get("timestep", 0.0), trans_diff=p.get("trans_diffusion", 0.0),
                             rot_diff=p.get("rot_diffusion", 0.0), active=p.get("stress_active", 0.0),
                             magnetic=p.get("stress_magnetic", 0.0), shape=p.get("shape", 0.0),
                             magnetic_drag=p.get("magnetic_drag", 0.0),
                             hydro_screening=p.get("hydro_screening", 0.0),
                             volume_exclusion=p.get("volume_exclusion", 0.0),
                             magnetic_reorientation=p.get("magnetic_reorientation", 0.0),
                             magnetic_dipole_dipole=p.get("magnetic_dipole_dipole", 0.0), quasi2d=q2d, seed=seed)
    o = oracle.Simulation(s, n, nthreads=nthreads or min(16, os.cpu_count() or 1))
    return g, o, s


# --------------------------------------------------------- Langevin KATs
def test_modifier_kats_on_gpu(oracle):
    from test_oracle import BS, MODIFIER_KATS, _p
    ss = _gpu()
    for name, kw, start, expect in MODIFIER_KATS:
        mask = getattr(oracle, name)
        got = ss.langevin(_p(oracle, *start)[None], mask, box=BS, **kw)[0]
        want = _p(oracle, *expect)
        assert np.allclose(got, want, rtol=4e-16, atol=4e-16), (name, got, want)


def test_full_chain_on_gpu_matches_oracle(oracle):
    ss = _gpu()
    rng = np.random.default_rng(5)
    n = 4096
    box = (5.0, 4.0, 3.0)
    p = _particles(rng, n, box, False)
    kw = dict(flow=rng.standard_normal(3), drag=0.3, gradb=rng.standard_normal(9), reorientation=0.7,
              b=rng.standard_normal(3), vort=rng.standard_normal(9), shape=0.5, strain=rng.standard_normal(9),
              dt=0.01, xi=rng.standard_normal(3), diff=0.04, axis_angle=1.3, rotate_angle=0.2)
    got = ss.langevin(p, oracle.ALL, box=box, **kw)
    want = np.array([oracle.langevin(q, oracle.ALL, box=box, **kw) for q in p])
    assert rel_l2(got, want) < 1e-15
    for mask in [0, oracle.STEP | oracle.ROT_DIFFUSION, oracle.EXTERNAL_FIELD | oracle.JEFFREY_STRAIN]:
        got = ss.langevin(p[:64], mask, box=box, **kw)
        want = np.array([oracle.langevin(q, mask, box=box, **kw) for q in p[:64]])
        assert rel_l2(got, want) < 1e-15, mask


# ------------------------------------------------------- binning, bit-exact
@pytest.mark.parametrize("cfg", CONFIGS, ids=[c[0] for c in CONFIGS])
def test_init_histogram_bit_exact(oracle, cfg):
    g, o, s = _pair(oracle, cfg)
    rng = np.random.default_rng(11)
    p = _particles(rng, cfg[4], cfg[2], cfg[5])
    # out-of-box and negative inputs, exact cell edges, the box border
    gw = oracle.grid_width(s)
    k = min(len(p), 200)
    p[:k, 0] = gw[0] * rng.integers(-3, 2 * s.gx, k)
    p[:k, 3] = gw[3] * rng.integers(-2 * s.gphi, 2 * s.gphi, k)
    p[k:2 * k, 0] = np.nextafter(cfg[2][0], 0.0)
    p[k:2 * k, 1] = -rng.random(k) * 3 * cfg[2][1]
    p[2 * k:3 * k, 3] = np.nextafter(TWOPI, 0.0)
    if not cfg[5]:
        p[3 * k:4 * k, 4] = PI
        p[4 * k:5 * k, 4] = -rng.random(k)
    g.init(p)
    o.init(p)
    assert np.array_equal(g.get_particles(), o.particles())
    counts = g.get_counts()
    hist = oracle.histogram(s, o.particles())
    assert counts.sum() == cfg[4]
    assert np.array_equal(counts.astype(np.float64), hist)
    assert np.array_equal(g.get_distribution(), o.distribution())
    g.close()


# ------------------------------------------------------------ one step
@pytest.mark.parametrize("cfg", CONFIGS, ids=[c[0] for c in CONFIGS])
def test_one_step_matches_oracle(oracle, cfg):
    # EVEN2D runs the step without the dipolar solver (its couplings are zero)
    always_mag = cfg is not EVEN2D
    g, o, s = _pair(oracle, cfg, always_magnetic=always_mag)
    rng = np.random.default_rng(21)
    p = _particles(rng, cfg[4], cfg[2], cfg[5])
    noise = _noise(rng, cfg[4], cfg[3])
    g.init(p)
    o.init(p)
    assert g.do_timestep(noise) == 1
    o.do_timestep(noise)
    u, gu = g.get_flow_complex()
    assert rel_l2(u, o.flow()) < TOL
    assert rel_l2(gu, o.flow_grad()) < TOL
    assert np.array_equal(g.get_distribution(), o.distribution())
    gp, op = g.get_particles(), o.particles()
    # computed lazily from the same histogram when the step skipped it
    b, gb = g.get_magnetic_complex()
    assert rel_l2(b, o.mag()) < TOL
    assert rel_l2(gb, o.mag_grad()) < TOL
    assert rel_l2(gp[:, :3], op[:, :3]) < TOL
    assert rel_l2(gp[:, 3:], op[:, 3:]) < TOL
    # per particle: every displacement agrees to 1e-12 of its own size
    d_g = np.abs(gp - op).max(axis=0)
    assert np.all(d_g < 1e-12 * np.array([*cfg[2], TWOPI, PI])), d_g
    # the histogram the update bins into is the one the next step solves from
    g.do_timestep(_noise(rng, cfg[4], cfg[3]))
    assert np.array_equal(g.get_counts().astype(np.float64), oracle.histogram(s, gp))
    g.close()


@pytest.mark.parametrize("cfg", [C0, ODD3D], ids=["c0_2d", "odd_3d_magnetic"])
def test_philox_trajectory_matches_oracle(oracle, cfg):
    """Five steps of the production path (on-device Philox noise, sort, CUDA
    graph) against the oracle fed the same noise."""
    g, o, s = _pair(oracle, cfg)
    rng = np.random.default_rng(31)
    p = _particles(rng, cfg[4], cfg[2], cfg[5])
    g.init(p)
    o.init(p)
    for t in range(5):
        noise = g.noise(t)
        g.do_timestep()
        o.do_timestep(noise)
        gp, op = g.get_particles(), o.particles()
        assert rel_l2(gp[:, :3], op[:, :3]) < TOL, t
        assert rel_l2(gp[:, 3:], op[:, 3:]) < TOL, t
    u, _ = g.get_flow_complex()
    assert rel_l2(u, o.flow()) < TOL
    g.close()


def test_quasi2d_off_canonical_rows(oracle):
    """Quasi2d rows off the canonical state (theta != pi/2, z != 0): the first
    step runs the full chain, the following ones the canonical quasi-2-D
    chain (z and theta neither read nor written); every step against the
    oracle fed the same noise, histograms bit-exact."""
    g, o, s = _pair(oracle, EVEN2D)
    name, grid, box, params, n, q2d = EVEN2D
    rng = np.random.default_rng(61)
    p = _particles(rng, n, box, False)
    g.init(p)
    o.init(p)
    for t in range(4):
        noise = g.noise(t)
        g.do_timestep()
        o.do_timestep(noise)
        gp, op = g.get_particles(), o.particles()
        assert np.all(gp[:, 2] == 0.0) and np.all(gp[:, 4] == PI / 2), t
        assert rel_l2(gp[:, :3], op[:, :3]) < TOL, t
        assert rel_l2(gp[:, 3:], op[:, 3:]) < TOL, t
        assert np.array_equal(g.get_distribution(), o.distribution()), t
    g.close()


def test_fp64_rate_probe():
    """ss_fp64_rate: the FP64 FMA rate of the device, a positive finite rate
    below the nominal peak of any current GPU."""
    import ctypes
    ss = _gpu()
    from stochasticsampling_gb300 import _lib
    r = ctypes.c_double()
    _lib.check(_lib.load().ss_fp64_rate(ctypes.byref(r)))
    assert 1e9 < r.value < 1e14, r.value


def test_philox_noise_statistics():
    ss = _gpu()
    n = 1_000_000
    g = ss.Simulation(grid=(8, 8, 4, 4, 4), box=(1, 1, 1),
                      params=dict(number_of_particles=n, timestep=0.01, rot_diffusion=2.0, seed=9))
    z = g.noise(3)
    assert np.all(np.isfinite(z))
    se = 5 / np.sqrt(n)
    for c in range(3):
        assert abs(z[:, c].mean()) < se and abs(z[:, c].var() - 1) < 5 * np.sqrt(2 / n)
    assert abs(z[:, 3].mean() / TWOPI - 0.5) < se and z[:, 3].min() >= 0 and z[:, 3].max() < TWOPI
    sigma = np.sqrt(2 * 2.0 * 0.01)
    assert abs((z[:, 4] ** 2).mean() / (2 * sigma ** 2) - 1) < 10 / np.sqrt(n)  # Rayleigh: E[r^2] = 2 sigma^2
    assert not np.array_equal(g.noise(4)[:, 0], z[:, 0])
    assert np.array_equal(g.noise(3), z)
    g.close()


# ---------------------------------------------- invariances of the GPU path
def test_sort_graph_invariance(oracle):
    ss = _gpu()
    name, grid, box, params, n, q2d = ODD3D
    rng = np.random.default_rng(41)
    p = _particles(rng, n, box, q2d)
    out = []
    for kw in [dict(), dict(sort=False, graph=False), dict(sort=True, graph=False), dict(sort=False)]:
        g = ss.Simulation(grid=grid, box=box, params=dict(params, number_of_particles=n, seed=3), quasi2d=q2d, **kw)
        g.init(p)
        g.run(4)
        out.append((g.get_particles(), g.get_counts()))
        g.close()
    for a, c in out[1:]:
        assert np.array_equal(a, out[0][0]) and np.array_equal(c, out[0][1])


def test_resume_is_exact(oracle):
    ss = _gpu()
    name, grid, box, params, n, q2d = C0
    rng = np.random.default_rng(51)
    p = _particles(rng, n, box, q2d)
    mk = lambda: ss.Simulation(grid=grid, box=box, params=dict(params, number_of_particles=n, seed=7), quasi2d=q2d)
    a = mk()
    a.init(p)
    a.run(3)
    snap = a.get_snapshot()
    a.run(3)
    b = mk()
    b.resume(snap["particles"], snap["timestep"])
    assert b.get_timestep() == 3
    b.run(3)
    assert b.get_timestep() == 6
    assert np.array_equal(a.get_particles(), b.get_particles())
    a.close()
    b.close()


# ------------------------------------------------------------ spectral seams
def test_flow_golden_on_gpu(oracle):
    ss = _gpu()
    g = ss.Simulation(grid=(11, 11, 11, 11, 11), box=(11.0, 11.0, 11.0),
                      params=dict(number_of_particles=1, stress_active=1.0))
    g.init(np.array([[0.0, 0.0, 0.0, PI / 2, PI / 2]]))
    u, _ = g.mean_flow_field(0.0, g.get_distribution())
    gold = np.load(os.path.join(GOLDEN, "ff_test.npy"))
    assert rel_l2(u.real, gold) < 1e-14
    g.close()


@pytest.mark.parametrize("grid", [(8, 6, 4, 4, 2), (7, 5, 3, 3, 5), (16, 16, 1, 8, 1), (1, 9, 4, 2, 2), (2, 2, 2, 1, 1)])
def test_mean_fields_random_distribution(oracle, grid):
    ss = _gpu()
    box = (2.0 + grid[0], 1.5 + grid[1], 1.0 + grid[2])
    params = dict(number_of_particles=4, stress_active=-1.7, stress_magnetic=0.3, shape=0.2)
    g = ss.Simulation(grid=grid, box=box, params=params)
    s = oracle.make_settings(grid, box, active=-1.7, magnetic=0.3, shape=0.2)
    d = np.random.default_rng(sum(grid)).random(grid) * 3.0
    for scr in (0.0, 0.7):
        u, gu = g.mean_flow_field(scr, d)
        ou, og = oracle.flow_field(s, d, scr)
        assert rel_l2(u, ou) < 1e-13 and rel_l2(gu, og) < 1e-13
    b, gb = g.mean_magnetic_field(d)
    ob, ogb = oracle.magnetic_field(s, d)
    assert rel_l2(b, ob) < 1e-13 and rel_l2(gb, ogb) < 1e-13
    g.close()


def test_lazy_magnetic_field(oracle):
    ss = _gpu()
    name, grid, box, params, n, q2d = C0
    rng = np.random.default_rng(61)
    p = _particles(rng, n, box, q2d)
    noise = _noise(rng, n, params)
    sims = [ss.Simulation(grid=grid, box=box, params=dict(params, number_of_particles=n), quasi2d=q2d,
                          always_magnetic=am) for am in (False, True)]
    for g in sims:
        assert np.all(g.get_magnetic_field() == 0.0)
        g.init(p)
        g.do_timestep(noise)
    lazy, full = sims[0].get_magnetic_field(), sims[1].get_magnetic_field()
    assert rel_l2(lazy, full) < 1e-14 and np.linalg.norm(full) > 0
    # the step without the dipolar solve runs the canonical quasi-2-D chain
    # (cos(pi/2) taken as 0), the magnetic step the full chain: last bits only
    a, b = sims[0].get_particles(), sims[1].get_particles()
    assert rel_l2(a, b) < 1e-15
    assert np.array_equal(sims[0].get_counts(), sims[1].get_counts())
    for g in sims:
        g.close()


# ------------------------------------------------------ trilinear gather
@pytest.mark.parametrize("gather", [1, 2], ids=["trilinear", "trilinear_zfromy"])
@pytest.mark.parametrize("cfg", [SMALL3D, EVEN2D], ids=["small_3d_all_terms", "even_2d_screened"])
def test_trilinear_gather_matches_oracle(oracle, cfg, gather):
    """The gather of src/mesh/interpolate.rs (periodic trilinear between cell
    centres) in place of the nearest cell, on every gathered field."""
    ss = _gpu()
    name, grid, box, params, n, q2d = cfg
    p_ = dict(params, number_of_particles=n, seed=1)
    g = ss.Simulation(grid=grid, box=box, params=p_, quasi2d=q2d, always_magnetic=True,
                      gather={1: "trilinear", 2: "trilinear_zfromy"}[gather])
    s = oracle.make_settings(grid, box, timestep=p_["timestep"], trans_diff=p_.get("trans_diffusion", 0.0),
                             rot_diff=p_.get("rot_diffusion", 0.0), active=p_.get("stress_active", 0.0),
                             magnetic=p_.get("stress_magnetic", 0.0), shape=p_.get("shape", 0.0),
                             magnetic_drag=p_.get("magnetic_drag", 0.0),
                             hydro_screening=p_.get("hydro_screening", 0.0),
                             volume_exclusion=p_.get("volume_exclusion", 0.0),
                             magnetic_reorientation=p_.get("magnetic_reorientation", 0.0),
                             magnetic_dipole_dipole=p_.get("magnetic_dipole_dipole", 0.0), quasi2d=q2d,
                             gather=gather)
    o = oracle.Simulation(s, n, nthreads=8)
    rng = np.random.default_rng(101)
    p = _particles(rng, n, box, q2d)
    noise = _noise(rng, n, params)
    g.init(p)
    o.init(p)
    g.do_timestep(noise)
    o.do_timestep(noise)
    gp, op = g.get_particles(), o.particles()
    assert rel_l2(gp[:, :3], op[:, :3]) < TOL and rel_l2(gp[:, 3:], op[:, 3:]) < TOL
    g.close()


# ---------------------------------------------------------------- errors
def test_error_paths(oracle):
    ss = _gpu()
    g = ss.Simulation(grid=(4, 4, 1, 4, 1), box=(1, 1, 1), params=dict(number_of_particles=8, timestep=0.1),
                      quasi2d=True)
    with pytest.raises(ss.SsError) as e:
        g.do_timestep()
    assert e.value.code == 4
    with pytest.raises(ss.SsError) as e:
        g.init(np.zeros((7, 5)))
    assert e.value.code == 5
    bad = np.zeros((8, 5))
    bad[3, 1] = np.nan
    with pytest.raises(ss.SsError) as e:
        g.init(bad)
    assert e.value.code == 1
    g.init(np.zeros((8, 5)))
    with pytest.raises(ss.SsError):
        g.get_particles_head(9)
    assert g.get_particles_head(3).shape == (3, 5)
    g.do_timestep()
    g.synchronize()
    g.close()


# -------------------------------------------------- full benchmark sizes
def _c1_particles(rng, n):
    # 1 % sinusoidal density along x (wavenumber 2 pi / 40), by inverse CDF
    L = 40.0
    u = rng.random(n)
    x = u * L
    for _ in range(30):  # Newton on F(x) = x/L - 0.01 cos(2 pi x/L)/(2 pi) + 0.01/(2 pi) - u
        f = x / L + 0.01 * (1 - np.cos(TWOPI * x / L)) / TWOPI - u
        x -= f / ((1 + 0.01 * np.sin(TWOPI * x / L)) / L)
    return np.column_stack([np.mod(x, L), L * rng.random(n), np.zeros(n), TWOPI * rng.random(n), np.full(n, PI / 2)])


def test_c1_full_size_step(oracle):
    """Production size 2-D: N = 1e7, grid 128x128x1x32x1, box 40x40, Dt 0.1,
    Dr 1.0, active -2, dt 0.005.  Initial histogram bit-exact; one Philox step
    matches the oracle fed the same noise; the histogram of the positions it
    wrote is bit-exact; the histogram sum is N after more steps."""
    cfg = ("c1", (128, 128, 1, 32, 1), (40.0, 40.0, 1.0),
           dict(timestep=0.005, trans_diffusion=0.1, rot_diffusion=1.0, stress_active=-2.0), 10_000_000, True)
    g, o, s = _pair(oracle, cfg)
    p = _c1_particles(np.random.default_rng(1), cfg[4])
    g.init(p)
    o.init(p)
    assert np.array_equal(g.get_counts().astype(np.float64), oracle.histogram(s, o.particles()))
    noise = g.noise(0)
    g.do_timestep()
    o.do_timestep(noise)
    u, gu = g.get_flow_complex()
    assert rel_l2(u, o.flow()) < TOL and rel_l2(gu, o.flow_grad()) < TOL
    gp, op = g.get_particles(), o.particles()
    assert rel_l2(gp[:, :2], op[:, :2]) < TOL and rel_l2(gp[:, 3], op[:, 3]) < TOL
    # the histogram the update binned into (the next step's input) is the
    # reference's histogram of the positions the step wrote, bit for bit
    g.do_timestep()
    assert np.array_equal(g.get_counts().astype(np.float64), oracle.histogram(s, gp))
    g.run(3)
    g.do_timestep()
    assert int(g.get_counts().sum()) == cfg[4]
    g.close()


def test_c2_full_size_step(oracle):
    """3-D with the dipolar solver at full size: N = 2e7, grid 64^3 x 16 x 8,
    box 20^3, dipolar coupling 0.5, field along the reference's axis (y)."""
    cfg = ("c2", (64, 64, 64, 16, 8), (20.0, 20.0, 20.0),
           dict(timestep=0.002, trans_diffusion=0.1, rot_diffusion=1.0, stress_active=-1.0,
                magnetic_reorientation=1.0, magnetic_dipole_dipole=0.5), 20_000_000, False)
    g, o, s = _pair(oracle, cfg)
    p = _particles(np.random.default_rng(2), cfg[4], cfg[2], False)
    g.init(p)
    o.init(p)
    assert np.array_equal(g.get_counts().astype(np.float64), oracle.histogram(s, o.particles()))
    noise = g.noise(0)
    g.do_timestep()
    o.do_timestep(noise)
    b, gb = g.get_magnetic_complex()
    assert rel_l2(b, o.mag()) < TOL and rel_l2(gb, o.mag_grad()) < TOL
    gp, op = g.get_particles(), o.particles()
    assert rel_l2(gp[:, :3], op[:, :3]) < TOL and rel_l2(gp[:, 3:], op[:, 3:]) < TOL
    g.close()
