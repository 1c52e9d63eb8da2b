"""The FP64 mode with SS_FLAG_F32X2: the update (the canonical quasi-2-D chain
and the full chain: 3-D, dipolar terms, quasi-2-D rows off the canonical
state) computes the step's increments in two-float arithmetic
(csrc/f32x2.cuh) and adds them to the FP64 state in FP64.  Against the
oracle with the bars of the FP64 mode (1e-12 norm-wise; histograms of the
positions bit-exact) and, tighter, against the accuracy the pair arithmetic
gives: a few 1e-14 absolute per step on positions and on the orientation
(phi's error weighted by sin theta: phi is ill-conditioned near a pole in
any arithmetic)."""
import numpy as np
import pytest

from conftest import rel_l2
from test_gpu_parity import (C0, EVEN2D, ODD3D, PI, SMALL3D, TOL, TWOPI, _c1_particles, _gpu, _noise, _pair,
                             _particles)

pytestmark = pytest.mark.gpu

# per-step deviation from the FP64 oracle: a few 2^-48 of the increments
# (dx, dy ~ 0.1, dphi ~ 0.5) plus the rounding of the FP64 sums
STEP_ABS = (2e-14, 2e-14, 0.0, 4e-14, 0.0)


@pytest.mark.parametrize("cfg", [C0, EVEN2D], ids=["c0_2d", "even_2d_screened"])
def test_one_step_matches_oracle(oracle, cfg):
    name, grid, box, params, n, q2d = cfg
    g, o, s = _pair(oracle, cfg, f32x2=True)
    rng = np.random.default_rng(21)
    p = _particles(rng, n, box, True)
    noise = _noise(rng, n, params)
    g.init(p)
    o.init(p)
    assert g.do_timestep(noise) == 1
    o.do_timestep(noise)
    gp, op = g.get_particles(), o.particles()
    assert rel_l2(gp[:, :3], op[:, :3]) < TOL
    assert rel_l2(gp[:, 3:], op[:, 3:]) < TOL
    d = np.abs(gp - op).max(axis=0)
    assert np.all(d <= np.array(STEP_ABS)), d
    # the histogram the update bins into is that of the positions it wrote
    g.do_timestep(_noise(rng, n, params))
    assert np.array_equal(g.get_counts().astype(np.float64), oracle.histogram(s, gp))
    g.close()


def test_philox_trajectory_matches_oracle(oracle):
    """Five steps of the production path (Philox noise drawn on the device as
    floats, sort, CUDA graph) against the oracle fed the same noise."""
    g, o, s = _pair(oracle, C0, f32x2=True)
    rng = np.random.default_rng(31)
    p = _particles(rng, C0[4], C0[2], True)
    g.init(p)
    o.init(p)
    for t in range(5):
        noise = g.noise(t)
        g.do_timestep()
        o.do_timestep(noise)
        gp, op = g.get_particles(), o.particles()
        assert rel_l2(gp[:, :3], op[:, :3]) < TOL, t
        assert rel_l2(gp[:, 3:], op[:, 3:]) < TOL, t
        d = np.abs(gp - op).max(axis=0)
        assert np.all(d <= 3 * np.array(STEP_ABS)), (t, d)
    g.close()


def test_c1_full_size_against_fp64_mode():
    """Production size (N = 1e7, grid 128x128x32, box 40x40, dt 0.005): ten
    Philox steps in the FP64 mode and with SS_FLAG_F32X2 from the same state;
    positions agree to 1e-12 of the box and the histograms differ only by the
    few particles within that distance of a bin edge."""
    ss = _gpu()
    grid, box = (128, 128, 1, 32, 1), (40.0, 40.0, 1.0)
    n = 10_000_000
    params = dict(timestep=0.005, trans_diffusion=0.1, rot_diffusion=1.0, stress_active=-2.0,
                  number_of_particles=n, seed=5)
    p = _c1_particles(np.random.default_rng(2), n)
    sims = [ss.Simulation(grid=grid, box=box, params=params, quasi2d=True, sort=False, f32x2=f) for f in (False, True)]
    for g in sims:
        g.init(p)
        g.run(10)
    a, b = (g.get_particles() for g in sims)
    d = np.abs(a - b)
    d = np.minimum(d, np.array([40.0, 40.0, 1.0, TWOPI, PI]) - d)  # a wrap on one side only
    assert d.max(axis=0)[[0, 1, 3]].max() < 1e-12, d.max(axis=0)
    assert np.array_equal(a[:, [2, 4]], b[:, [2, 4]])
    ca, cb = (g.get_counts() for g in sims)
    assert int(ca.sum()) == int(cb.sum()) == n
    assert np.abs(ca.astype(np.int64) - cb.astype(np.int64)).sum() <= 20
    for g in sims:
        g.close()


def test_rejected_with_mixed_modes():
    ss = _gpu()
    for mixed in (True, "fixed64"):
        with pytest.raises(Exception, match="F32X2"):
            ss.Simulation(grid=(8, 8, 1, 8, 1), box=(1.0, 1.0, 1.0), params=dict(number_of_particles=100),
                          quasi2d=True, mixed=mixed, f32x2=True)


def _orientation_errors(gp, op):
    """largest position, theta and sin(theta)-weighted phi deviation"""
    d = np.abs(gp - op)
    dphi = np.minimum(d[:, 3], TWOPI - d[:, 3]) * np.sin(op[:, 4])
    return d[:, :3].max(), d[:, 4].max(), dphi.max()


@pytest.mark.parametrize("cfg", [SMALL3D, ODD3D], ids=["small_3d_all_terms", "odd_3d_magnetic"])
def test_full_chain_one_step_matches_oracle(oracle, cfg):
    name, grid, box, params, n, q2d = cfg
    g, o, s = _pair(oracle, cfg, f32x2=True, always_magnetic=True)
    rng = np.random.default_rng(21)
    p = _particles(rng, n, box, q2d)
    noise = _noise(rng, n, params)
    g.init(p)
    o.init(p)
    assert g.do_timestep(noise) == 1
    o.do_timestep(noise)
    gp, op = g.get_particles(), o.particles()
    assert rel_l2(gp[:, :3], op[:, :3]) < TOL
    assert rel_l2(gp[:, 3:], op[:, 3:]) < TOL
    dpos, dth, dphi = _orientation_errors(gp, op)
    assert dpos < 2e-14 and dth < 5e-14 and dphi < 5e-14, (dpos, dth, dphi)
    g.do_timestep(_noise(rng, n, params))
    assert np.array_equal(g.get_counts().astype(np.float64), oracle.histogram(s, gp))
    g.close()


def test_full_chain_philox_trajectory_matches_oracle(oracle):
    g, o, s = _pair(oracle, ODD3D, f32x2=True)
    rng = np.random.default_rng(31)
    p = _particles(rng, ODD3D[4], ODD3D[2], False)
    g.init(p)
    o.init(p)
    for t in range(5):
        noise = g.noise(t)
        g.do_timestep()
        o.do_timestep(noise)
        gp, op = g.get_particles(), o.particles()
        assert rel_l2(gp[:, :3], op[:, :3]) < TOL, t
        assert rel_l2(gp[:, 3:], op[:, 3:]) < TOL, t
        dpos, dth, dphi = _orientation_errors(gp, op)
        assert dpos < 1e-13 and dth < 2e-13 and dphi < 2e-13, (t, dpos, dth, dphi)
    g.close()


def test_quasi2d_off_canonical_rows(oracle):
    """The first step of rows off the canonical state runs the full chain in
    pairs, the next ones the canonical chain in pairs; every step against the
    oracle fed the same noise, histograms bit-exact."""
    g, o, s = _pair(oracle, EVEN2D, f32x2=True)
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


def test_c2_full_size_against_fp64_mode():
    """3-D with the dipolar solver at full size (N = 2e7, grid 64^3 x 16 x 8,
    box 20^3): five Philox steps in the FP64 mode and with SS_FLAG_F32X2
    from the same state; positions and orientations agree to 1e-12 and the
    histograms differ only by the few particles that close to a bin edge."""
    ss = _gpu()
    grid, box = (64, 64, 64, 16, 8), (20.0, 20.0, 20.0)
    n = 20_000_000
    params = dict(timestep=0.002, trans_diffusion=0.1, rot_diffusion=1.0, stress_active=-1.0,
                  magnetic_reorientation=1.0, magnetic_dipole_dipole=0.5, number_of_particles=n, seed=4)
    p = _particles(np.random.default_rng(3), n, box, False)
    sims = [ss.Simulation(grid=grid, box=box, params=params, sort=False, f32x2=f) for f in (False, True)]
    for g in sims:
        g.init(p)
        g.run(5)
    a, b = (g.get_particles() for g in sims)
    d = np.abs(a - b)
    d[:, :3] = np.minimum(d[:, :3], np.array(box) - d[:, :3])
    d[:, 3] = np.minimum(d[:, 3], TWOPI - d[:, 3]) * np.sin(a[:, 4])
    assert d.max(axis=0).max() < 1e-12, d.max(axis=0)
    ca, cb = (g.get_counts() for g in sims)
    assert int(ca.sum()) == int(cb.sum()) == n
    assert np.abs(ca.astype(np.int64) - cb.astype(np.int64)).sum() <= 40
    for g in sims:
        g.close()
