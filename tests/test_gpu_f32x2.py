"""The FP64 mode with SS_FLAG_F32X2: the canonical quasi-2-D update computes
the step's increments in two-float arithmetic (csrc/f32x2.cuh) and adds them
to the FP64 state in FP64.  Against the oracle with the bars of the FP64
mode (1e-12 norm-wise; histograms of the positions bit-exact) and, tighter,
against the accuracy the pair arithmetic gives: about 1e-14 absolute per
step on x, y and phi."""
import numpy as np
import pytest

from conftest import rel_l2
from test_gpu_parity import C0, EVEN2D, PI, TOL, TWOPI, _c1_particles, _gpu, _noise, _pair, _particles

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
