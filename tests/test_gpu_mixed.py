"""The FP32 mixed-precision path against the FP64 oracle, with positions
accumulated in FP64 (SS_FLAG_MIXED) or in 64-bit fixed point (SS_FLAG_FIXED64).

The mixed path keeps positions and the spectral k = 0 / mean handling in FP64
and does everything else in FP32, so it is not held to 1e-12; each field's
error against the FP64 oracle is bounded instead (one step from identical
state and noise; measured on GB300 in brackets):
  histogram       differs only for particles within FP32 rounding of a bin
                  edge (none for the seeded clouds of the one-step test)
  u, grad u       relative L2 error < 2e-6 (1.8e-7 .. 3.8e-7)
  B               relative L2 error < 1e-5
  positions       relative L2 error < 5e-9 (4.7e-10 .. 1.1e-9; FP64
                  accumulation of FP32 steps)
  phi             RMS error < 1e-6 rad (1.8e-7 .. 2.0e-7)
"""
import numpy as np
import pytest

from conftest import rel_l2
from test_gpu_parity import C0, EVEN2D, ODD3D, _c1_particles, _gpu, _noise, _pair, _particles

pytestmark = pytest.mark.gpu


MODES = pytest.mark.parametrize("mode", [True, "fixed64"], ids=["fp64_positions", "fixed64_positions"])


def _wrapdiff(a, b, period):
    d = np.abs(a - b)
    return np.minimum(d, period - d)


@MODES
@pytest.mark.parametrize("cfg", [C0, EVEN2D, ODD3D], ids=["c0_2d", "even_2d_screened", "odd_3d_magnetic"])
def test_mixed_one_step_errors(oracle, cfg, mode):
    g, o, s = _pair(oracle, cfg, mixed=mode)
    rng = np.random.default_rng(71)
    n = cfg[4]
    p = _particles(rng, n, cfg[2], cfg[5])
    noise = _noise(rng, n, cfg[3])
    g.init(p)
    o.init(p)
    c_g = g.get_counts().astype(np.float64)
    c_o = oracle.histogram(s, o.particles())
    assert c_g.sum() == n
    # FP32 binning differs from the reference's only within FP32 rounding of a
    # bin edge; none of these seeded particles lies that close
    assert np.array_equal(c_g, c_o)
    g.do_timestep(noise)
    o.do_timestep(noise)
    u, gu = g.get_flow_complex()
    ou = o.flow()
    eu, egu = rel_l2(u, ou), rel_l2(gu, o.flow_grad())
    gp, op = g.get_particles(), o.particles()
    ex = rel_l2(gp[:, :3], op[:, :3])
    ephi = float(np.sqrt(np.mean(_wrapdiff(gp[:, 3], op[:, 3], 2 * np.pi) ** 2)))
    print(f"mixed {cfg[0]} {mode}: hist {np.abs(c_g - c_o).sum() / n:.3e} u {eu:.3e} grad u {egu:.3e} "
          f"positions {ex:.3e} phi rms {ephi:.3e}")
    assert eu < 2e-6 and egu < 2e-6
    assert ex < 5e-9
    assert ephi < 1e-6
    g.close()


@MODES
def test_mixed_fields_from_identical_histogram(oracle, mode):
    """Fields of the mixed solve when its histogram equals the FP64 one:
    particles at bin centres, so FP32 binning cannot differ."""
    ss = _gpu()
    name, grid, box, params, n, q2d = ODD3D
    rng = np.random.default_rng(81)
    gw = np.array(box) / np.array(grid[:3])
    idx = np.column_stack([rng.integers(0, grid[k], n) for k in range(3)])
    ang = np.column_stack([rng.integers(0, grid[3], n), rng.integers(0, grid[4], n)])
    p = np.column_stack([(idx + 0.5) * gw, (ang[:, 0] + 0.5) * 2 * np.pi / grid[3], (ang[:, 1] + 0.5) * np.pi / grid[4]])
    g, o, s = _pair(oracle, ODD3D, mixed=mode)
    g.init(p)
    o.init(p)
    assert np.array_equal(g.get_counts().astype(np.float64), oracle.histogram(s, o.particles()))
    noise = _noise(rng, n, params)
    g.do_timestep(noise)
    o.do_timestep(noise)
    u, gu = g.get_flow_complex()
    assert rel_l2(u, o.flow()) < 1e-5 and rel_l2(gu, o.flow_grad()) < 1e-5
    b, gb = g.get_magnetic_complex()
    assert rel_l2(b, o.mag()) < 1e-5 and rel_l2(gb, o.mag_grad()) < 1e-5
    gp, op = g.get_particles(), o.particles()
    assert rel_l2(gp[:, :3], op[:, :3]) < 1e-8
    assert rel_l2(gp[:, 3:], op[:, 3:]) < 1e-6
    g.close()


@MODES
def test_mixed_runs_and_conserves(oracle, mode):
    ss = _gpu()
    name, grid, box, params, n, q2d = C0
    rng = np.random.default_rng(91)
    p = _particles(rng, n, box, q2d)
    g = ss.Simulation(grid=grid, box=box, params=dict(params, number_of_particles=n, seed=5), quasi2d=q2d,
                      mixed=mode)
    g.init(p)
    g.run(20)
    g.do_timestep()
    assert g.get_counts().sum() == n
    q = g.get_particles()
    assert np.all(np.isfinite(q))
    assert np.all((q[:, 0] >= 0) & (q[:, 0] < box[0]) & (q[:, 1] >= 0) & (q[:, 1] < box[1]))
    assert np.all(q[:, 2] == 0.0)
    # mean squared displacement of the translational noise dominates: sanity only
    z = g.noise(3)
    assert abs(z[:, 0].mean()) < 0.05 and abs(z[:, 0].var() - 1) < 0.05
    g.close()


@MODES
def test_mixed_c1_full_size(oracle, mode):
    """Production size 2-D in mixed precision: one step against the oracle fed
    the same noise, then ten more steps."""
    cfg = ("c1", (128, 128, 1, 32, 1), (40.0, 40.0, 1.0),
           dict(timestep=0.005, trans_diffusion=0.1, rot_diffusion=1.0, stress_active=-2.0), 10_000_000, True)
    g, o, s = _pair(oracle, cfg, mixed=mode)
    p = _c1_particles(np.random.default_rng(1), cfg[4])
    g.init(p)
    o.init(p)
    noise = g.noise(0)
    g.do_timestep()
    o.do_timestep(noise)
    u, _ = g.get_flow_complex()
    assert rel_l2(u, o.flow()) < 1e-2
    gp, op = g.get_particles(), o.particles()
    assert rel_l2(gp[:, :2], op[:, :2]) < 1e-6
    g.run(10)
    g.do_timestep()
    assert int(g.get_counts().sum()) == cfg[4]
    g.close()


def test_fixed64_wraps_and_bins_exactly(oracle):
    """64-bit fixed point: crossing the box faces wraps by integer overflow and
    the histogram of the stored positions is the FP64 binning of them."""
    ss = _gpu()
    grid, box = (16, 12, 1, 8, 1), (8.0, 6.0, 1.0)
    n = 50_000
    rng = np.random.default_rng(5)
    p = _particles(rng, n, box, True)
    p[:1000, 0] = box[0] - 1e-9  # next to the face: most cross it in one step
    g = ss.Simulation(grid=grid, box=box, params=dict(number_of_particles=n, timestep=0.01, trans_diffusion=0.5,
                                                      rot_diffusion=0.5, stress_active=-1.0), quasi2d=True,
                      mixed="fixed64")
    g.init(p)
    g.run(5)
    g.do_timestep()
    q = g.get_particles()
    assert np.all((q[:, 0] >= 0) & (q[:, 0] < box[0]) & (q[:, 1] >= 0) & (q[:, 1] < box[1]))
    s = oracle.make_settings(grid, box, quasi2d=True)
    # the counts of the last step were binned from the positions before it
    g2 = ss.Simulation(grid=grid, box=box, params=dict(number_of_particles=n), quasi2d=True, mixed="fixed64")
    g2.init(q)
    hist = oracle.histogram(s, np.column_stack([q[:, :3], q[:, 3], np.full(n, np.pi / 2)]))
    assert np.abs(g2.get_counts().astype(np.float64) - hist).sum() <= 1e-4 * n  # FP32 angle bins only
    g.close()
    g2.close()


@MODES
def test_mixed_fields_follow_replayed_steps(mode):
    """The FP64 copy of the mixed fields that the getters read is refreshed
    after graph-replayed steps (not only after directly launched ones)."""
    ss = _gpu()
    name, grid, box, params, n, q2d = C0
    p = dict(params, number_of_particles=n, seed=3)
    g = ss.Simulation(grid=grid, box=box, params=p, quasi2d=True, mixed=mode)
    rng = np.random.default_rng(5)
    g.init(_particles(rng, n, box, True))
    g.run(2)
    u1 = g.get_flow_field()
    g.run(1)
    u2 = g.get_flow_field()
    assert np.linalg.norm(u2 - u1) > 1e-3 * np.linalg.norm(u1)
    # the same state re-solved from scratch gives the same field
    h = ss.Simulation(grid=grid, box=box, params=p, quasi2d=True, mixed=mode)
    h.resume(g.get_particles(), g.get_timestep())
    h.run(1)
    g.run(1)
    assert np.linalg.norm(h.get_flow_field() - g.get_flow_field()) <= 1e-5 * np.linalg.norm(g.get_flow_field())
    g.close()
    h.close()
