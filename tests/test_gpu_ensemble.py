"""Batched ensembles (ss_ensemble_*): every member against a stand-alone
quasi-2-D mixed-precision context with the same grid, box, parameters,
initial rows and seed.

Both run the same FP32 arithmetic and the same Philox stream; they differ
only in how cuFFT batches the transforms and in the summation order of the
FP64 component sums, so
  initial histogram   bit-exact (same binning)
  fields, one step    relative L2 < 1e-5 (FFT round-off)
  positions, k steps  equal to FP32 round-off for all but the few particles
                      that a rounding moved across a cell edge
"""
import numpy as np
import pytest

from conftest import rel_l2
from test_gpu_parity import _gpu

pytestmark = pytest.mark.gpu

# (grid, box, params, n, seed): shared and distinct grid shapes, odd edges,
# uneven particle counts, every Langevin term the ensemble supports
MEMBERS = [
    ((32, 32, 1, 16, 1), (10.0, 10.0, 1.0), dict(timestep=0.01, trans_diffusion=0.1, rot_diffusion=0.5,
                                                   stress_active=-1.0), 60_000, 11),
    ((32, 32, 1, 16, 1), (12.0, 8.0, 1.0), dict(timestep=0.005, trans_diffusion=0.2, rot_diffusion=1.0,
                                                  stress_active=-2.5, hydro_screening=0.2), 25_000, 12),
    ((16, 12, 1, 8, 1), (8.0, 6.0, 1.0), dict(timestep=0.005, trans_diffusion=0.1, rot_diffusion=1.0,
                                                stress_active=-2.0, hydro_screening=0.3, shape=0.4,
                                                volume_exclusion=0.1), 40_000, 13),
    ((64, 48, 1, 32, 1), (20.0, 15.0, 1.0), dict(timestep=0.002, trans_diffusion=0.05, rot_diffusion=2.0,
                                                   stress_active=-0.5, stress_magnetic=0.3,
                                                   magnetic_reorientation=0.7), 150_000, 14),
    ((32, 32, 1, 16, 1), (10.0, 10.0, 1.0), dict(timestep=0.01, trans_diffusion=0.1, rot_diffusion=0.5,
                                                   stress_active=-3.0), 5_000, 15),
    ((7, 9, 1, 5, 1), (3.5, 4.5, 1.0), dict(timestep=0.01, trans_diffusion=0.3, rot_diffusion=0.3,
                                              stress_active=1.0), 3_000, 16),
]


# flow after one step against the FP64 oracle: 2e-6 when the member's FP32
# histogram equals the oracle's (measured 3e-7 .. 4.5e-7); when the FP32
# binning put a few particles at bin edges into the neighbouring bin, the
# flow (driven by the density fluctuations) moves with them (measured 2.4e-3
# for 150,000 particles)
ENS_FLOW_TOL_EXACT = 2e-6
ENS_FLOW_TOL_EDGE = 1e-2


def _members(spec=MEMBERS):
    return [dict(grid=g, box=b, params=dict(p, number_of_particles=n, seed=s)) for g, b, p, n, s in spec]


def _rows(rng, members):
    from stochasticsampling_gb300.ensemble import uniform_particles
    return uniform_particles(members, seed=int(rng.integers(1 << 30)))


def _single(ss, m):
    return ss.Simulation(grid=m["grid"], box=m["box"], params=m["params"], quasi2d=True, mixed=True)


def _wrapdiff(a, b, period):
    d = np.abs(a - b)
    return np.minimum(d, period - d)


def test_ensemble_matches_single_contexts():
    ss = _gpu()
    members = _members()
    rows = _rows(np.random.default_rng(3), members)
    ens = ss.Ensemble(members)
    ens.init(rows)
    n, groups, _ = ens.info()
    assert n == sum(m["params"]["number_of_particles"] for m in members)
    assert groups == 4  # 32x32, 16x12, 64x48, 7x9
    singles = []
    for i, m in enumerate(members):
        s = _single(ss, m)
        s.init(rows[ens.offsets[i]:ens.offsets[i + 1]])
        assert np.array_equal(ens.get_counts(i), s.get_counts()), i
        singles.append(s)
    # one step from identical histograms: the fields agree to FFT round-off
    ens.run(1)
    for i, s in enumerate(singles):
        s.do_timestep()
        assert rel_l2(ens.get_flow_field(i), s.get_flow_field()) < 1e-5, i
        assert np.array_equal(ens.get_counts(i), s.get_counts()), i
    for s in singles:
        s.run(4)
    ens.run(4)
    for i, (m, s) in enumerate(zip(members, singles)):
        ep, sp = ens.get_particles(i), s.get_particles()
        nm = m["params"]["number_of_particles"]
        assert ep.shape == (nm, 5)
        assert np.all(ep[:, 2] == 0.0) and np.all(ep[:, 4] == np.pi / 2)
        dx = np.maximum(_wrapdiff(ep[:, 0], sp[:, 0], m["box"][0]), _wrapdiff(ep[:, 1], sp[:, 1], m["box"][1]))
        dphi = _wrapdiff(ep[:, 3], sp[:, 3], 2 * np.pi)
        # all but the particles that a rounding difference moved across a cell edge
        assert np.mean(dx > 1e-5) < 2e-3 and np.median(dx) < 1e-6, i
        assert np.mean(dphi > 1e-4) < 2e-3, i
        ce, cs = ens.get_counts(i).astype(np.int64), s.get_counts().astype(np.int64)
        assert ce.sum() == cs.sum() == nm
        assert np.abs(ce - cs).sum() <= max(4, 4e-3 * nm), i
    for s in singles:
        s.close()
    ens.close()


def test_ensemble_one_step_against_oracle(oracle):
    """Three members with uneven particle counts and grids, one ensemble step
    against oracle.Simulation (the FP64 restatement of the reference step)
    from the same rows, fed each member's own noise: the Philox stream of a
    stand-alone mixed context with the member's seed (ss_noise), which the
    ensemble draws for that member.  The mixed path's per-field bounds hold:
    the initial histogram differs only for particles within FP32 rounding of
    a bin edge, and the flow, positions (< 1e-8, measured <= 3.6e-9) and
    angles (< 1e-6 rad RMS, measured <= 2.7e-7) after the step are within the
    FP32 bounds of tests/test_gpu_mixed.py."""
    from test_gpu_parity import _pair
    ss = _gpu()
    spec = [MEMBERS[0], MEMBERS[2], MEMBERS[3]]
    members = _members(spec)
    rows = _rows(np.random.default_rng(17), members)
    ens = ss.Ensemble(members)
    ens.init(rows)
    oracles, same_hist = [], []
    for i, (grid, box, params, n, seed) in enumerate(spec):
        r = rows[ens.offsets[i]:ens.offsets[i + 1]]
        g, o, st = _pair(oracle, (f"member{i}", grid, box, params, n, True), seed=seed, mixed=True)
        g.init(r)
        noise = g.noise(0)
        g.close()
        o.init(r)
        h = oracle.histogram(st, o.particles()).ravel()
        c = ens.get_counts(i).astype(np.float64).ravel()
        assert c.sum() == n and np.abs(c - h).sum() <= 2e-3 * n, i
        same_hist.append(bool(np.array_equal(c, h)))
        o.do_timestep(noise)
        oracles.append(o)
    ens.run(1)
    for i, ((grid, box, params, n, seed), o) in enumerate(zip(spec, oracles)):
        eu = rel_l2(ens.get_flow_field(i), o.flow().real)
        ep, op = ens.get_particles(i), o.particles()
        ex = rel_l2(ep[:, :2], op[:, :2])
        ephi = float(np.sqrt(np.mean(_wrapdiff(ep[:, 3], op[:, 3], 2 * np.pi) ** 2)))
        print(f"ensemble member {i} vs oracle: flow {eu:.3e} positions {ex:.3e} phi rms {ephi:.3e}")
        assert eu < (ENS_FLOW_TOL_EXACT if same_hist[i] else ENS_FLOW_TOL_EDGE), (i, eu, same_hist[i])
        assert ex < 1e-8, (i, ex)
        assert ephi < 1e-6, (i, ephi)
        assert np.all(ep[:, 2] == 0.0) and np.all(ep[:, 4] == np.pi / 2)
    ens.close()


def test_ensemble_deterministic_and_autotune_leaves_state():
    ss = _gpu()
    members = _members()
    rows = _rows(np.random.default_rng(5), members)
    a = ss.Ensemble(members)
    a.init(rows)
    before = [a.get_particles(i) for i in range(len(members))]
    threads, bps, unit, plan = a.autotune()
    assert threads in (128, 256, 512) and bps in (2, 4, 8) and unit in (4096, 16384, 65536) and plan in (1, 2, 3)
    for i in range(len(members)):
        assert np.array_equal(a.get_particles(i), before[i])
    a.run(3)
    # another launch shape gives the same trajectory, bit for bit
    b = ss.Ensemble(members)
    b.init(rows)
    b.set_config((128, 2, 4096, 3) if plan != 3 else (512, 8, 65536, 1))
    b.run(3)
    for i in range(len(members)):
        assert np.array_equal(a.get_particles(i), b.get_particles(i))
        assert np.array_equal(a.get_counts(i), b.get_counts(i))
    _, _, launches = a.info()
    assert launches > 0
    a.close()
    b.close()


def test_ensemble_invariants_over_steps():
    ss = _gpu()
    members = _members()
    rows = _rows(np.random.default_rng(7), members)
    ens = ss.Ensemble(members)
    ens.init(rows)
    for _ in range(3):
        ens.run(2)
        for i, m in enumerate(members):
            c = ens.get_counts(i)
            assert int(c.sum()) == m["params"]["number_of_particles"]
            p = ens.get_particles(i)
            assert np.all((p[:, 0] >= 0) & (p[:, 0] < m["box"][0]))
            assert np.all((p[:, 1] >= 0) & (p[:, 1] < m["box"][1]))
            assert np.all((p[:, 3] >= 0) & (p[:, 3] < 2 * np.pi))
    ens.close()


def test_ensemble_errors():
    ss = _gpu()
    members = _members()
    ens = ss.Ensemble(members)
    rows = _rows(np.random.default_rng(9), members)
    with pytest.raises(ss.SsError):
        ens.init(rows[:-1])
    bad = rows.copy()
    bad[5, 4] = 1.0  # theta != pi/2
    with pytest.raises(ss.SsError):
        ens.init(bad)
    bad = rows.copy()
    bad[7, 2] = 0.5  # z != 0
    with pytest.raises(ss.SsError):
        ens.init(bad)
    with pytest.raises(ss.SsError):
        ens.run(1)  # not initialised
    ens.init(rows)
    ens.run(1)
    with pytest.raises(IndexError):
        ens.get_particles(len(members))
    from stochasticsampling_gb300 import _lib
    out = np.empty((10, 5))
    rc = ens.lib.ss_ensemble_get_particles(ens._h, len(members), out.ctypes.data_as(_lib.ctypes.POINTER(_lib.ctypes.c_double)))
    assert rc == _lib.SS_ERR_INVALID_ARGUMENT
    ens.close()


def test_ensemble_parameter_scan_full_size():
    """64 members, particle counts log-uniform in [50k, 2M], grid edges from
    {32, 64, 128} with 16 or 32 phi bins, active stress uniform in [-3, 0]:
    every histogram keeps its particles, and three members (smallest,
    largest, one between) follow their stand-alone contexts."""
    ss = _gpu()
    from stochasticsampling_gb300.ensemble import parameter_scan, uniform_particles
    members = parameter_scan(64, seed=1)
    rows = uniform_particles(members, seed=2)
    ens = ss.Ensemble(members)
    ens.init(rows)
    ens.run(5)
    for i, m in enumerate(members):
        assert int(ens.get_counts(i).sum()) == m["params"]["number_of_particles"]
    ns = np.array([m["params"]["number_of_particles"] for m in members])
    for i in (int(np.argmin(ns)), int(np.argmax(ns)), int(np.argsort(ns)[32])):
        m = members[i]
        s = _single(ss, m)
        s.init(rows[ens.offsets[i]:ens.offsets[i + 1]])
        s.run(5)
        ep, sp = ens.get_particles(i), s.get_particles()
        dx = np.maximum(_wrapdiff(ep[:, 0], sp[:, 0], m["box"][0]), _wrapdiff(ep[:, 1], sp[:, 1], m["box"][1]))
        assert np.mean(dx > 1e-5) < 2e-3 and np.median(dx) < 1e-6, i
        s.close()
    ens.close()
