"""ss_step_host: one step of host-resident particles in one call (the rows
replace the state, the step runs, the new state comes back), with the
chunked update overlapping the read-back.  It must give exactly what
ss_resume + ss_do_timestep + ss_get_particles give."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GRID = (32, 32, 1, 16, 1)
BOX = (10.0, 10.0, 1.0)
PARAMS = dict(timestep=0.01, trans_diffusion=0.1, rot_diffusion=0.5, stress_active=-1.0, shape=0.3)


def _gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import stochasticsampling_gb300 as ss
    return ss


def _rows(rng, n, canonical=True):
    th = np.full(n, np.pi / 2) if canonical else np.arccos(1 - 2 * rng.random(n))
    z = np.zeros(n) if canonical else rng.random(n)
    return np.column_stack([BOX[0] * rng.random(n), BOX[1] * rng.random(n), z, 2 * np.pi * rng.random(n), th])


@pytest.mark.parametrize("n", [100_003, 1_000_000], ids=["ragged", "1e6"])
@pytest.mark.parametrize("flags", [dict(), dict(sort=False), dict(sort=False, f32x2=True), dict(mixed=True),
                                   dict(mixed="fixed64")],
                         ids=["fp64_sort", "fp64", "f32x2", "mixed", "fixed64"])
def test_step_host_equals_resume_step_get(n, flags):
    ss = _gpu()
    rng = np.random.default_rng(5)
    p = _rows(rng, n)
    mk = lambda: ss.Simulation(grid=GRID, box=BOX, params=dict(PARAMS, number_of_particles=n, seed=11),
                               quasi2d=True, **flags)
    a, b = mk(), mk()
    a.init(p)
    b.init(p)
    cur = p.copy()
    for t in range(3):
        a.resume(cur, t)
        a.do_timestep()
        ref = a.get_particles()
        got = b.step_host(cur)
        assert b.get_timestep() == t + 1
        assert np.array_equal(got, ref), t
        assert np.array_equal(a.get_counts(), b.get_counts()), t
        assert np.array_equal(a.get_flow_field(), b.get_flow_field()), t
        cur = ref
    # graph-replayed steps after the host steps (the state now lives in the
    # other particle buffer of b)
    a.run(2)
    b.run(2)
    assert np.array_equal(a.get_particles(), b.get_particles())
    assert np.array_equal(a.get_counts(), b.get_counts())
    a.close()
    b.close()


def test_step_host_in_place_and_off_canonical_rows():
    ss = _gpu()
    n = 300_000
    rng = np.random.default_rng(6)
    p = _rows(rng, n, canonical=False)
    mk = lambda: ss.Simulation(grid=GRID, box=BOX, params=dict(PARAMS, number_of_particles=n, seed=12),
                               quasi2d=True)
    a, b = mk(), mk()
    a.init(p)
    b.init(p)
    buf = p.copy()
    for t in range(3):
        a.resume(buf if t else p, t)
        a.do_timestep()
        ref = a.get_particles()
        b.step_host(buf, out=buf)  # in place
        assert np.array_equal(buf, ref), t
        # every step writes the canonical quasi-2-D state
        assert np.all(buf[:, 2] == 0.0) and np.all(buf[:, 4] == np.pi / 2)
    a.close()
    b.close()


def test_step_host_rejects_bad_rows_and_keeps_state():
    ss = _gpu()
    n = 10_000
    rng = np.random.default_rng(7)
    p = _rows(rng, n)
    g = ss.Simulation(grid=GRID, box=BOX, params=dict(PARAMS, number_of_particles=n, seed=13), quasi2d=True)
    g.init(p)
    g.run(2)
    before, t0 = g.get_particles(), g.get_timestep()
    bad = p.copy()
    bad[123, 1] = np.nan
    with pytest.raises(Exception, match="non-finite"):
        g.step_host(bad)
    assert g.get_timestep() == t0
    assert np.array_equal(g.get_particles(), before)
    with pytest.raises(Exception):
        g.step_host(p[:-1])  # wrong particle count
    with pytest.raises(ValueError):
        g.step_host(p, out=np.empty((n, 5), dtype=np.float32))
    with pytest.raises(ValueError):
        g.get_particles(out=np.empty((n, 4)))
    g.close()


def test_step_host_with_stage_timing():
    """With per-stage timing on, ss_step_host runs as resume + step + read-back."""
    ss = _gpu()
    n = 50_000
    rng = np.random.default_rng(8)
    p = _rows(rng, n)
    mk = lambda: ss.Simulation(grid=GRID, box=BOX, params=dict(PARAMS, number_of_particles=n, seed=14),
                               quasi2d=True, sort=False)
    a, b = mk(), mk()
    a.init(p)
    b.init(p)
    b.profile(True)
    a.resume(p, 0)
    a.do_timestep()
    assert np.array_equal(b.step_host(p), a.get_particles())
    ms, steps = b.profile_read()
    assert steps == 1 and ms["update"] > 0
    b.profile(False)
    a.close()
    b.close()
