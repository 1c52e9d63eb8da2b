"""ss_set_resort: a counting sort of the resident particles by cell every K
steps.  It must change no result: after the same steps, the particles (read
back in the caller's order) and the histogram equal those of a context that
never re-sorts, bit for bit, for every mode, through CUDA graphs and direct
steps alike."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GRID2 = (32, 32, 1, 16, 1)
BOX2 = (10.0, 10.0, 1.0)
GRID3 = (16, 16, 16, 8, 4)
BOX3 = (5.0, 5.0, 5.0)
PARAMS = dict(timestep=0.01, trans_diffusion=0.1, rot_diffusion=0.5, stress_active=-1.0, shape=0.3)
PARAMS3 = dict(PARAMS, magnetic_reorientation=1.0, magnetic_dipole_dipole=0.5)


def _gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import stochasticsampling_gb300 as ss
    return ss


def _rows(rng, n, box, canonical):
    th = np.full(n, np.pi / 2) if canonical else np.arccos(1 - 2 * rng.random(n))
    z = np.zeros(n) if canonical else box[2] * rng.random(n)
    return np.column_stack([box[0] * rng.random(n), box[1] * rng.random(n), z, 2 * np.pi * rng.random(n), th])


CASES = [
    ("mixed_2d", dict(mixed=True), True),
    ("fixed64_2d", dict(mixed="fixed64"), True),
    ("mixed_3d", dict(mixed=True), False),
    ("fp64_2d_nosort", dict(sort=False), True),
    ("fp64_3d_nosort", dict(sort=False), False),
    ("f32x2_3d", dict(sort=False, f32x2=True), False),
]


@pytest.mark.parametrize("name,flags,q2d", CASES, ids=[c[0] for c in CASES])
def test_resort_changes_no_result(name, flags, q2d):
    ss = _gpu()
    rng = np.random.default_rng(8)
    n = 60_011
    grid, box, params = (GRID2, BOX2, PARAMS) if q2d else (GRID3, BOX3, PARAMS3)
    p = _rows(rng, n, box, canonical=q2d)
    mk = lambda: ss.Simulation(grid=grid, box=box, params=dict(params, number_of_particles=n, seed=13),
                               quasi2d=q2d, **flags)
    a, b = mk(), mk()
    a.init(p)
    b.init(p)
    b.set_resort(2)
    # graph-replayed steps, then direct steps (the profiled path runs them one by one)
    a.run(5)
    b.run(5)
    a.profile(True)
    b.profile(True)
    for _ in range(3):
        a.do_timestep()
        b.do_timestep()
    sort_ms = b.profile_read()[0]["sort"]
    assert np.array_equal(a.get_particles(), b.get_particles())
    assert np.array_equal(a.get_counts(), b.get_counts())
    assert a.get_timestep() == b.get_timestep() == 8
    # the re-sort ran: the sort stage has time in the context that re-sorts
    assert sort_ms > 0.0
    a.close()
    b.close()


def test_resort_rejects_null_context():
    ss = _gpu()
    lib = ss._lib.load()
    assert lib.ss_set_resort(None, 2) != 0
