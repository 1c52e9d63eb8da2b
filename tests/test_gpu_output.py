"""ss_output_begin / ss_output_wait: the outputs of a step, taken on the
device and transferred while later steps run, equal what the blocking getters
return at that step, bit for bit, in every mode; the slot rules; and the
driver writes the same files with and without the overlap."""
import numpy as np
import pytest

from stochasticsampling_gb300 import output as io

from test_gpu_parity import _gpu

pytestmark = pytest.mark.gpu

PARAMS = dict(timestep=0.01, trans_diffusion=0.1, rot_diffusion=0.5, stress_active=-1.0, shape=0.3)

CASES = [
    ("fp64_2d", (32, 32, 1, 16, 1), (10.0, 10.0, 1.0), dict(quasi2d=True), PARAMS),
    ("mixed_2d", (32, 32, 1, 16, 1), (10.0, 10.0, 1.0), dict(quasi2d=True, mixed=True), PARAMS),
    ("fixed64_2d", (32, 32, 1, 16, 1), (10.0, 10.0, 1.0), dict(quasi2d=True, mixed="fixed64"), PARAMS),
    ("fp64_3d_dipolar", (16, 16, 16, 8, 4), (5.0, 5.0, 5.0), dict(),
     dict(PARAMS, magnetic_reorientation=1.0, magnetic_dipole_dipole=0.5)),
    ("mixed_3d_mag_on_demand", (16, 16, 16, 8, 4), (5.0, 5.0, 5.0), dict(mixed=True), PARAMS),
]


def _rows(rng, n, box, q2d):
    th = np.full(n, np.pi / 2) if q2d else np.arccos(1 - 2 * rng.random(n))
    z = np.zeros(n) if q2d else box[2] * rng.random(n)
    return np.column_stack([box[0] * rng.random(n), box[1] * rng.random(n), z, 2 * np.pi * rng.random(n), th])


def _blocking(sim, head):
    return (sim.get_distribution(), sim.get_flow_field(), sim.get_magnetic_field(), sim.get_particles_head(head))


@pytest.mark.parametrize("name,grid,box,flags,params", CASES, ids=[c[0] for c in CASES])
def test_overlapped_outputs_equal_the_getters(name, grid, box, flags, params):
    ss = _gpu()
    n = 50_003
    rng = np.random.default_rng(21)
    q2d = flags.get("quasi2d", False)
    sim = ss.Simulation(grid=grid, box=box, params=dict(params, number_of_particles=n, seed=5), **flags)
    sim.init(_rows(rng, n, box, q2d))
    fshape = (3,) + grid[:3]
    bufs = [[sim.host_array(grid), sim.host_array(fshape), sim.host_array(fshape), sim.host_array((n, 5))]
            for _ in range(2)]
    sim.run(2)
    want0 = _blocking(sim, n)
    sim.output_begin(0, *[b.array for b in bufs[0]])
    sim.run(3)  # these steps overwrite the state while slot 0 is in flight
    sim.output_begin(1, bufs[1][0].array, bufs[1][1].array, None, bufs[1][3].array[:1000])
    sim.run(2)
    sim.output_wait(0)
    for got, want in zip(bufs[0], want0):
        assert np.array_equal(got.array, want)
    sim.output_wait(1)
    assert sim.output_ready(0) and sim.output_ready(1)
    # slot 1 holds step 5; replay a second context to step 5 for the blocking values
    ref = ss.Simulation(grid=grid, box=box, params=dict(params, number_of_particles=n, seed=5), **flags)
    ref.init(_rows(np.random.default_rng(21), n, box, q2d))
    ref.run(5)
    want1 = _blocking(ref, 1000)
    assert np.array_equal(bufs[1][0].array, want1[0])
    assert np.array_equal(bufs[1][1].array, want1[1])
    assert np.array_equal(bufs[1][3].array[:1000], want1[3])
    assert sim.get_timestep() == 7
    sim.close()
    ref.close()
    for pair in bufs:
        for b in pair:
            b.close()


def test_output_slot_rules():
    ss = _gpu()
    from stochasticsampling_gb300._lib import SS_ERR_INVALID_ARGUMENT, SS_ERR_STATE, SsError
    grid, box = (16, 16, 1, 8, 1), (4.0, 4.0, 1.0)
    n = 1000
    sim = ss.Simulation(grid=grid, box=box, params=dict(PARAMS, number_of_particles=n, seed=2), quasi2d=True)
    d = sim.host_array(grid)
    with pytest.raises(SsError) as e:  # before init
        sim.output_begin(0, dist=d.array)
    assert e.value.code == SS_ERR_STATE
    sim.init(_rows(np.random.default_rng(0), n, box, True))
    assert sim.output_ready(0)
    sim.output_wait(0)  # nothing in flight: returns at once
    sim.output_begin(0, dist=d.array)
    with pytest.raises(SsError) as e:  # slot still in flight
        sim.output_begin(0, dist=d.array)
    assert e.value.code == SS_ERR_STATE
    with pytest.raises(SsError) as e:
        sim.output_begin(2, dist=d.array)
    assert e.value.code == SS_ERR_INVALID_ARGUMENT
    sim.output_wait(0)
    assert np.array_equal(d.array, sim.get_distribution())
    # pageable host memory works too (the runtime stages the copy)
    rows = np.empty((10, 5))
    sim.output_begin(1, particles=rows)
    sim.output_wait(1)
    assert np.array_equal(rows, sim.get_particles_head(10))
    with pytest.raises(ValueError):
        sim.output_begin(0, dist=np.empty((3, 3)))
    sim.close()
    d.close()


def test_driver_overlap_writes_the_same_files(tmp_path):
    _gpu()
    from stochasticsampling_gb300 import driver
    from test_gpu_driver import _settings
    s = _settings()
    out = {}
    for overlap in (False, True):
        root = tmp_path / str(overlap)
        root.mkdir()
        path = driver.run(s, str(root), quasi2d=True, overlap=overlap)
        header, entries = io.read_output(path)
        import glob
        snaps = sorted(glob.glob(str(root / "*" / "*.snapshot.*.msgpack-lzma")))
        out[overlap] = ([io.packb(e) for e in entries], [io.read_particles_file(f) for f in snaps])
    assert out[True][0] == out[False][0]
    assert len(out[True][1]) == len(out[False][1]) == 2
    for (pa, ta), (pb, tb) in zip(out[True][1], out[False][1]):
        assert ta == tb and np.array_equal(pa, pb)
