"""The driver (src/bin/main.rs run_simulation), the initial-condition
samplers and snapshot resume, on the GPU."""
import numpy as np
import pytest

from stochasticsampling_gb300 import output as io

from test_gpu_parity import _gpu

pytestmark = pytest.mark.gpu

TOML = """
[environment]
    prefix = "drv"
    io_queue_size = 2
[simulation]
    number_of_particles = 4000
    number_of_timesteps = 6
    timestep = 0.01
    seed = 3
    init_distribution = "{init}"
    [simulation.box_size]
        x = 8.0
        y = 8.0
        z = 1.0
    [simulation.grid_size]
        x = 16
        y = 16
        z = 1
        phi = 8
        theta = 1
    [simulation.output_at_timestep]
        distribution = 2
        flowfield = 3
        magneticfield = 3
        particles = 2
        particles_head = 10
        snapshot = 4
[parameters]
    magnetic_reorientation = 0.5
    [parameters.magnetic_dipole]
    [parameters.diffusion]
        rotational = 0.5
        translational = 0.1
    [parameters.stress]
        active = -1.0
        magnetic = 0.0
"""


def _settings(init="Isotropic"):
    import tomllib
    from stochasticsampling_gb300.settings import parse_settings
    return parse_settings(tomllib.loads(TOML.format(init=init)))


def test_run_writes_reference_layout(tmp_path):
    ss = _gpu()
    from stochasticsampling_gb300 import driver
    s = _settings()
    path = driver.run(s, str(tmp_path), quasi2d=True)
    header, entries = io.read_output(path)
    assert header["simulation"]["number_of_particles"] == 4000
    # initial entry, then steps 2, 3, 4, 6 (distribution every 2, flow every 3); 7 steps run (main.rs:178-182)
    assert [e["timestep"] for e in entries] == [0, 2, 3, 4, 6]
    first = entries[0]
    d = io.ndarray_from(first["distribution"]["dist"])
    gw = first["distribution"]["grid_width"]
    assert np.isclose(d.sum() * gw["x"] * gw["y"] * gw["z"] * gw["phi"] * gw["theta"], 8.0 * 8.0)
    assert np.asarray(first["particles"]).reshape(-1, 5).shape == (10, 5)  # particles_head
    e3 = entries[2]
    assert e3["distribution"] is None and e3["particles"] is None
    assert io.ndarray_from(e3["flowfield"]).shape == (3, 16, 16, 1)
    assert io.ndarray_from(e3["magneticfield"]).shape == (3, 16, 16, 1)
    import glob
    snaps = sorted(glob.glob(str(tmp_path / "*" / "*.snapshot.*.msgpack-lzma")))
    assert len(snaps) == 2  # step 4 and the final snapshot (step 7)
    parts, ts = io.read_particles_file(snaps[-1])
    assert ts == 7 and parts.shape == (4000, 5)


def test_resume_from_snapshot_file(tmp_path):
    ss = _gpu()
    from stochasticsampling_gb300 import driver
    s = _settings()
    a = driver.init_simulation(s, quasi2d=True)
    a.run(3)
    f = str(tmp_path / "snap.msgpack-lzma")
    with open(f, "wb") as fh:
        import lzma
        fh.write(lzma.compress(io.packb(io.snapshot_record(a.get_particles(), a.get_timestep())), preset=1))
    a.run(4)
    b = driver.init_simulation(s, resume=f, quasi2d=True)
    assert b.get_timestep() == 3
    b.run(4)
    assert np.array_equal(a.get_particles(), b.get_particles())
    a.close()
    b.close()


def test_isotropic_sampler():
    ss = _gpu()
    s = _settings()
    s.simulation.number_of_particles = 200_000
    s.simulation.grid_size.z = 4
    s.simulation.grid_size.theta = 4
    s.simulation.box_size.z = 2.0
    g = ss.Simulation(s)
    g.init_distribution("Isotropic")
    p = g.get_particles()
    box = (8.0, 8.0, 2.0)
    se = 5 / np.sqrt(len(p))
    for k in range(3):
        assert np.all((p[:, k] >= 0) & (p[:, k] < box[k]))
        assert abs(p[:, k].mean() / box[k] - 0.5) < se
    assert abs(np.cos(p[:, 4]).mean()) < se  # uniform on the sphere: <cos theta> = 0
    assert abs((np.cos(p[:, 4]) ** 2).mean() - 1 / 3) < se
    assert g.get_counts().sum() == len(p)
    g.close()


def test_homogeneous_sampler():
    ss = _gpu()
    s = _settings("Homogeneous")
    s.simulation.number_of_particles = 200_000
    g = ss.Simulation(s)
    kappa = 0.5 / 0.5
    g.init_distribution("Homogeneous")
    p = g.get_particles()
    # orientations follow exp(kappa n_y) (rotated from the z axis onto y, particle.rs:271-276):
    # <n_y> = coth(kappa) - 1/kappa
    ny = np.sin(p[:, 4]) * np.sin(p[:, 3])
    assert abs(ny.mean() - (1 / np.tanh(kappa) - 1 / kappa)) < 5 / np.sqrt(len(p))
    g.close()
    s.parameters.magnetic_reorientation = 0.0
    g = ss.Simulation(s)
    with pytest.raises(ss.SsError, match="Alignment of zero"):
        g.init_distribution("Homogeneous")
    g.close()
