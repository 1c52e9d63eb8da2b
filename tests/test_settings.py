"""The parameter.toml schema: src/bin/simulation/settings/mod.rs:227-384."""
import pytest

from stochasticsampling_gb300.settings import (DEFAULT_IO_QUEUE_SIZE, DEFAULT_OUTPUT_FORMAT, SettingsError,
                                               parse_settings, read_parameter_file, to_toml)

FULL = """
[environment]
    init_file = "foo/bar.cbor"
    io_queue_size = 50
    output_format = "Bincode"
    prefix = "foo"
[simulation]
    init_distribution = "Homogeneous"
    number_of_particles = 100
    number_of_timesteps = 500
    timestep = 0.1
    seed = 1
    [simulation.box_size]
        x = 1.0
        y = 2.0
        z = 3.0
    [simulation.grid_size]
        x = 11
        y = 12
        z = 13
        phi = 6
        theta = 7
    [simulation.output_at_timestep]
        distribution = 12
        flowfield = 42
        magneticfield = 41
        particles = 100
        particles_head = 10
        snapshot = 666
        initial_condition = false
        final_snapshot = false
[parameters]
    magnetic_drag = 123.4
    shape = 44.3
    volume_exclusion = 265.6
    magnetic_reorientation = 1.0
    hydro_screening = 1.3
    [parameters.magnetic_dipole]
        magnetic_dipole_dipole = 5.0
    [parameters.diffusion]
        rotational = 0.5
        translational = 1.0
    [parameters.stress]
        active = 1.0
        magnetic = 1.0
"""

MINIMAL = """
[environment]
    prefix = "foo"
[simulation]
    number_of_particles = 100
    number_of_timesteps = 500
    timestep = 0.1
    seed = 1
    [simulation.box_size]
        x = 1.0
        y = 2.0
        z = 3.0
    [simulation.grid_size]
        x = 11
        y = 12
        z = 13
        phi = 6
        theta = 7
    [simulation.output_at_timestep]
[parameters]
    magnetic_reorientation = 1.0
    [parameters.magnetic_dipole]
    [parameters.diffusion]
        rotational = 0.5
        translational = 1.0
    [parameters.stress]
        active = 1.0
        magnetic = 1.0
"""


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_read_settings(tmp_path):
    s = read_parameter_file(_write(tmp_path, "parameter.toml", FULL))
    s.set_version("version")
    d = read_parameter_file(_write(tmp_path, "no_defaults.toml", MINIMAL))
    assert d.environment.init_file is None
    assert s.environment.init_file == "foo/bar.cbor"
    assert d.environment.io_queue_size == DEFAULT_IO_QUEUE_SIZE
    assert s.environment.io_queue_size == 50
    assert d.environment.output_format == DEFAULT_OUTPUT_FORMAT
    assert s.environment.output_format == "Bincode"
    assert s.environment.prefix == "foo"
    assert s.environment.version == "version"
    assert s.parameters.diffusion.rotational == 0.5
    assert s.parameters.diffusion.translational == 1.0
    assert s.parameters.stress.active == 1.0 and s.parameters.stress.magnetic == 1.0
    assert s.parameters.magnetic_dipole.magnetic_dipole_dipole == 5.0
    assert d.parameters.magnetic_dipole.magnetic_dipole_dipole == 0.0
    assert s.parameters.magnetic_reorientation == 1.0
    assert s.parameters.magnetic_drag == 123.4 and d.parameters.magnetic_drag == 0.0
    assert s.parameters.shape == 44.3
    assert d.parameters.hydro_screening == 0.0 and s.parameters.hydro_screening == 1.3
    assert d.parameters.volume_exclusion == 0.0 and s.parameters.volume_exclusion == 265.6
    assert (s.simulation.box_size.x, s.simulation.box_size.y, s.simulation.box_size.z) == (1.0, 2.0, 3.0)
    g = s.simulation.grid_size
    assert (g.x, g.y, g.z, g.phi, g.theta) == (11, 12, 13, 6, 7)
    assert s.simulation.init_distribution == "Homogeneous"
    assert d.simulation.init_distribution == "Isotropic"
    assert s.simulation.number_of_particles == 100 and s.simulation.number_of_timesteps == 500
    assert s.simulation.timestep == 0.1 and s.simulation.seed == 1
    o, od = s.simulation.output_at_timestep, d.simulation.output_at_timestep
    assert o.distribution == 12 and od.distribution is None
    assert od.final_snapshot is True and o.final_snapshot is False
    assert o.flowfield == 42 and od.flowfield is None
    assert o.magneticfield == 41 and od.magneticfield is None
    assert o.particles == 100 and od.particles is None
    assert o.particles_head == 10 and od.particles_head is None
    assert od.initial_condition is True and o.initial_condition is False
    assert o.snapshot == 666 and od.snapshot is None


def test_settings_unused_keys(tmp_path):
    # test_settings_unused_keys: an unknown key in [simulation] is rejected
    bad = MINIMAL.replace("number_of_particles = 100", "non_existing_key = 10\n    number_of_particles = 100")
    with pytest.raises(SettingsError, match="unknown field"):
        read_parameter_file(_write(tmp_path, "unused.toml", bad))


@pytest.mark.parametrize("edit,msg", [
    (("x = 1.0", "x = 0.0"), "Box size is invalid"),
    (("[simulation.output_at_timestep]", "[simulation.output_at_timestep]\n        particles_head = 101"),
     "Cannot output more particles"),
    (("prefix = \"foo\"", "prefix = \"foo\"\n    output_format = \"Json\""), "unknown variant"),
    (("timestep = 0.1", "timestep = \"a\""), "expected a float"),
    (("seed = 1", "seed = [1, 1]"), "non-negative integer"),
    (("magnetic_reorientation = 1.0", ""), "missing field"),
])
def test_settings_rejected(tmp_path, edit, msg):
    with pytest.raises(SettingsError, match=msg):
        read_parameter_file(_write(tmp_path, "bad.toml", MINIMAL.replace(*edit, 1)))


def test_roundtrip_without_version(tmp_path):
    import tomllib
    s = read_parameter_file(_write(tmp_path, "parameter.toml", FULL))
    doc = tomllib.loads(to_toml(s))
    # `version` is written but, like serde skip_deserializing under
    # deny_unknown_fields, not accepted back
    with pytest.raises(SettingsError, match="unknown field `version`"):
        parse_settings(doc)
    del doc["environment"]["version"]
    s2 = parse_settings(doc)
    assert s2 == s


SI = FULL.split("[parameters]")[0] + """
[parameters]
    hydro_screening = 0.0
    volume_exclusion = 0.0
    viscocity = 1e-3
    temperature = 300
    volume_fraction = 1e-2
    external_field = 1e-3
    [parameters.particle]
        radius = 1e-6
        self_propulsion_speed = 1e-4
        force_dipole = 1.88496e-18
        magnetic_dipole_moment = 1e-15
        persistance_time = 0.75
"""


def test_si_conversion(tmp_path):
    # SettingsSI::into_settings, src/bin/simulation/settings/si.rs:126-199
    import math
    from stochasticsampling_gb300.settings import read_parameter_file_si
    s = read_parameter_file_si(_write(tmp_path, "si.toml", SI.replace("x = 1.0\n", "x = 1.0e-4\n", 1)))
    r, v, eta, T, phi, B, m, tau = 1e-6, 1e-4, 1e-3, 300.0, 1e-2, 1e-3, 1e-15, 0.75
    n = phi / (4 / 3 * math.pi * r ** 3)
    xc = n ** (-1 / 3)
    kT = 1.38064852e-23 * T
    fr, ft = 8 * math.pi * eta * r ** 3, 6 * math.pi * eta * r
    dr = n ** (-1 / 3) / v * (kT / fr + 1 / (2 * tau))
    assert math.isclose(s.parameters.diffusion.rotational, dr, rel_tol=1e-12)
    assert math.isclose(s.parameters.diffusion.translational, n ** (1 / 3) / v * kT / ft, rel_tol=1e-12)
    assert math.isclose(s.parameters.stress.active, n ** (2 / 3) / v / eta * 1.88496e-18, rel_tol=1e-12)
    assert math.isclose(s.parameters.stress.magnetic, n ** (2 / 3) / v / eta * m * B, rel_tol=1e-12)
    assert math.isclose(s.parameters.magnetic_reorientation, m * B / fr / (kT / fr + 1 / (2 * tau)) * dr,
                        rel_tol=1e-12)
    assert math.isclose(s.parameters.magnetic_drag, n / v / ft * 4e-7 * math.pi * m * m, rel_tol=1e-12)
    assert math.isclose(s.simulation.box_size.x, 1.0e-4 / xc, rel_tol=1e-12)
    assert math.isclose(s.simulation.timestep, 0.1 / (xc / v), rel_tol=1e-12)
    assert s.simulation.grid_size.x == 11 and s.environment.prefix == "foo"


def test_si_requires_every_parameter(tmp_path):
    # the SI parameters table has no defaults (si.rs:62-73)
    from stochasticsampling_gb300.settings import read_parameter_file_si
    with pytest.raises(SettingsError, match="missing field `hydro_screening`"):
        read_parameter_file_si(_write(tmp_path, "si.toml", SI.replace("    hydro_screening = 0.0\n", "")))
