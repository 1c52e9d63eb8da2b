"""The reference's ``parameter.toml`` schema (src/bin/simulation/settings/mod.rs).

``read_parameter_file`` mirrors ``read_parameter_file`` (mod.rs:171-183): every
table rejects unknown keys (serde ``deny_unknown_fields``), optional keys take
the reference defaults, and ``check_settings`` (mod.rs:185-205) runs last.
Errors raise ``SettingsError``.
"""
import dataclasses
import tomllib
from dataclasses import dataclass, field
from typing import Optional

DEFAULT_IO_QUEUE_SIZE = 1          # mod.rs:13
DEFAULT_OUTPUT_FORMAT = "MsgPack"  # mod.rs:14
DEFAULT_INIT_TYPE = "Isotropic"    # mod.rs:15
OUTPUT_FORMATS = ("CBOR", "Bincode", "MsgPack")
INIT_DISTRIBUTIONS = ("Isotropic", "Homogeneous")


class SettingsError(ValueError):
    pass


@dataclass
class BoxSize:
    x: float
    y: float
    z: float


@dataclass
class GridSize:
    x: int
    y: int
    z: int
    phi: int
    theta: int


@dataclass
class DiffusionConstants:
    translational: float
    rotational: float


@dataclass
class StressPrefactors:
    active: float
    magnetic: float


@dataclass
class MagneticDipolePrefactors:
    magnetic_dipole_dipole: float = 0.0


@dataclass
class Parameters:
    magnetic_reorientation: float
    diffusion: DiffusionConstants
    stress: StressPrefactors
    magnetic_dipole: MagneticDipolePrefactors
    magnetic_drag: float = 0.0
    shape: float = 0.0
    hydro_screening: float = 0.0
    volume_exclusion: float = 0.0


@dataclass
class Output:
    initial_condition: bool = True
    final_snapshot: bool = True
    distribution: Optional[int] = None
    flowfield: Optional[int] = None
    magneticfield: Optional[int] = None
    particles_head: Optional[int] = None
    particles: Optional[int] = None
    snapshot: Optional[int] = None


@dataclass
class SimulationSettings:
    number_of_particles: int
    number_of_timesteps: int
    timestep: float
    seed: int
    output_at_timestep: Output
    box_size: BoxSize
    grid_size: GridSize
    init_distribution: str = DEFAULT_INIT_TYPE


@dataclass
class EnvironmentSettings:
    prefix: str
    init_file: Optional[str] = None
    io_queue_size: int = DEFAULT_IO_QUEUE_SIZE
    output_format: str = DEFAULT_OUTPUT_FORMAT
    version: str = ""  # skip_deserializing in the reference: never read from the file


@dataclass
class Settings:
    simulation: SimulationSettings
    parameters: Parameters
    environment: EnvironmentSettings

    def set_version(self, version):
        self.environment.version = version


def _num(v, where, integer=False):
    if isinstance(v, bool):
        raise SettingsError(f"{where}: expected a number, got a boolean")
    if integer:
        if not isinstance(v, int) or v < 0:
            raise SettingsError(f"{where}: expected a non-negative integer, got {v!r}")
        return int(v)
    if not isinstance(v, (int, float)):
        raise SettingsError(f"{where}: expected a float, got {v!r}")
    return float(v)


def _table(d, where, required, optional):
    if not isinstance(d, dict):
        raise SettingsError(f"{where}: expected a table")
    allowed = set(required) | set(optional)
    for k in d:
        if k not in allowed:
            raise SettingsError(f"unknown field `{k}` in {where}, expected one of {sorted(allowed)}")
    for k in required:
        if k not in d:
            raise SettingsError(f"missing field `{k}` in {where}")
    return d


def parse_settings(doc):
    """Build Settings from a parsed TOML document (dict)."""
    _table(doc, "settings", ["simulation", "parameters", "environment"], [])
    s = _table(doc["simulation"], "simulation",
               ["number_of_particles", "number_of_timesteps", "timestep", "seed", "output_at_timestep",
                "box_size", "grid_size"], ["init_distribution"])
    b = _table(s["box_size"], "simulation.box_size", ["x", "y", "z"], [])
    g = _table(s["grid_size"], "simulation.grid_size", ["x", "y", "z", "phi", "theta"], [])
    o = _table(s["output_at_timestep"], "simulation.output_at_timestep", [],
               [f.name for f in dataclasses.fields(Output)])
    out = Output()
    for k, v in o.items():
        if k in ("initial_condition", "final_snapshot"):
            if not isinstance(v, bool):
                raise SettingsError(f"output_at_timestep.{k}: expected a boolean")
            setattr(out, k, v)
        else:
            setattr(out, k, _num(v, f"output_at_timestep.{k}", integer=True))
    init = s.get("init_distribution", DEFAULT_INIT_TYPE)
    if init not in INIT_DISTRIBUTIONS:
        raise SettingsError(f"unknown variant `{init}`, expected one of {INIT_DISTRIBUTIONS}")
    sim = SimulationSettings(
        number_of_particles=_num(s["number_of_particles"], "number_of_particles", True),
        number_of_timesteps=_num(s["number_of_timesteps"], "number_of_timesteps", True),
        timestep=_num(s["timestep"], "timestep"),
        seed=_num(s["seed"], "seed", True),
        output_at_timestep=out,
        box_size=BoxSize(*[_num(b[k], f"box_size.{k}") for k in "xyz"]),
        grid_size=GridSize(*[_num(g[k], f"grid_size.{k}", True) for k in ("x", "y", "z", "phi", "theta")]),
        init_distribution=init,
    )
    p = _table(doc["parameters"], "parameters",
               ["magnetic_reorientation", "diffusion", "stress", "magnetic_dipole"],
               ["magnetic_drag", "shape", "hydro_screening", "volume_exclusion"])
    dif = _table(p["diffusion"], "parameters.diffusion", ["translational", "rotational"], [])
    st = _table(p["stress"], "parameters.stress", ["active", "magnetic"], [])
    md = _table(p["magnetic_dipole"], "parameters.magnetic_dipole", [], ["magnetic_dipole_dipole"])
    par = Parameters(
        magnetic_reorientation=_num(p["magnetic_reorientation"], "magnetic_reorientation"),
        diffusion=DiffusionConstants(_num(dif["translational"], "translational"),
                                     _num(dif["rotational"], "rotational")),
        stress=StressPrefactors(_num(st["active"], "active"), _num(st["magnetic"], "magnetic")),
        magnetic_dipole=MagneticDipolePrefactors(_num(md.get("magnetic_dipole_dipole", 0.0),
                                                      "magnetic_dipole_dipole")),
        magnetic_drag=_num(p.get("magnetic_drag", 0.0), "magnetic_drag"),
        shape=_num(p.get("shape", 0.0), "shape"),
        hydro_screening=_num(p.get("hydro_screening", 0.0), "hydro_screening"),
        volume_exclusion=_num(p.get("volume_exclusion", 0.0), "volume_exclusion"),
    )
    e = _table(doc["environment"], "environment", ["prefix"], ["init_file", "io_queue_size", "output_format"])
    fmt = e.get("output_format", DEFAULT_OUTPUT_FORMAT)
    if fmt not in OUTPUT_FORMATS:
        raise SettingsError(f"unknown variant `{fmt}`, expected one of {OUTPUT_FORMATS}")
    if not isinstance(e["prefix"], str):
        raise SettingsError("environment.prefix: expected a string")
    env = EnvironmentSettings(prefix=e["prefix"], init_file=e.get("init_file"),
                              io_queue_size=_num(e.get("io_queue_size", DEFAULT_IO_QUEUE_SIZE),
                                                 "io_queue_size", True),
                              output_format=fmt)
    settings = Settings(simulation=sim, parameters=par, environment=env)
    check_settings(settings)
    return settings


def check_settings(s):
    """check_settings, src/bin/simulation/settings/mod.rs:185-205."""
    bs = s.simulation.box_size
    if bs.x <= 0.0 or bs.y <= 0.0 or bs.z <= 0.0:
        raise SettingsError(f"Box size is invalid. Must be bigger than 0: {bs}")
    ph = s.simulation.output_at_timestep.particles_head
    if ph is not None and s.simulation.number_of_particles < ph:
        raise SettingsError("Cannot output more particles than available. `particles_head` must be smaller "
                            "or equal to `number_of_particles`")


def read_parameter_file(path):
    """read_parameter_file, src/bin/simulation/settings/mod.rs:171-183."""
    try:
        with open(path, "rb") as f:
            doc = tomllib.load(f)
    except OSError as exc:
        raise SettingsError(f"Unable to read parameter file: {exc}") from exc
    except tomllib.TOMLDecodeError as exc:
        raise SettingsError(f"Unable to parse parameter file: {exc}") from exc
    s = parse_settings(doc)
    s.environment.version = ""
    return s


# ---------------------------------------------------------------- SI units
BOLTZMANN = 1.38064852e-23  # src/bin/simulation/settings/si.rs:22


@dataclass
class ParticleSI:
    radius: float
    self_propulsion_speed: float
    force_dipole: float
    magnetic_dipole_moment: float
    persistance_time: float
    shape: float = 0.0


@dataclass
class ParametersSI:
    hydro_screening: float
    volume_exclusion: float
    viscocity: float
    temperature: float
    volume_fraction: float
    external_field: float
    particle: ParticleSI


@dataclass
class SettingsSI:
    simulation: SimulationSettings
    parameters: ParametersSI
    environment: EnvironmentSettings


def parse_settings_si(doc):
    """SettingsSI (src/bin/simulation/settings/si.rs:24-73): the simulation and
    environment tables of the dimensionless schema, physical parameters in SI."""
    _table(doc, "settings", ["simulation", "parameters", "environment"], [])
    shell = {"simulation": doc["simulation"], "environment": doc["environment"],
             "parameters": {"magnetic_reorientation": 0.0, "diffusion": {"translational": 0.0, "rotational": 0.0},
                            "stress": {"active": 0.0, "magnetic": 0.0}, "magnetic_dipole": {}}}
    base = parse_settings(shell)
    p = _table(doc["parameters"], "parameters",
               ["hydro_screening", "volume_exclusion", "viscocity", "temperature", "volume_fraction",
                "external_field", "particle"], [])
    q = _table(p["particle"], "parameters.particle",
               ["radius", "self_propulsion_speed", "force_dipole", "magnetic_dipole_moment", "persistance_time"],
               ["shape"])
    par = ParametersSI(**{k: _num(p[k], k) for k in ["hydro_screening", "volume_exclusion", "viscocity",
                                                     "temperature", "volume_fraction", "external_field"]},
                       particle=ParticleSI(**{k: _num(v, k) for k, v in q.items()}))
    return SettingsSI(simulation=base.simulation, parameters=par, environment=base.environment)


def into_settings(si):
    """SettingsSI::into_settings (si.rs:126-199): lengths in units of the mean
    particle distance n^(-1/3), velocities in units of the swimming speed."""
    import math
    pi = math.pi
    a = si.parameters.particle
    par = si.parameters
    volp = 4.0 / 3.0 * pi * (a.radius * a.radius * a.radius)
    number_density = par.volume_fraction / volp
    xc = number_density ** (-1.0 / 3.0)
    uc = a.self_propulsion_speed
    tc = xc / uc
    stressf = number_density ** (2.0 / 3.0) / a.self_propulsion_speed / par.viscocity
    rotfriction = 8.0 * pi * par.viscocity * (a.radius * a.radius * a.radius)
    transfriction = 6.0 * pi * par.viscocity * a.radius
    rotdiff_brown = BOLTZMANN * par.temperature / rotfriction
    rotdiff_active = 1.0 / 2.0 / a.persistance_time
    transdiff_brown = BOLTZMANN * par.temperature / transfriction
    diff = DiffusionConstants(translational=number_density ** (1.0 / 3.0) / uc * transdiff_brown,
                              rotational=number_density ** (-1.0 / 3.0) / uc * (rotdiff_brown + rotdiff_active))
    alignment = a.magnetic_dipole_moment * par.external_field / rotfriction / (rotdiff_brown + rotdiff_active)
    m2 = a.magnetic_dipole_moment * a.magnetic_dipole_moment
    params = Parameters(
        magnetic_reorientation=alignment * diff.rotational,
        diffusion=diff,
        stress=StressPrefactors(active=stressf * a.force_dipole,
                                magnetic=stressf * a.magnetic_dipole_moment * par.external_field),
        magnetic_dipole=MagneticDipolePrefactors(
            magnetic_dipole_dipole=number_density ** (2.0 / 3.0) / uc / rotfriction * 4.0e-7 * pi * m2),
        magnetic_drag=number_density / uc / transfriction * 4.0e-7 * pi * m2,
        shape=a.shape,
        hydro_screening=par.hydro_screening,
        volume_exclusion=par.volume_exclusion,
    )
    sim = dataclasses.replace(si.simulation)
    bs = si.simulation.box_size
    sim.box_size = BoxSize(bs.x / xc, bs.y / xc, bs.z / xc)
    sim.timestep = si.simulation.timestep / tc
    return Settings(simulation=sim, parameters=params, environment=dataclasses.replace(si.environment))


def read_parameter_file_si(path):
    """si::read_parameter_file (si.rs:87-101) followed by into_settings."""
    try:
        with open(path, "rb") as f:
            doc = tomllib.load(f)
    except OSError as exc:
        raise SettingsError(f"Unable to read parameter file: {exc}") from exc
    except tomllib.TOMLDecodeError as exc:
        raise SettingsError(f"Unable to parse parameter file: {exc}") from exc
    s = into_settings(parse_settings_si(doc))
    s.environment.version = ""
    check_settings(s)
    return s


def _toml_value(v):
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, int):
        return str(v)
    if isinstance(v, float):
        return repr(v)
    return '"' + str(v).replace("\\", "\\\\").replace('"', '\\"') + '"'


def to_toml(s):
    """Serialise Settings as TOML (Settings::save_to_file, mod.rs:213-224).
    Keys absent from the reference output (None options) are omitted."""
    lines = []

    def emit(table, obj):
        scalars, subs = [], []
        for f in dataclasses.fields(obj):
            v = getattr(obj, f.name)
            if v is None:
                continue
            (subs if dataclasses.is_dataclass(v) else scalars).append((f.name, v))
        lines.append(f"[{table}]")
        for k, v in scalars:
            lines.append(f"{k} = {_toml_value(v)}")
        lines.append("")
        for k, v in subs:
            emit(f"{table}.{k}", v)

    emit("environment", s.environment)
    emit("simulation", s.simulation)
    emit("parameters", s.parameters)
    return "\n".join(lines)
