"""The simulation driver around the GPU timestep: `run` and `run_simulation`
of src/bin/main.rs:68-289, with the output layout of the reference's IO worker.

This is the library form of the reference's binary (no command line): read
the settings, set up the simulation with an initial condition, write the
metadata, step, and emit output entries and snapshots on the reference's
schedule.  Schedule quirks kept from main.rs:
  - the loop runs from timestep_start = get_timestep() + 1 to
    number_of_timesteps + timestep_start inclusive, i.e. one step more than
    number_of_timesteps (:178-182);
  - an entry is appended only when it carries a distribution, a flow field or
    particles; a magnetic field alone does not trigger it (:245-251);
  - the initial condition entry holds the distribution and, if particles are
    output at all, the (head of the) particles (:145-161).
"""
import os

from . import output as io
from .settings import to_toml
from .simulation import Simulation


def init_simulation(settings, init=None, resume=None, **sim_kwargs):
    """init_simulation (src/bin/init.rs:52-117).

    init: None -> InitType::Distribution (the settings' init_distribution,
          sampled on the GPU); a path -> InitType::File; an (n, 5) array ->
          particles given directly (InitType::Stdin reads the same list).
    resume: a snapshot path -> InitType::Resume.
    """
    sim = Simulation(settings, **sim_kwargs)
    if resume is not None:
        particles, timestep = io.read_particles_file(resume)
        sim.resume(particles, timestep or 0)
    elif init is None:
        sim.init_distribution(settings.simulation.init_distribution)
    elif isinstance(init, (str, os.PathLike)):
        particles, _ = io.read_particles_file(os.fspath(init))
        sim.init(particles)
    else:
        sim.init(init)
    return sim


def _particles_out(settings, sim):
    o = settings.simulation.output_at_timestep
    if o.particles_head is not None:
        return sim.get_particles_head(o.particles_head)
    return sim.get_particles()


def run_simulation(settings, sim, out, progress=None):
    """run_simulation, src/bin/main.rs:139-289."""
    o = settings.simulation.output_at_timestep
    grid = sim.grid
    box = sim.box
    if o.initial_condition:
        out.append(io.output_entry(
            0, distribution=io.distribution_record(sim.get_distribution(), grid, box),
            particles=_particles_out(settings, sim) if o.particles is not None else None))
    timestep_start = sim.get_timestep() + 1
    n = settings.simulation.number_of_timesteps + timestep_start
    for timestep in range(timestep_start, n + 1):
        sim.do_timestep()
        due = lambda every: every is not None and timestep % every == 0
        dist = io.distribution_record(sim.get_distribution(), grid, box) if due(o.distribution) else None
        flow = sim.get_flow_field() if due(o.flowfield) else None
        mag = sim.get_magnetic_field() if due(o.magneticfield) else None
        parts = _particles_out(settings, sim) if due(o.particles) else None
        if dist is not None or flow is not None or parts is not None:
            out.append(io.output_entry(timestep, dist, flow, mag, parts))
        if due(o.snapshot):
            out.write_snapshot(io.snapshot_record(sim.get_particles(), sim.get_timestep()))
        if progress is not None:
            progress(timestep)
    if o.final_snapshot:
        out.write_snapshot(io.snapshot_record(sim.get_particles(), sim.get_timestep()))


def run(settings, output_root, init=None, resume=None, **sim_kwargs):
    """run, src/bin/main.rs:68-135: output directory <root>/<id>/ holding
    <id>.toml, <id>.msgpack-lzma, <id>.index and the snapshots.  Returns the
    output file path."""
    output_id = io.create_output_id(settings.environment.prefix)
    directory = os.path.join(output_root, output_id)
    os.makedirs(directory, exist_ok=False)
    with open(os.path.join(directory, f"{output_id}.toml"), "w") as f:
        f.write(to_toml(settings))
    sim = init_simulation(settings, init=init, resume=resume, **sim_kwargs)
    out = io.Worker(directory, output_id, settings.environment.output_format, settings.environment.io_queue_size)
    try:
        out.write_metadata(settings)
        run_simulation(settings, sim, out)
    finally:
        out.quit()
        sim.close()
    return out.path
