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

The reference's loop sends each due output to its IO worker thread and steps
on while the worker serialises and compresses it (:182-262).  Here the
device half overlaps too: a due step's outputs are taken into one of two
device slots and copied into page-locked host buffers while the next steps
run (ss_output_begin); the host turns them into records for the IO worker
when the slot is needed again, in step order.
"""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np

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


def _copy(a, pool, nthreads):
    """A copy of the C-contiguous host array a; one of more than 16 MB is
    copied in nthreads row blocks on the pool's threads (numpy releases the
    GIL while it copies), so that the particle rows of an output do not hold
    up the loop for long."""
    out = np.empty_like(a)
    if pool is None or nthreads < 2 or a.nbytes < (16 << 20) or a.shape[0] < 2:
        np.copyto(out, a)
        return out
    rows = a.shape[0]
    step = -(-rows // nthreads)
    list(pool.map(lambda i: np.copyto(out[i:i + step], a[i:i + step]), range(0, rows, step)))
    return out


class _OverlappedOutputs:
    """The due outputs of the loop, two steps' worth in flight at a time.

    begin() takes a step's outputs on the device and starts their transfer
    (Simulation.output_begin into slot k % 2); complete() waits for a slot,
    copies its host buffers into records and hands them to the IO worker.
    Slots alternate, so the slot reused next always holds the oldest output
    and the worker receives entries in step order.  The page-locked host
    buffers belong to the simulation (sim.output_buffers, released by its
    close()), so later runs on it reuse them."""

    def __init__(self, sim, out):
        self.sim, self.out = sim, out
        self.bufs = sim.output_buffers
        self.pending = [None, None]
        self.k = 0
        self.nthreads = max(1, min(16, os.cpu_count() or 1))
        self.pool = ThreadPoolExecutor(max_workers=self.nthreads)

    def _array(self, slot, name, shape):
        """The slot's host buffer `name`: the first shape[0] rows of a
        page-locked array that grows to the largest request."""
        b = self.bufs[slot].get(name)
        if b is None or b.array.shape[0] < shape[0] or b.array.shape[1:] != shape[1:]:
            if b is not None:
                b.close()
            b = self.bufs[slot][name] = self.sim.host_array(shape)
        return b.array[:shape[0]]

    def begin(self, timestep, dist, flow, mag, parts_n, snapshot):
        """Outputs of the current state: dist/flow/mag flags, the number of
        particle rows of the entry (None: none), and whether a snapshot is due."""
        slot = self.k % 2
        self.k += 1
        if self.pending[slot] is not None:
            self.complete(slot)
        sim = self.sim
        fshape = (3,) + tuple(sim.grid[:3])
        rows = sim.n if snapshot else parts_n
        self.sim.output_begin(
            slot,
            dist=self._array(slot, "dist", tuple(sim.dist_shape)) if dist else None,
            flow=self._array(slot, "flow", fshape) if flow else None,
            mag=self._array(slot, "mag", fshape) if mag else None,
            particles=self._array(slot, "rows", (rows, 5)) if rows is not None else None)
        self.pending[slot] = (timestep, dist, flow, mag, parts_n, snapshot)

    def complete(self, slot):
        timestep, dist, flow, mag, parts_n, snapshot = self.pending[slot]
        self.pending[slot] = None
        self.sim.output_wait(slot)
        b = self.bufs[slot]
        def cp(a):
            return _copy(a, self.pool, self.nthreads)
        d = io.distribution_record(cp(b["dist"].array), self.sim.grid, self.sim.box) if dist else None
        f = cp(b["flow"].array) if flow else None
        m = cp(b["mag"].array) if mag else None
        p = cp(b["rows"].array[:parts_n]) if parts_n is not None else None
        if d is not None or f is not None or p is not None:
            self.out.append(io.output_entry(timestep, d, f, m, p))
        if snapshot:
            self.out.write_snapshot(io.snapshot_record(cp(b["rows"].array[:self.sim.n]), timestep))

    def finish(self):
        for _, slot in sorted((p[0], s) for s, p in enumerate(self.pending) if p is not None):
            self.complete(slot)

    def close(self):
        """Wait for transfers still in flight (after an error in the loop)."""
        for slot in range(2):
            if self.pending[slot] is not None:
                self.pending[slot] = None
                try:
                    self.sim.output_wait(slot)
                except Exception:
                    pass
        self.pool.shutdown()


def run_simulation(settings, sim, out, progress=None, overlap=True):
    """run_simulation, src/bin/main.rs:139-289.  overlap=True takes the due
    outputs without stalling the steps (ss_output_begin, two in flight);
    overlap=False reads each one back with the blocking getters.  Both give
    the same entries and snapshots."""
    o = settings.simulation.output_at_timestep
    grid = sim.grid
    box = sim.box
    if o.initial_condition:
        out.append(io.output_entry(
            0, distribution=io.distribution_record(sim.get_distribution(), grid, box),
            particles=_particles_out(settings, sim) if o.particles is not None else None))
    timestep_start = sim.get_timestep() + 1
    n = settings.simulation.number_of_timesteps + timestep_start
    if overlap:
        outs = _OverlappedOutputs(sim, out)
        try:
            for timestep in range(timestep_start, n + 1):
                sim.do_timestep()
                due = lambda every: every is not None and timestep % every == 0
                dist, flow, parts = due(o.distribution), due(o.flowfield), due(o.particles)
                entry = dist or flow or parts
                snap = due(o.snapshot)
                if entry or snap:
                    parts_n = (sim.n if o.particles_head is None else int(o.particles_head)) if parts else None
                    outs.begin(timestep, dist, flow, entry and due(o.magneticfield), parts_n, snap)
                if progress is not None:
                    progress(timestep)
            outs.finish()
        finally:
            outs.close()
        if o.final_snapshot:
            out.write_snapshot(io.snapshot_record(sim.get_particles(), sim.get_timestep()))
        return
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


def run(settings, output_root, init=None, resume=None, overlap=True, **sim_kwargs):
    """run, src/bin/main.rs:68-135: output directory <root>/<id>/ holding
    <id>.toml, <id>.msgpack-lzma, <id>.index and the snapshots.  Returns the
    output file path.  overlap as for run_simulation."""
    output_id = io.create_output_id(settings.environment.prefix)
    directory = os.path.join(output_root, output_id)
    os.makedirs(directory, exist_ok=False)
    with open(os.path.join(directory, f"{output_id}.toml"), "w") as f:
        f.write(to_toml(settings))
    sim = init_simulation(settings, init=init, resume=resume, **sim_kwargs)
    out = io.Worker(directory, output_id, settings.environment.output_format, settings.environment.io_queue_size)
    try:
        out.write_metadata(settings)
        run_simulation(settings, sim, out, overlap=overlap)
    finally:
        out.quit()
        sim.close()
    return out.path
