"""The overlapped output path of the driver (run_simulation with
overlap=True) against the blocking one, on the host: a stand-in simulation
whose outputs are functions of the step counter, whose output_begin records
the values of the moment and fills the host arrays only in output_wait (NaN
before), and an IO sink that keeps the objects it is handed.  Both paths must
hand the sink the same entries and snapshots, in step order."""
import numpy as np
import pytest

from stochasticsampling_gb300 import driver
from stochasticsampling_gb300 import output as io

TOML = """
[environment]
    prefix = "ovl"
[simulation]
    number_of_particles = 7
    number_of_timesteps = {steps}
    timestep = 0.01
    seed = 1
    init_distribution = "Isotropic"
    [simulation.box_size]
        x = 2.0
        y = 3.0
        z = 1.0
    [simulation.grid_size]
        x = 4
        y = 3
        z = 1
        phi = 2
        theta = 1
    [simulation.output_at_timestep]
{outputs}
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


class _Holder:
    def __init__(self, shape):
        self.array = np.full(shape, np.nan)
        self.closed = False

    def close(self):
        self.closed = True


class FakeSim:
    def __init__(self, n=7, grid=(4, 3, 1, 2, 1), box=(2.0, 3.0, 1.0)):
        self.n, self.grid, self.box, self.dist_shape = n, grid, box, grid
        self.t = 0
        self.inflight = {}
        self.holders = []
        self.output_buffers = [{}, {}]

    def _dist(self):
        return np.arange(np.prod(self.grid), dtype=np.float64).reshape(self.grid) + 0.5 * self.t

    def _field(self, k):
        return np.arange(3 * np.prod(self.grid[:3]), dtype=np.float64).reshape((3,) + self.grid[:3]) * k + self.t

    def _rows(self):
        return np.arange(5 * self.n, dtype=np.float64).reshape(self.n, 5) + 100.0 * self.t

    def get_timestep(self):
        return self.t

    def do_timestep(self):
        self.t += 1

    def get_distribution(self):
        return self._dist()

    def get_flow_field(self):
        return self._field(2.0)

    def get_magnetic_field(self):
        return self._field(-3.0)

    def get_particles(self):
        return self._rows()

    def get_particles_head(self, n):
        return self._rows()[:n]

    def host_array(self, shape):
        h = _Holder(shape)
        self.holders.append(h)
        return h

    def output_begin(self, slot, dist=None, flow=None, mag=None, particles=None):
        assert slot in (0, 1) and slot not in self.inflight
        vals = [(dist, self._dist()), (flow, self._field(2.0)), (mag, self._field(-3.0))]
        if particles is not None:
            vals.append((particles, self._rows()[:particles.shape[0]]))
        vals = [(a, v) for a, v in vals if a is not None]
        for a, v in vals:
            assert a.shape == v.shape and a.flags.c_contiguous
            a[...] = np.nan  # not landed yet
        self.inflight[slot] = vals

    def output_wait(self, slot):
        for a, v in self.inflight.pop(slot, []):
            a[...] = v


class Sink:
    def __init__(self):
        self.entries, self.snapshots = [], []

    def append(self, e):
        self.entries.append(e)

    def write_snapshot(self, s):
        self.snapshots.append(s)


def _settings(outputs, steps):
    import tomllib
    from stochasticsampling_gb300.settings import parse_settings
    return parse_settings(tomllib.loads(TOML.format(steps=steps, outputs=outputs)))


def _run(outputs, steps, overlap):
    sim, sink = FakeSim(), Sink()
    driver.run_simulation(_settings(outputs, steps), sim, sink, overlap=overlap)
    return sim, sink


OUTPUTS = {
    "every_kind": """        distribution = 2
        flowfield = 3
        magneticfield = 3
        particles = 2
        particles_head = 3
        snapshot = 4""",
    "snapshot_and_all_particles_each_step": """        distribution = 1
        particles = 1
        snapshot = 1
        magneticfield = 1""",
    "magnetic_alone_makes_no_entry": """        magneticfield = 1
        snapshot = 5""",
    "sparse": """        flowfield = 7
        particles = 5""",
}


@pytest.mark.parametrize("name", sorted(OUTPUTS))
@pytest.mark.parametrize("steps", [0, 1, 12])
def test_overlapped_outputs_equal_blocking_ones(name, steps):
    sa, a = _run(OUTPUTS[name], steps, overlap=False)
    sb, b = _run(OUTPUTS[name], steps, overlap=True)
    assert sa.t == sb.t == steps + 1  # one step more than number_of_timesteps (main.rs:178-182)
    assert [e["timestep"] for e in b.entries] == [e["timestep"] for e in a.entries]
    assert [io.packb(e) for e in b.entries] == [io.packb(e) for e in a.entries]
    assert [io.packb(s) for s in b.snapshots] == [io.packb(s) for s in a.snapshots]
    assert not sb.inflight



def test_overlapped_entries_are_copies_of_the_host_buffers():
    """Entries handed to the IO worker must not alias the reused host
    buffers: after the run, every entry still holds its own step's values."""
    sim, sink = _run(OUTPUTS["every_kind"], 12, overlap=True)
    probe = FakeSim()
    for e in sink.entries:
        if e["distribution"] is None:
            continue
        probe.t = e["timestep"]
        assert np.array_equal(e["distribution"]["dist"].a, probe._dist())
        if e["particles"] is not None:
            assert np.array_equal(e["particles"], probe._rows()[:3])


def test_a_later_run_reuses_the_page_locked_buffers():
    outputs = """        distribution = 1
        flowfield = 1"""
    sim = FakeSim()
    driver.run_simulation(_settings(outputs, 4), sim, Sink(), overlap=True)
    held = {(s, k): v for s, d in enumerate(sim.output_buffers) for k, v in d.items()}
    assert len(held) == 4  # dist and flow in both slots
    n = len(sim.holders)
    driver.run_simulation(_settings(outputs, 4), sim, Sink(), overlap=True)
    assert len(sim.holders) == n
    assert all(sim.output_buffers[s][k] is v for (s, k), v in held.items())


def test_a_failing_step_leaves_no_transfer_in_flight():
    """A step that raises in the middle of the run: the error reaches the
    caller, and the transfers begun before it are waited for (the slots are
    free, the host buffers no longer written by the device)."""
    class Failing(FakeSim):
        def do_timestep(self):
            if self.t == 5:
                raise RuntimeError("step failed")
            super().do_timestep()

    sim, sink = Failing(), Sink()
    with pytest.raises(RuntimeError, match="step failed"):
        driver.run_simulation(_settings(OUTPUTS["every_kind"], 12), sim, sink, overlap=True)
    assert not sim.inflight
    # the entries completed before the failure reached the sink in step order
    steps = [e["timestep"] for e in sink.entries]
    assert steps == sorted(steps)
