"""Host-side mirror of the reference's ``Simulation`` (src/bin/simulation/mod.rs)
over the C ABI of libssgpu.so.

    sim = Simulation(settings)          # Simulation::new        (:91-160)
    sim.init(particles)                 # Simulation::init       (:163-196)
    sim.do_timestep()                   # Simulation::do_timestep (:251-374)
    sim.get_particles() / get_distribution() / get_flow_field() /
    get_magnetic_field() / get_timestep() / get_snapshot() / resume()

Particles are numpy arrays of shape (n, 5) with columns (x, y, z, phi, theta),
the reference's serialised Particle layout (src/particle.rs:363-395).  All
arithmetic runs on the GPU; there is no CPU fallback.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import Box, Grid, LangevinArgs, Params, check

_dp = ctypes.POINTER(ctypes.c_double)


def _ptr(a):
    return a.ctypes.data_as(_dp)


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


class PinnedArray:
    """Page-locked host memory (ss_host_alloc) viewed as a float64 numpy
    array, for the transfers of Simulation.output_begin.  close() releases
    it; the array must not be used afterwards."""

    def __init__(self, shape):
        self.lib = _lib.load()
        shape = tuple(int(v) for v in shape)
        count = int(np.prod(shape))
        if count < 1:
            raise ValueError("a pinned array holds at least one element")
        p = ctypes.c_void_p()
        check(self.lib.ss_host_alloc(8 * count, ctypes.byref(p)))
        self._p = p
        self.array = np.ctypeslib.as_array((ctypes.c_double * count).from_address(p.value)).reshape(shape)

    def close(self):
        p = getattr(self, "_p", None)
        if p is not None and p.value:
            self.array = None
            self.lib.ss_host_free(p)
        self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def geometry_from_settings(settings):
    """(grid, box, params) of a Settings object, the ss_grid / ss_box /
    ss_params triple of the C ABI."""
    sim, par = settings.simulation, settings.parameters
    grid = (sim.grid_size.x, sim.grid_size.y, sim.grid_size.z, sim.grid_size.phi, sim.grid_size.theta)
    box = (sim.box_size.x, sim.box_size.y, sim.box_size.z)
    params = dict(timestep=sim.timestep, trans_diffusion=par.diffusion.translational,
                  rot_diffusion=par.diffusion.rotational, stress_active=par.stress.active,
                  stress_magnetic=par.stress.magnetic, shape=par.shape, magnetic_drag=par.magnetic_drag,
                  hydro_screening=par.hydro_screening, volume_exclusion=par.volume_exclusion,
                  magnetic_reorientation=par.magnetic_reorientation,
                  magnetic_dipole_dipole=par.magnetic_dipole.magnetic_dipole_dipole,
                  number_of_particles=sim.number_of_particles, seed=sim.seed)
    return grid, box, params


class Simulation:
    """One simulation on the current CUDA device.

    Keyword flags of ``ss_create``: ``quasi2d`` (the cargo feature),
    ``sort=False`` (no counting sort by cell), ``graph=False`` (direct
    launches), ``always_magnetic`` (the dipolar solve every step),
    ``mixed`` (True: FP32 with FP64 positions, "fixed64": FP32 with 64-bit
    fixed-point positions), ``gather`` ("nearest", "trilinear",
    "trilinear_zfromy"), ``f32x2`` (FP64 state with each step's increments in
    two-float arithmetic, within 1e-14 of the FP64 step; FP64 mode and
    nearest-cell gather only)."""

    def __init__(self, settings=None, *, grid=None, box=None, params=None, quasi2d=False, sort=True, graph=True,
                 always_magnetic=False, mixed=False, gather="nearest", f32x2=False, stream=None):
        if settings is not None:
            grid, box, params = geometry_from_settings(settings)
        if grid is None or box is None or params is None:
            raise ValueError("give settings, or grid, box and params")
        self.lib = _lib.load()
        self.grid = tuple(int(v) for v in grid)
        self.box = tuple(float(v) for v in box)
        self.params = dict(params)
        g = Grid(*self.grid)
        b = Box(*self.box)
        p = Params()
        for k, v in self.params.items():
            setattr(p, k, v)
        self.n = int(p.number_of_particles)
        flags = 0
        if quasi2d:
            flags |= _lib.FLAG_QUASI2D
        if not sort:
            flags |= _lib.FLAG_NO_SORT
        if not graph:
            flags |= _lib.FLAG_NO_GRAPH
        if always_magnetic:
            flags |= _lib.FLAG_ALWAYS_MAGNETIC
        if f32x2:
            flags |= _lib.FLAG_F32X2
        if mixed == "fixed64":
            flags |= _lib.FLAG_FIXED64
        elif mixed:
            flags |= _lib.FLAG_MIXED
        flags |= {"nearest": 0, "trilinear": _lib.FLAG_TRILINEAR,
                  "trilinear_zfromy": _lib.FLAG_TRILINEAR_ZFROMY}[gather]
        self.flags = flags
        h = ctypes.c_void_p()
        rc = self.lib.ss_create(ctypes.byref(g), ctypes.byref(b), ctypes.byref(p), flags,
                                ctypes.c_void_p(stream) if stream else None, ctypes.byref(h))
        check(rc)
        self._h = h
        self._inflight = {}
        self.output_buffers = [{}, {}]  # the driver's page-locked output buffers per slot
        gx, gy, gz, gp, gt = self.grid
        self.ncell = gx * gy * gz
        self.dist_shape = (gx, gy, gz, gp, gt)

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self.lib.ss_destroy(h)  # waits for transfers in flight
        self._h = None
        for slot in getattr(self, "output_buffers", []):
            for b in slot.values():
                b.close()
            slot.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc):
        check(rc, self._h)

    # --- Simulation API ---------------------------------------------------
    def set_denoiser(self, denoiser):
        """Contract the denoised histogram instead of the counts every step
        (quasi2d mixed contexts; None removes it).  The simulation keeps a
        reference to the denoiser while it is set."""
        self._denoiser = denoiser
        self._check(self.lib.ss_set_denoiser(self._h, denoiser._h if denoiser is not None else None))

    def init(self, particles):
        p = _f64(particles, (-1, 5))
        self._check(self.lib.ss_init(self._h, _ptr(p), p.shape[0]))

    def init_distribution(self, kind):
        """Sample the initial condition on the GPU: "Isotropic" or "Homogeneous"
        (init_simulation with InitType::Distribution)."""
        k = {"Isotropic": 0, "Homogeneous": 1}[kind] if isinstance(kind, str) else int(kind)
        self._check(self.lib.ss_init_distribution(self._h, k))

    def resume(self, particles, timestep):
        p = _f64(particles, (-1, 5))
        self._check(self.lib.ss_resume(self._h, _ptr(p), p.shape[0], int(timestep)))

    def do_timestep(self, noise=None):
        t = ctypes.c_uint64()
        if noise is None:
            self._check(self.lib.ss_do_timestep(self._h, None, ctypes.byref(t)))
        else:
            z = _f64(noise, (self.n, 5))
            self._check(self.lib.ss_do_timestep(self._h, _ptr(z), ctypes.byref(t)))
        return t.value

    def step_host(self, particles, out=None):
        """One step of host-resident particles (ss_step_host): `particles`
        replace the state at the current step, the step runs, and the new
        state comes back in `out` ((n, 5) float64, C-contiguous; may be
        `particles` itself).  Returns `out`."""
        p = _f64(particles, (-1, 5))
        out = np.empty((p.shape[0], 5)) if out is None else self._out_rows(out, p.shape[0])
        t = ctypes.c_uint64()
        self._check(self.lib.ss_step_host(self._h, _ptr(p), _ptr(out), p.shape[0], ctypes.byref(t)))
        return out

    @staticmethod
    def _out_rows(out, n):
        if not (isinstance(out, np.ndarray) and out.dtype == np.float64 and out.flags.c_contiguous
                and out.shape == (n, 5) and out.flags.writeable):
            raise ValueError(f"out must be a writeable C-contiguous float64 array of shape ({n}, 5)")
        return out

    def run(self, steps):
        t = ctypes.c_uint64()
        self._check(self.lib.ss_run(self._h, int(steps), ctypes.byref(t)))
        return t.value

    def noise(self, timestep):
        """The Philox noise step `timestep` uses, as RandomVector rows (n, 5)."""
        out = np.empty((self.n, 5))
        self._check(self.lib.ss_noise(self._h, int(timestep), _ptr(out)))
        return out

    def synchronize(self):
        self._check(self.lib.ss_synchronize(self._h))

    def get_particles(self, out=None):
        out = np.empty((self.n, 5)) if out is None else self._out_rows(out, self.n)
        self._check(self.lib.ss_get_particles(self._h, _ptr(out), self.n))
        return out

    def get_particles_head(self, n):
        out = np.empty((int(n), 5))
        self._check(self.lib.ss_get_particles(self._h, _ptr(out), int(n)))
        return out

    def get_distribution(self):
        out = np.empty(self.dist_shape)
        self._check(self.lib.ss_get_distribution(self._h, _ptr(out)))
        return out

    def get_counts(self):
        out = np.empty(self.dist_shape, dtype=np.uint32)
        self._check(self.lib.ss_get_counts(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))))
        return out

    def get_flow_field(self):
        out = np.empty((3,) + self.grid[:3])
        self._check(self.lib.ss_get_flow_field(self._h, _ptr(out)))
        return out

    def get_magnetic_field(self):
        out = np.empty((3,) + self.grid[:3])
        self._check(self.lib.ss_get_magnetic_field(self._h, _ptr(out)))
        return out

    def get_flow_complex(self):
        u = np.empty((3,) + self.grid[:3], dtype=np.complex128)
        g = np.empty((3, 3) + self.grid[:3], dtype=np.complex128)
        self._check(self.lib.ss_get_flow_complex(self._h, _ptr(u.view(np.float64)), _ptr(g.view(np.float64))))
        return u, g

    def get_magnetic_complex(self):
        b = np.empty((3,) + self.grid[:3], dtype=np.complex128)
        g = np.empty((3, 3) + self.grid[:3], dtype=np.complex128)
        self._check(self.lib.ss_get_magnetic_complex(self._h, _ptr(b.view(np.float64)),
                                                     _ptr(g.view(np.float64))))
        return b, g

    def get_timestep(self):
        t = ctypes.c_uint64()
        self._check(self.lib.ss_get_timestep(self._h, ctypes.byref(t)))
        return t.value

    # --- output overlapped with the steps ---------------------------------
    def host_array(self, shape):
        """A page-locked host array for output_begin (a PinnedArray)."""
        return PinnedArray(shape)

    def output_begin(self, slot, dist=None, flow=None, mag=None, particles=None):
        """ss_output_begin: take the current state's outputs into device slot
        `slot` (0 or 1) and start their transfer into the given host arrays
        (float64, C-contiguous, the shapes of get_distribution,
        get_flow_field, get_magnetic_field and get_particles_head(n)); the
        call does not wait, and steps may be queued at once.  The arrays hold
        the outputs once output_wait(slot) has returned; page-locked arrays
        (host_array) keep the transfer asynchronous."""
        def arg(a, shape):
            if a is None:
                return None
            if a.dtype != np.float64 or not a.flags.c_contiguous or a.shape != shape:
                raise ValueError(f"output array must be C-contiguous float64 of shape {shape}")
            return _ptr(a)
        n = 0
        if particles is not None:
            n = particles.shape[0] if particles.ndim == 2 else -1
            if not 0 <= n <= self.n:
                raise ValueError(f"particles must be (n, 5) with n <= {self.n}")
        fshape = (3,) + self.grid[:3]
        ptrs = (arg(dist, self.dist_shape), arg(flow, fshape), arg(mag, fshape), arg(particles, (n, 5)))
        self._check(self.lib.ss_output_begin(self._h, int(slot), *ptrs, n))
        self._inflight[int(slot)] = (dist, flow, mag, particles)  # alive until the transfer has landed

    def output_wait(self, slot):
        """ss_output_wait: block until slot's transfer has landed."""
        try:
            self._check(self.lib.ss_output_wait(self._h, int(slot)))
        finally:
            self._inflight.pop(int(slot), None)

    def output_ready(self, slot):
        """ss_output_query: True when output_wait(slot) would not block."""
        r = ctypes.c_int()
        self._check(self.lib.ss_output_query(self._h, int(slot), ctypes.byref(r)))
        return bool(r.value)

    def get_snapshot(self):
        """Snapshot (src/bin/simulation/mod.rs:80-86,210-217): the particles and
        the step counter.  The noise is counter based (Philox keyed by seed), so
        (seed, timestep) is the whole RNG state."""
        return {"particles": self.get_particles(), "rng_state": {"philox_seed": int(self.params["seed"])},
                "timestep": self.get_timestep()}

    # --- library seams ----------------------------------------------------
    def mean_flow_field(self, screening, dist):
        d = _f64(dist, self.dist_shape)
        u = np.empty((3,) + self.grid[:3], dtype=np.complex128)
        g = np.empty((3, 3) + self.grid[:3], dtype=np.complex128)
        self._check(self.lib.ss_mean_flow_field(self._h, float(screening), _ptr(d), _ptr(u.view(np.float64)),
                                                _ptr(g.view(np.float64))))
        return u, g

    def mean_magnetic_field(self, dist):
        d = _f64(dist, self.dist_shape)
        b = np.empty((3,) + self.grid[:3], dtype=np.complex128)
        g = np.empty((3, 3) + self.grid[:3], dtype=np.complex128)
        self._check(self.lib.ss_mean_magnetic_field(self._h, _ptr(d), _ptr(b.view(np.float64)),
                                                    _ptr(g.view(np.float64))))
        return b, g

    # --- instrumentation --------------------------------------------------
    def set_resort(self, every_steps):
        """Counting-sort the particles by cell every every_steps steps (0: never);
        no result changes (ss_set_resort)."""
        self._check(self.lib.ss_set_resort(self._h, int(every_steps)))

    def profile(self, enable=True):
        self._check(self.lib.ss_profile_enable(self._h, 1 if enable else 0))

    def profile_read(self):
        ms = np.zeros(_lib.NUM_STAGES)
        n = ctypes.c_uint64()
        self._check(self.lib.ss_profile_read(self._h, _ptr(ms), ctypes.byref(n)))
        return dict(zip(_lib.STAGES, ms.tolist())), n.value

    def launch_count(self):
        n = ctypes.c_uint64()
        self._check(self.lib.ss_launch_count(self._h, ctypes.byref(n)))
        return n.value


def langevin(particles, mask, **kw):
    """Run the LangevinBuilder chain (modifier bits in do_timestep order) on
    independent particles with shared arguments, on the GPU."""
    lib = _lib.load()
    a = LangevinArgs()
    a.box_x, a.box_y, a.box_z = kw.pop("box", (10.0, 10.0, 10.0))
    for k, v in kw.items():
        cur = getattr(a, k)
        if isinstance(cur, float):
            setattr(a, k, float(v))
        else:
            for i, x in enumerate(np.asarray(v, dtype=np.float64).ravel()):
                cur[i] = x
    p = _f64(particles, (-1, 5))
    out = np.empty_like(p)
    check(lib.ss_langevin(_ptr(p), p.shape[0], int(mask), ctypes.byref(a), _ptr(out)))
    return out
