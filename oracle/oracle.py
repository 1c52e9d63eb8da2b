"""ctypes front end of the CPU oracle (test infrastructure, not product).

Only the parity tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py`` import this module.  It loads ``oracle/liboracle.so``, the FP64
C restatement of the reference timestep (see ``ss_oracle.h`` for the
reference files it follows).
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

c_double_p = ctypes.POINTER(ctypes.c_double)
c_u64_p = ctypes.POINTER(ctypes.c_uint64)


class Settings(ctypes.Structure):
    """Mirror of ``orc_settings`` (reference Settings flattened)."""

    _fields_ = [
        ("gx", ctypes.c_uint64), ("gy", ctypes.c_uint64), ("gz", ctypes.c_uint64),
        ("gphi", ctypes.c_uint64), ("gtheta", ctypes.c_uint64),
        ("bx", ctypes.c_double), ("by", ctypes.c_double), ("bz", ctypes.c_double),
        ("timestep", ctypes.c_double),
        ("trans_diff", ctypes.c_double), ("rot_diff", ctypes.c_double),
        ("stress_active", ctypes.c_double), ("stress_magnetic", ctypes.c_double),
        ("shape", ctypes.c_double), ("magnetic_drag", ctypes.c_double),
        ("hydro_screening", ctypes.c_double), ("volume_exclusion", ctypes.c_double),
        ("magnetic_reorientation", ctypes.c_double), ("magnetic_dipole_dipole", ctypes.c_double),
        ("quasi2d", ctypes.c_int32), ("gather", ctypes.c_int32),
        ("seed", ctypes.c_uint64),
    ]


class LangevinArgs(ctypes.Structure):
    _fields_ = [
        ("flow", ctypes.c_double * 3), ("drag", ctypes.c_double), ("gradb", ctypes.c_double * 9),
        ("reorientation", ctypes.c_double), ("b", ctypes.c_double * 3),
        ("vort", ctypes.c_double * 9), ("shape", ctypes.c_double), ("strain", ctypes.c_double * 9),
        ("dt", ctypes.c_double), ("xi", ctypes.c_double * 3), ("diff", ctypes.c_double),
        ("axis_angle", ctypes.c_double), ("rotate_angle", ctypes.c_double),
        ("bx", ctypes.c_double), ("by", ctypes.c_double), ("bz", ctypes.c_double),
    ]


SELF_PROPULSION, CONVECTION, MDD_FORCE, EXTERNAL_FIELD, MDD_ROTATION = 1, 2, 4, 8, 16
JEFFREY_VORTICITY, JEFFREY_STRAIN, STEP, TRANS_DIFFUSION, ROT_DIFFUSION = 32, 64, 128, 256, 512
ALL = 1023


def build():
    """Compile liboracle.so from the committed C sources (make)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        sp = ctypes.POINTER(Settings)
        L.orc_modulo.restype = ctypes.c_double
        L.orc_modulo.argtypes = [ctypes.c_double, ctypes.c_double]
        L.orc_ang_pbc.argtypes = [ctypes.c_double, ctypes.c_double, c_double_p]
        L.orc_particle_new.argtypes = [sp, c_double_p, c_double_p]
        L.orc_from_vector.argtypes = [c_double_p, c_double_p]
        L.orc_grid_width.argtypes = [sp, c_double_p]
        L.orc_coord_to_grid.argtypes = [sp, c_double_p, c_u64_p]
        L.orc_cell_index.argtypes = [sp, c_double_p, c_u64_p]
        L.orc_k_sampling.argtypes = [ctypes.c_uint64, ctypes.c_double, c_double_p]
        for f in ("orc_k_mesh", "orc_norm_k_mesh", "orc_inverse_norm_squared",
                  "orc_stress_kernel", "orc_orientation_kernel"):
            getattr(L, f).argtypes = [sp, c_double_p]
        L.orc_histogram.argtypes = [sp, c_double_p, ctypes.c_uint64, c_double_p]
        L.orc_sample_from.argtypes = [sp, c_double_p, ctypes.c_uint64, c_double_p]
        for f in ("orc_stress_active", "orc_stress_magnetic", "orc_stress_magnetic_rods"):
            getattr(L, f).argtypes = [ctypes.c_double, ctypes.c_double, c_double_p]
        L.orc_fft3d.argtypes = [c_double_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int]
        L.orc_average_stress.argtypes = [sp, c_double_p, c_double_p, c_double_p]
        L.orc_director_field.argtypes = [sp, c_double_p, c_double_p]
        L.orc_flow_field.argtypes = [sp, c_double_p, ctypes.c_double, c_double_p, c_double_p, ctypes.c_int]
        L.orc_magnetic_field.argtypes = [sp, c_double_p, c_double_p, c_double_p, ctypes.c_int]
        L.orc_vector_gradient.argtypes = [sp, c_double_p, c_double_p]
        L.orc_interpolate.argtypes = [sp, c_double_p, ctypes.c_int, c_double_p, ctypes.c_int, c_double_p]
        L.orc_langevin.argtypes = [c_double_p, ctypes.c_uint32, ctypes.POINTER(LangevinArgs), c_double_p]
        L.orc_sim_new.restype = ctypes.c_void_p
        L.orc_sim_new.argtypes = [sp, ctypes.c_uint64, ctypes.c_int]
        L.orc_sim_free.argtypes = [ctypes.c_void_p]
        L.orc_sim_init.restype = ctypes.c_int
        L.orc_sim_init.argtypes = [ctypes.c_void_p, c_double_p, ctypes.c_uint64]
        L.orc_sim_step.restype = ctypes.c_uint64
        L.orc_sim_step.argtypes = [ctypes.c_void_p, c_double_p]
        for f in ("orc_sim_particles", "orc_sim_distribution", "orc_sim_flow", "orc_sim_flow_grad",
                  "orc_sim_mag", "orc_sim_mag_grad", "orc_sim_density", "orc_sim_noise"):
            getattr(L, f).restype = c_double_p
            getattr(L, f).argtypes = [ctypes.c_void_p]
        L.orc_sim_timestep.restype = ctypes.c_uint64
        L.orc_sim_timestep.argtypes = [ctypes.c_void_p]
        L.orc_sim_set_timestep.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        L.orc_max_threads.restype = ctypes.c_int
        _LIB = L
    return _LIB


def _p(a):
    return a.ctypes.data_as(c_double_p)


def make_settings(grid, box, timestep=0.0, trans_diff=0.0, rot_diff=0.0, active=0.0, magnetic=0.0,
                  shape=0.0, magnetic_drag=0.0, hydro_screening=0.0, volume_exclusion=0.0,
                  magnetic_reorientation=0.0, magnetic_dipole_dipole=0.0, quasi2d=False, seed=1, gather=0):
    s = Settings()
    s.gx, s.gy, s.gz, s.gphi, s.gtheta = [int(v) for v in grid]
    s.bx, s.by, s.bz = [float(v) for v in box]
    s.timestep, s.trans_diff, s.rot_diff = timestep, trans_diff, rot_diff
    s.stress_active, s.stress_magnetic, s.shape = active, magnetic, shape
    s.magnetic_drag, s.hydro_screening, s.volume_exclusion = magnetic_drag, hydro_screening, volume_exclusion
    s.magnetic_reorientation, s.magnetic_dipole_dipole = magnetic_reorientation, magnetic_dipole_dipole
    s.quasi2d = 1 if quasi2d else 0
    s.gather = int(gather)
    s.seed = seed
    return s


def modulo(f, m):
    return lib().orc_modulo(f, m)


def ang_pbc(phi, theta):
    o = np.zeros(2)
    lib().orc_ang_pbc(phi, theta, _p(o))
    return o[0], o[1]


def particle_new(s, p):
    i = np.ascontiguousarray(p, dtype=np.float64)
    o = np.zeros(5)
    lib().orc_particle_new(ctypes.byref(s), _p(i), _p(o))
    return o


def from_vector(v):
    i = np.ascontiguousarray(v, dtype=np.float64)
    o = np.zeros(2)
    lib().orc_from_vector(_p(i), _p(o))
    return o[0], o[1]


def grid_width(s):
    o = np.zeros(5)
    lib().orc_grid_width(ctypes.byref(s), _p(o))
    return o


def coord_to_grid(s, p):
    i = np.ascontiguousarray(p, dtype=np.float64)
    o = np.zeros(5, dtype=np.uint64)
    lib().orc_coord_to_grid(ctypes.byref(s), _p(i), o.ctypes.data_as(c_u64_p))
    return o


def cell_index(s, p):
    i = np.ascontiguousarray(p, dtype=np.float64)
    o = np.zeros(3, dtype=np.uint64)
    lib().orc_cell_index(ctypes.byref(s), _p(i), o.ctypes.data_as(c_u64_p))
    return o


def k_sampling(n, box):
    o = np.zeros(n)
    lib().orc_k_sampling(n, box, _p(o))
    return o


def _ncell(s):
    return s.gx * s.gy * s.gz


def k_mesh(s):
    o = np.zeros((3, s.gx, s.gy, s.gz))
    lib().orc_k_mesh(ctypes.byref(s), _p(o))
    return o


def norm_k_mesh(s):
    o = np.zeros((3, s.gx, s.gy, s.gz))
    lib().orc_norm_k_mesh(ctypes.byref(s), _p(o))
    return o


def inverse_norm_squared(s):
    o = np.zeros((s.gx, s.gy, s.gz))
    lib().orc_inverse_norm_squared(ctypes.byref(s), _p(o))
    return o


def stress_kernel(s):
    o = np.zeros((3, 3, s.gphi, s.gtheta))
    lib().orc_stress_kernel(ctypes.byref(s), _p(o))
    return o


def orientation_kernel(s):
    o = np.zeros((3, s.gphi, s.gtheta))
    lib().orc_orientation_kernel(ctypes.byref(s), _p(o))
    return o


def histogram(s, particles):
    p = np.ascontiguousarray(particles, dtype=np.float64).reshape(-1, 5)
    o = np.zeros((s.gx, s.gy, s.gz, s.gphi, s.gtheta))
    lib().orc_histogram(ctypes.byref(s), _p(p), p.shape[0], _p(o))
    return o


def sample_from(s, particles):
    p = np.ascontiguousarray(particles, dtype=np.float64).reshape(-1, 5)
    o = np.zeros((s.gx, s.gy, s.gz, s.gphi, s.gtheta))
    lib().orc_sample_from(ctypes.byref(s), _p(p), p.shape[0], _p(o))
    return o


def fft3d(a, sign):
    """Unnormalised complex 3-D DFT of a complex array (returns a copy)."""
    z = np.ascontiguousarray(a, dtype=np.complex128).copy()
    nx, ny, nz = z.shape
    lib().orc_fft3d(z.ctypes.data_as(c_double_p), nx, ny, nz, sign)
    return z


def flow_field(s, dist, screening, nthreads=1):
    d = np.ascontiguousarray(dist, dtype=np.float64)
    u = np.zeros((3, s.gx, s.gy, s.gz), dtype=np.complex128)
    g = np.zeros((3, 3, s.gx, s.gy, s.gz), dtype=np.complex128)
    lib().orc_flow_field(ctypes.byref(s), _p(d), screening, u.ctypes.data_as(c_double_p),
                         g.ctypes.data_as(c_double_p), nthreads)
    return u, g


def magnetic_field(s, dist, nthreads=1):
    d = np.ascontiguousarray(dist, dtype=np.float64)
    b = np.zeros((3, s.gx, s.gy, s.gz), dtype=np.complex128)
    g = np.zeros((3, 3, s.gx, s.gy, s.gz), dtype=np.complex128)
    lib().orc_magnetic_field(ctypes.byref(s), _p(d), b.ctypes.data_as(c_double_p),
                             g.ctypes.data_as(c_double_p), nthreads)
    return b, g


def director_field(s, dist):
    d = np.ascontiguousarray(dist, dtype=np.float64)
    p = np.zeros((3, s.gx, s.gy, s.gz), dtype=np.complex128)
    lib().orc_director_field(ctypes.byref(s), _p(d), p.ctypes.data_as(c_double_p))
    return p


def vector_gradient(s, bk):
    b = np.ascontiguousarray(bk, dtype=np.complex128)
    g = np.zeros((3, 3, s.gx, s.gy, s.gz), dtype=np.complex128)
    lib().orc_vector_gradient(ctypes.byref(s), b.ctypes.data_as(c_double_p), g.ctypes.data_as(c_double_p))
    return g


def interpolate(s, field, p, zbug=False):
    f = np.ascontiguousarray(field, dtype=np.float64)
    ncomp = f.shape[0]
    q = np.ascontiguousarray(p, dtype=np.float64)
    o = np.zeros(ncomp)
    lib().orc_interpolate(ctypes.byref(s), _p(f), ncomp, _p(q), 1 if zbug else 0, _p(o))
    return o


def langevin(p, mask, box=(10.0, 10.0, 10.0), **kw):
    a = LangevinArgs()
    a.bx, a.by, a.bz = box
    for k, v in kw.items():
        if isinstance(getattr(a, k), (int, float)):
            setattr(a, k, float(v))
        else:
            arr = getattr(a, k)
            flat = np.asarray(v, dtype=np.float64).ravel()
            for i, x in enumerate(flat):
                arr[i] = x
    i = np.ascontiguousarray(p, dtype=np.float64)
    o = np.zeros(5)
    lib().orc_langevin(_p(i), mask, ctypes.byref(a), _p(o))
    return o


class Simulation:
    """Oracle ``Simulation`` (src/bin/simulation/mod.rs:88-375)."""

    def __init__(self, settings, n, nthreads=1):
        self.s = settings
        self.n = int(n)
        self.ncell = _ncell(settings)
        self.nbins = self.ncell * settings.gphi * settings.gtheta
        self._h = lib().orc_sim_new(ctypes.byref(settings), self.n, int(nthreads))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().orc_sim_free(h)
            self._h = None

    def init(self, particles):
        p = np.ascontiguousarray(particles, dtype=np.float64).reshape(-1, 5)
        rc = lib().orc_sim_init(self._h, _p(p), p.shape[0])
        if rc != 0:
            raise ValueError("number of particles does not match the settings")

    def do_timestep(self, noise=None):
        if noise is None:
            return lib().orc_sim_step(self._h, None)
        z = np.ascontiguousarray(noise, dtype=np.float64).reshape(self.n, 5)
        return lib().orc_sim_step(self._h, _p(z))

    def _view(self, fn, count, shape, dtype=np.float64):
        ptr = getattr(lib(), fn)(self._h)
        a = np.ctypeslib.as_array(ptr, shape=(count,)).copy()
        if dtype == np.complex128:
            a = a.view(np.complex128)
        return a.reshape(shape)

    def particles(self):
        return self._view("orc_sim_particles", 5 * self.n, (self.n, 5))

    def distribution(self):
        s = self.s
        return self._view("orc_sim_distribution", self.nbins, (s.gx, s.gy, s.gz, s.gphi, s.gtheta))

    def flow(self):
        s = self.s
        return self._view("orc_sim_flow", 6 * self.ncell, (3, s.gx, s.gy, s.gz), np.complex128)

    def flow_grad(self):
        s = self.s
        return self._view("orc_sim_flow_grad", 18 * self.ncell, (3, 3, s.gx, s.gy, s.gz), np.complex128)

    def mag(self):
        s = self.s
        return self._view("orc_sim_mag", 6 * self.ncell, (3, s.gx, s.gy, s.gz), np.complex128)

    def mag_grad(self):
        s = self.s
        return self._view("orc_sim_mag_grad", 18 * self.ncell, (3, 3, s.gx, s.gy, s.gz), np.complex128)

    def density(self):
        s = self.s
        return self._view("orc_sim_density", self.ncell, (s.gx, s.gy, s.gz))

    def noise(self):
        return self._view("orc_sim_noise", 5 * self.n, (self.n, 5))

    def timestep(self):
        return lib().orc_sim_timestep(self._h)

    def set_timestep(self, t):
        lib().orc_sim_set_timestep(self._h, int(t))


def max_threads():
    return lib().orc_max_threads()
