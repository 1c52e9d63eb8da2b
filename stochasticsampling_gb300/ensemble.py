"""Batched ensembles of independent quasi-2-D simulations over the C ABI
(``ss_ensemble_*`` of include/ssgpu.h).

The reference runs one simulation per process (src/bin/simulation/main.rs); a
parameter scan or an ensemble average runs the binary once per parameter set.
``Ensemble`` steps many such simulations together on one GPU:

    ens = Ensemble([dict(grid=(64, 64, 1, 16, 1), box=(20, 20, 1), params=p0),
                    settings_1, ...])
    ens.init([particles_0, particles_1, ...])     # (n_m, 5) arrays
    ens.run(100)
    ens.get_particles(m), ens.get_counts(m), ens.get_flow_field(m)

Member m evolves like ``Simulation(..., quasi2d=True, mixed=True)`` with the
same grid, box and parameters (FP32 arithmetic, FP64 positions, Philox noise
keyed by the member's seed).  There is no CPU fallback.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import Box, Grid, Params, check
from .simulation import geometry_from_settings

_dp = ctypes.POINTER(ctypes.c_double)


def parameter_scan(count=64, seed=0, n_range=(50_000, 2_000_000), edges=(32, 64, 128), phi_bins=(16, 32),
                   active_range=(-3.0, 0.0), cell_width=0.3125, timestep=0.005, trans_diffusion=0.1,
                   rot_diffusion=1.0):
    """Members of a seeded random parameter scan of 2-D simulations: particle
    count log-uniform in n_range, square grid edge from `edges` (box edge =
    edge x cell_width), phi bins from `phi_bins`, active stress uniform in
    active_range, member m seeded with seed * 1000003 + m."""
    rng = np.random.default_rng(seed)
    members = []
    for m in range(count):
        n = int(round(np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1])))))
        e = int(rng.choice(edges))
        nphi = int(rng.choice(phi_bins))
        active = float(rng.uniform(*active_range))
        members.append(dict(grid=(e, e, 1, nphi, 1), box=(e * cell_width, e * cell_width, 1.0),
                            params=dict(timestep=timestep, trans_diffusion=trans_diffusion,
                                        rot_diffusion=rot_diffusion, stress_active=active, number_of_particles=n,
                                        seed=seed * 1000003 + m)))
    return members


def uniform_particles(members, seed=0):
    """Seeded uniform initial rows (x, y, 0, phi, pi/2) for every member, one
    (sum n_m, 5) array."""
    rng = np.random.default_rng(seed)
    out = []
    for m in members:
        n = int(m["params"]["number_of_particles"])
        bx, by = m["box"][0], m["box"][1]
        out.append(np.column_stack([bx * rng.random(n), by * rng.random(n), np.zeros(n),
                                    2 * np.pi * rng.random(n), np.full(n, np.pi / 2)]))
    return np.concatenate(out)


class Ensemble:
    """Independent quasi-2-D simulations stepped together on the current CUDA device."""

    def __init__(self, members, stream=None):
        self.lib = _lib.load()
        geo = []
        for m in members:
            if isinstance(m, dict):
                geo.append((tuple(int(v) for v in m["grid"]), tuple(float(v) for v in m["box"]), dict(m["params"])))
            else:
                g, b, p = geometry_from_settings(m)
                geo.append((tuple(int(v) for v in g), tuple(float(v) for v in b), p))
        count = len(geo)
        if count == 0:
            raise ValueError("an ensemble needs at least one member")
        grids = (Grid * count)(*[Grid(*g) for g, _, _ in geo])
        boxes = (Box * count)(*[Box(*b) for _, b, _ in geo])
        params = (Params * count)()
        for i, (_, _, p) in enumerate(geo):
            for k, v in p.items():
                setattr(params[i], k, v)
        self.members = geo
        self.n = [int(params[i].number_of_particles) for i in range(count)]
        self.offsets = np.concatenate([[0], np.cumsum(self.n)]).astype(np.int64)
        h = ctypes.c_void_p()
        check(self.lib.ss_ensemble_create(grids, boxes, params, count, _lib.FLAG_QUASI2D | _lib.FLAG_MIXED,
                                          ctypes.c_void_p(stream) if stream else None, ctypes.byref(h)))
        self._h = h

    def __len__(self):
        return len(self.members)

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self.lib.ss_ensemble_destroy(h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def init(self, particles):
        """particles: one (n_m, 5) array per member, or one (sum n_m, 5) array
        with the members' rows one after the other (z = 0, theta = pi/2)."""
        if isinstance(particles, (list, tuple)):
            particles = np.concatenate([np.asarray(p, dtype=np.float64).reshape(-1, 5) for p in particles])
        p = np.ascontiguousarray(particles, dtype=np.float64).reshape(-1, 5)
        check(self.lib.ss_ensemble_init(self._h, p.ctypes.data_as(_dp), p.shape[0]))

    def autotune(self):
        """Time the update's launch shapes and keep the fastest; returns
        (threads per block, blocks per SM, particles per work unit, register plan)."""
        cfg = (ctypes.c_uint32 * 4)()
        check(self.lib.ss_ensemble_autotune(self._h, cfg))
        return tuple(int(v) for v in cfg)

    def set_config(self, config):
        """Set the update's launch shape (the 4-tuple autotune returns)."""
        cfg = (ctypes.c_uint32 * 4)(*[int(v) for v in config])
        check(self.lib.ss_ensemble_set_config(self._h, cfg))

    def run(self, steps):
        check(self.lib.ss_ensemble_run(self._h, int(steps)))

    def synchronize(self):
        check(self.lib.ss_ensemble_synchronize(self._h))

    def _member(self, member):
        member = int(member)
        if not 0 <= member < len(self.members):
            raise IndexError(f"member {member} of an ensemble of {len(self.members)}")
        return member

    def get_particles(self, member):
        member = self._member(member)
        out = np.empty((self.n[member], 5))
        check(self.lib.ss_ensemble_get_particles(self._h, int(member), out.ctypes.data_as(_dp)))
        return out

    def get_counts(self, member):
        member = self._member(member)
        g = self.members[member][0]
        out = np.empty(g, dtype=np.uint32)
        check(self.lib.ss_ensemble_get_counts(self._h, int(member),
                                              out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))))
        return out

    def get_flow_field(self, member):
        member = self._member(member)
        gx, gy, gz = self.members[member][0][:3]
        out = np.empty((3, gx, gy, gz))
        check(self.lib.ss_ensemble_get_flow_field(self._h, int(member), out.ctypes.data_as(_dp)))
        return out

    def info(self):
        """(total particles, grid-shape groups, kernel launches so far)"""
        n, g, nl = ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_uint64()
        check(self.lib.ss_ensemble_info(self._h, ctypes.byref(n), ctypes.byref(g), ctypes.byref(nl)))
        return n.value, g.value, nl.value
