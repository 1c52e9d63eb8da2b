"""ss_sample_distribution_noalloc, the entry point for callers that cannot
allocate device memory at the point where they need a histogram (a hook
inside another library's loop, where cudaFree's device-wide synchronisation
would stall that loop, or an application under a fixed memory budget).

It must give the same distribution as the allocating path (ss_init +
ss_get_distribution on a context) -- bit-exact, like every histogram here --
on two calls in a row, since every call reuses and clears the same static
scratch array.  This file is collected last so that a failure here never hides
the other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PI = np.pi


def _setup():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import stochasticsampling_gb300 as ss
    from stochasticsampling_gb300 import _lib
    return torch, ss, _lib, _lib.load()


def _cloud(rng, n, box, quasi2d):
    th = np.full(n, PI / 2) if quasi2d else np.arccos(1 - 2 * rng.random(n))
    z = np.zeros(n) if quasi2d else box[2] * rng.random(n)
    p = np.column_stack([box[0] * rng.random(n), box[1] * rng.random(n), z, 2 * PI * rng.random(n), th])
    # rows the sanitising Particle::new has to wrap
    p[:50, 0] -= 2.5 * box[0]
    p[50:100, 3] += 4 * PI
    return p


def _noalloc(torch, L, _lib, grid, box, particles, stream=None):
    dev_p = torch.tensor(particles, dtype=torch.float64, device="cuda")
    nbins = int(np.prod(grid))
    out = torch.full((nbins,), float("nan"), dtype=torch.float64, device="cuda")
    rc = L.ss_sample_distribution_noalloc(ctypes.byref(_lib.Grid(*grid)), ctypes.byref(_lib.Box(*box)),
                                          ctypes.c_void_p(dev_p.data_ptr()), particles.shape[0],
                                          ctypes.c_void_p(out.data_ptr()), stream)
    torch.cuda.synchronize()
    _lib.check(rc)
    return out.cpu().numpy().reshape(grid)


@pytest.mark.parametrize("grid,box,quasi2d", [((32, 32, 1, 16, 1), (10.0, 10.0, 1.0), True),
                                              ((9, 7, 5, 5, 3), (4.5, 3.5, 2.5), False)])
def test_noalloc_matches_allocating_path_twice(grid, box, quasi2d):
    torch, ss, _lib, L = _setup()
    rng = np.random.default_rng(7)
    n = 100_000
    p = _cloud(rng, n, box, quasi2d)
    sim = ss.Simulation(grid=grid, box=box, params=dict(number_of_particles=n), quasi2d=quasi2d)
    sim.init(p)
    want = sim.get_distribution()
    sim.close()
    first = _noalloc(torch, L, _lib, grid, box, p)
    second = _noalloc(torch, L, _lib, grid, box, p)
    assert np.array_equal(first, want)
    assert np.array_equal(second, want)


def test_noalloc_clears_between_different_calls():
    torch, ss, _lib, L = _setup()
    rng = np.random.default_rng(8)
    grid, box = (16, 12, 1, 8, 1), (8.0, 6.0, 1.0)
    a = _cloud(rng, 30_000, box, True)
    b = _cloud(rng, 5_000, box, True)
    want = []
    for p in (a, b):
        sim = ss.Simulation(grid=grid, box=box, params=dict(number_of_particles=p.shape[0]), quasi2d=True)
        sim.init(p)
        want.append(sim.get_distribution())
        sim.close()
    assert np.array_equal(_noalloc(torch, L, _lib, grid, box, a), want[0])
    assert np.array_equal(_noalloc(torch, L, _lib, grid, box, b), want[1])


def test_noalloc_rejects_grids_beyond_its_scratch():
    torch, ss, _lib, L = _setup()
    grid = (64, 64, 64, 16, 8)  # 33.5 M bins > SS_NOALLOC_MAX_BINS
    dummy = torch.zeros((1, 5), dtype=torch.float64, device="cuda")
    rc = L.ss_sample_distribution_noalloc(ctypes.byref(_lib.Grid(*grid)), ctypes.byref(_lib.Box(1.0, 1.0, 1.0)),
                                          ctypes.c_void_p(dummy.data_ptr()), 1, ctypes.c_void_p(dummy.data_ptr()),
                                          None)
    assert rc == _lib.SS_ERR_INVALID_ARGUMENT
    assert "at most 2097152" in _lib.last_error()


def test_noalloc_marks_a_non_finite_row_and_recovers():
    """A row with a NaN coordinate (which ss_init refuses) is not counted and
    turns every bin into NaN; the next call with finite rows is exact again."""
    torch, ss, _lib, L = _setup()
    rng = np.random.default_rng(9)
    grid, box = (16, 12, 1, 8, 1), (8.0, 6.0, 1.0)
    good = _cloud(rng, 20_000, box, True)
    bad = good.copy()
    bad[777, 3] = np.nan
    assert np.isnan(_noalloc(torch, L, _lib, grid, box, bad)).all()
    sim = ss.Simulation(grid=grid, box=box, params=dict(number_of_particles=good.shape[0]), quasi2d=True)
    sim.init(good)
    want = sim.get_distribution()
    sim.close()
    assert np.array_equal(_noalloc(torch, L, _lib, grid, box, good), want)
