"""Host side of the batched ensembles: member validation in
ss_ensemble_create (before any CUDA call), the parameter-scan generator and
the initial rows.  No GPU."""
import numpy as np
import pytest


def _member(**kw):
    m = dict(grid=(16, 16, 1, 8, 1), box=(5.0, 5.0, 1.0),
             params=dict(timestep=0.01, trans_diffusion=0.1, rot_diffusion=0.5, stress_active=-1.0,
                         number_of_particles=1000, seed=1))
    for k, v in kw.items():
        if k in m:
            m[k] = v
        else:
            m["params"][k] = v
    return m


@pytest.mark.parametrize("bad, text", [
    (dict(grid=(16, 16, 2, 8, 1)), "quasi-2-D"),
    (dict(grid=(16, 16, 1, 8, 2)), "quasi-2-D"),
    (dict(grid=(1, 16, 1, 8, 1)), "quasi-2-D"),
    (dict(grid=(16, 16, 1, 2048, 1)), "quasi-2-D"),
    (dict(box=(5.0, 0.0, 1.0)), "box"),
    (dict(box=(5.0, float("inf"), 1.0)), "box"),
    (dict(number_of_particles=0), "particles"),
    (dict(number_of_particles=1 << 32), "particles"),
    (dict(magnetic_dipole_dipole=0.5), "dipolar"),
    (dict(magnetic_drag=0.1), "dipolar"),
    (dict(timestep=float("nan")), "non-finite"),
])
def test_create_rejects_bad_members(bad, text):
    import stochasticsampling_gb300 as ss
    from stochasticsampling_gb300 import _lib
    with pytest.raises(ss.SsError) as e:
        ss.Ensemble([_member(), _member(**bad)])
    assert e.value.code == _lib.SS_ERR_INVALID_ARGUMENT
    assert text in str(e.value) and "member 1" in str(e.value)


def test_create_rejects_bad_flags_and_sizes():
    import ctypes
    from stochasticsampling_gb300 import _lib
    from stochasticsampling_gb300._lib import Box, Grid, Params
    L = _lib.load()
    h = ctypes.c_void_p()
    g, b, p = (Grid * 1)(Grid(8, 8, 1, 4, 1)), (Box * 1)(Box(1, 1, 1)), (Params * 1)(Params(number_of_particles=5))
    for flags in (0, _lib.FLAG_QUASI2D | _lib.FLAG_NO_SORT, _lib.FLAG_QUASI2D | _lib.FLAG_TRILINEAR):
        assert L.ss_ensemble_create(g, b, p, 1, flags, None, ctypes.byref(h)) == _lib.SS_ERR_INVALID_ARGUMENT
        assert "quasi-2-D and mixed" in _lib.last_error()
    assert L.ss_ensemble_create(g, b, p, 0, _lib.FLAG_QUASI2D, None, ctypes.byref(h)) == _lib.SS_ERR_INVALID_ARGUMENT
    assert L.ss_ensemble_create(None, b, p, 1, _lib.FLAG_QUASI2D, None, ctypes.byref(h)) == \
        _lib.SS_ERR_INVALID_ARGUMENT
    n = 4097
    g, b, p = (Grid * n)(), (Box * n)(), (Params * n)()
    assert L.ss_ensemble_create(g, b, p, n, _lib.FLAG_QUASI2D, None, ctypes.byref(h)) == _lib.SS_ERR_INVALID_ARGUMENT
    assert "at most 4096" in _lib.last_error()
    # other entry points reject a null ensemble
    assert L.ss_ensemble_run(None, 1) == _lib.SS_ERR_INVALID_ARGUMENT
    assert L.ss_ensemble_autotune(None, None) == _lib.SS_ERR_INVALID_ARGUMENT
    assert L.ss_ensemble_set_config(None, None) == _lib.SS_ERR_INVALID_ARGUMENT
    assert L.ss_ensemble_info(None, None, None, None) == _lib.SS_ERR_INVALID_ARGUMENT
    assert L.ss_ensemble_destroy(None) == _lib.SS_OK


def test_parameter_scan_matches_its_ranges():
    from stochasticsampling_gb300.ensemble import parameter_scan, uniform_particles
    members = parameter_scan(64, seed=1)
    assert members == parameter_scan(64, seed=1)
    ns = np.array([m["params"]["number_of_particles"] for m in members])
    assert ns.min() >= 50_000 and ns.max() <= 2_000_000
    assert len({m["params"]["seed"] for m in members}) == 64
    for m in members:
        e = m["grid"][0]
        assert e in (32, 64, 128) and m["grid"] == (e, e, 1, m["grid"][3], 1) and m["grid"][3] in (16, 32)
        assert m["box"][0] == e * 0.3125
        assert -3.0 <= m["params"]["stress_active"] <= 0.0
    small = parameter_scan(3, seed=4, n_range=(100, 1000))
    rows = uniform_particles(small, seed=5)
    assert rows.shape == (sum(m["params"]["number_of_particles"] for m in small), 5)
    assert np.all(rows[:, 2] == 0.0) and np.all(rows[:, 4] == np.pi / 2)
    assert np.all((rows[:, 3] >= 0) & (rows[:, 3] < 2 * np.pi))


def test_denoiser_rejects_bad_shapes_on_the_host():
    import ctypes
    from stochasticsampling_gb300 import _lib
    L = _lib.load()
    h = ctypes.c_void_p()
    for shape in [(5, 5, 5), (0, 128, 1), (128, 128, 0)]:
        assert L.ss_dn_create(*shape, 1, None, ctypes.byref(h)) == _lib.SS_ERR_INVALID_ARGUMENT
        assert "multiple of 128" in _lib.last_error()
    assert L.ss_dn_forward(None, None, None) == _lib.SS_ERR_INVALID_ARGUMENT
    assert L.ss_dn_destroy(None) == _lib.SS_OK
