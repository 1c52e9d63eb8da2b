"""The C-ABI library builds for sm_103a, loads, and exports every entry point
that include/ssgpu.h declares.  No compute call is made here (no GPU)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def _declared():
    text = open(os.path.join(ROOT, "include", "ssgpu.h")).read()
    return sorted(set(re.findall(r"^(?:int|const char \*)\s*(ss_\w+)\(", text, flags=re.M)))


def test_header_and_loader_agree():
    from stochasticsampling_gb300 import _lib
    assert _declared() == sorted(_lib.EXPORTS)


def test_flag_values_agree_with_the_header():
    from stochasticsampling_gb300 import _lib
    text = open(os.path.join(ROOT, "include", "ssgpu.h")).read()
    flags = dict(re.findall(r"^#define SS_(FLAG_\w+)\s+(\d+)u", text, flags=re.M))
    assert "FLAG_F32X2" in flags and len(flags) >= 9
    for name, value in flags.items():
        assert getattr(_lib, name) == int(value), name


def test_library_exports_every_declared_symbol():
    from stochasticsampling_gb300 import _lib
    L = _lib.load()
    for name in _declared():
        assert hasattr(L, name), name
    assert L.ss_version().startswith(b"ssgpu")


def test_invalid_arguments_are_rejected_on_the_host():
    from stochasticsampling_gb300 import _lib
    from stochasticsampling_gb300._lib import Box, Grid, Params
    L = _lib.load()
    h = ctypes.c_void_p()
    p = Params(number_of_particles=10)
    # quasi2d with z != 1 (src/bin/simulation/mod.rs:96-98)
    rc = L.ss_create(ctypes.byref(Grid(4, 4, 2, 4, 1)), ctypes.byref(Box(1, 1, 1)), ctypes.byref(p),
                     _lib.FLAG_QUASI2D, None, ctypes.byref(h))
    assert rc == _lib.SS_ERR_INVALID_ARGUMENT and "quasi2d" in _lib.last_error()
    # box <= 0 (check_settings)
    rc = L.ss_create(ctypes.byref(Grid(4, 4, 1, 4, 1)), ctypes.byref(Box(0, 1, 1)), ctypes.byref(p), 0, None,
                     ctypes.byref(h))
    assert rc == _lib.SS_ERR_INVALID_ARGUMENT and "Box size" in _lib.last_error()
    # zero particles, zero-sized grid
    rc = L.ss_create(ctypes.byref(Grid(4, 4, 1, 4, 1)), ctypes.byref(Box(1, 1, 1)),
                     ctypes.byref(Params(number_of_particles=0)), 0, None, ctypes.byref(h))
    assert rc == _lib.SS_ERR_INVALID_ARGUMENT
    rc = L.ss_create(ctypes.byref(Grid(0, 4, 1, 4, 1)), ctypes.byref(Box(1, 1, 1)), ctypes.byref(p), 0, None,
                     ctypes.byref(h))
    assert rc == _lib.SS_ERR_INVALID_ARGUMENT
    # non-finite parameters
    bad = Params(number_of_particles=10, timestep=float("nan"))
    rc = L.ss_create(ctypes.byref(Grid(4, 4, 1, 4, 1)), ctypes.byref(Box(1, 1, 1)), ctypes.byref(bad), 0, None,
                     ctypes.byref(h))
    assert rc == _lib.SS_ERR_INVALID_ARGUMENT
    # flag combinations the FP64 mode alone supports
    for fl, what in ((_lib.FLAG_MIXED | _lib.FLAG_F32X2, "F32X2"), (_lib.FLAG_FIXED64 | _lib.FLAG_F32X2, "F32X2"),
                     (_lib.FLAG_MIXED | _lib.FLAG_TRILINEAR, "trilinear")):
        h = ctypes.c_void_p()
        rc = L.ss_create(ctypes.byref(Grid(4, 4, 1, 4, 1)), ctypes.byref(Box(1, 1, 1)), ctypes.byref(p),
                         _lib.FLAG_QUASI2D | fl, None, ctypes.byref(h))
        assert rc == _lib.SS_ERR_INVALID_ARGUMENT and what in _lib.last_error() and not h.value
    # null context
    assert L.ss_do_timestep(None, None, None) == _lib.SS_ERR_INVALID_ARGUMENT
    # the overlapped outputs: null context, null result pointer, nothing to free
    assert L.ss_output_begin(None, 0, None, None, None, None, 0) == _lib.SS_ERR_INVALID_ARGUMENT
    assert L.ss_output_wait(None, 0) == _lib.SS_ERR_INVALID_ARGUMENT
    assert L.ss_output_query(None, 0, None) == _lib.SS_ERR_INVALID_ARGUMENT
    assert L.ss_host_alloc(16, None) == _lib.SS_ERR_INVALID_ARGUMENT
    assert L.ss_host_free(None) == _lib.SS_OK


def test_noalloc_refuses_more_rows_than_a_context_on_the_host():
    """ss_sample_distribution_noalloc takes at most 2^32 - 1 rows, like
    ss_create; the refusal comes before any device work (the pointers are
    never dereferenced)."""
    from stochasticsampling_gb300 import _lib
    from stochasticsampling_gb300._lib import Box, Grid
    L = _lib.load()
    fake = ctypes.c_void_p(256)
    for n in (0, 1 << 32):
        rc = L.ss_sample_distribution_noalloc(ctypes.byref(Grid(4, 4, 1, 4, 1)), ctypes.byref(Box(1, 1, 1)),
                                              fake, n, fake, None)
        assert rc == _lib.SS_ERR_INVALID_ARGUMENT
        assert "2^32-1" in _lib.last_error()


def test_no_cpu_fallback_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from stochasticsampling_gb300 import SsError, Simulation
    with pytest.raises(SsError):
        Simulation(grid=(4, 4, 1, 4, 1), box=(1, 1, 1), params=dict(number_of_particles=8), quasi2d=True)
