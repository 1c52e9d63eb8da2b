"""GB300-native (sm_103a) timestep of stochasticsampling.

The per-timestep hot path of the reference -- binning, angular contraction,
spectral Stokes and dipolar solves, nearest-cell field gather, Euler-Maruyama
Langevin update with periodic wrap -- runs as hand-written CUDA kernels (plus
cuFFT for the grid transforms) behind the C ABI of ``include/ssgpu.h``.  This
package is the host-side mirror of the reference's Simulation and settings.
"""
from . import _lib
from ._lib import SsError
from .settings import read_parameter_file, parse_settings, Settings, SettingsError
from .simulation import Simulation, langevin
from .ensemble import Ensemble

__all__ = ["Simulation", "Ensemble", "langevin", "read_parameter_file", "parse_settings", "Settings", "SettingsError",
           "SsError", "load_library"]


def load_library():
    """Load (building if needed) libssgpu.so and return the ctypes handle."""
    return _lib.load()
