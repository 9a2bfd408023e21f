"""cuimg_gb300: cuimg's semi-dense tracking hot path, GB300-native.

CUDA kernels for sm_103a behind the C ABI of include/cuimg_gb300.h; this
package holds the ctypes bindings and a host-side mirror of the reference's
tracker<F> / particle_container interface.  There is no CPU fallback: every
operation runs the CUDA library and fails loudly when it is missing.
"""
from . import synth  # noqa: F401
from ._native import GbtError, cuda_lib  # noqa: F401
from .tracker import BatchTracker, Tracker, sizes_ok  # noqa: F401

__all__ = ["Tracker", "BatchTracker", "GbtError", "sizes_ok", "synth", "cuda_lib"]
