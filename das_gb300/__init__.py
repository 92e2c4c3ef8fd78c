"""GB300-native (sm_103a) 2D finite-difference RTM engine.

A drop-in for the RTM path of ll23002/DAS (tsw_rtm/wave_solver.py,
tsw_rtm/rtm_engine.py over tsw_rtm/c_engine/wave2d.c): the same Python entry
points and the same C ABI, with every time step on the GPU.
"""
from __future__ import annotations

from . import _lib

__version__ = "0.1.0"


def lib():
    """The loaded CUDA engine (ctypes.CDLL); raises if it cannot be built or loaded."""
    return _lib.load()


def __getattr__(name):
    # lazy re-exports so that importing the package does not load CUDA
    if name in ("WaveSolver2D", "ricker_wavelet"):
        from . import wave_solver
        return getattr(wave_solver, name)
    if name in ("TSWRTMEngine", "RTMResult", "apply_laplacian_filter"):
        from . import rtm_engine
        return getattr(rtm_engine, name)
    if name in ("FloodModels", "generate_velocity_flood_models"):
        from . import velocity_flood
        return getattr(velocity_flood, name)
    raise AttributeError(name)
