"""Page-locked host arrays for fast shot transfers.

``pinned_array(shape)`` returns a float32 numpy array whose memory comes from
``w2d_host_alloc`` (cudaMallocHost) and is freed when the array is collected.
Passing such arrays to ``WaveSolver2D`` / ``TSWRTMEngine`` methods makes their
host<->device copies run at full link bandwidth.
"""
from __future__ import annotations

import ctypes
import weakref

import numpy as np

from . import _lib


def pinned_array(shape, dtype=np.float32) -> np.ndarray:
    lib = _lib.load()
    dtype = np.dtype(dtype)
    n = int(np.prod(shape)) if len(shape) else 1
    nbytes = max(1, n * dtype.itemsize)
    ptr = ctypes.c_void_p()
    _lib.check(lib.w2d_host_alloc(ctypes.byref(ptr), nbytes))
    buf = (ctypes.c_char * nbytes).from_address(ptr.value)
    arr = np.frombuffer(buf, dtype=dtype, count=n).reshape(shape)
    weakref.finalize(buf, lib.w2d_host_free, ptr.value)
    return arr
