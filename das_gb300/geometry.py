"""Source/receiver grid-index mapping, bit-exact with the reference drivers.

* ``linspace_indices``: ``np.linspace(start, stop, n, dtype=int)``
  (run_synthetic_benchmarks.py:50-51).
* ``halve_indices``: ``int(round(s / 2))`` per index, i.e. round half to even
  (run_das_pipeline.py:350-351).
* ``normalize_index``: NumPy indexing semantics for a scalar index into an axis
  of length n (negative values count from the end, others raise IndexError), as
  the reference's ``p_curr[iz, ix] += ...`` applies them.
"""
from __future__ import annotations

import numpy as np


def linspace_indices(start: float, stop: float, n: int) -> np.ndarray:
    return np.linspace(start, stop, n, dtype=int)


def halve_indices(idx) -> np.ndarray:
    a = np.asarray(idx, dtype=np.float64) / 2.0
    return np.rint(a).astype(int)


def normalize_index(i: int, n: int, what: str = "index") -> int:
    i = int(i)
    if i < -n or i >= n:
        raise IndexError(f"{what} {i} is out of bounds for axis with size {n}")
    return i + n if i < 0 else i


def normalize_indices(idx, n: int, what: str = "index") -> np.ndarray:
    a = np.asarray(idx)
    if a.ndim != 1:
        a = a.reshape(-1)
    if a.size and not np.issubdtype(a.dtype, np.integer):
        raise IndexError(f"{what} must be integers")
    a = a.astype(np.int64)
    if a.size and (a.min() < -n or a.max() >= n):
        raise IndexError(f"{what} out of bounds for axis with size {n}")
    return np.where(a < 0, a + n, a).astype(np.int32)
