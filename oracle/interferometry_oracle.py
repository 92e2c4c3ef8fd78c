"""CPU oracle of the virtual-source gather generation (test infrastructure only).

Restates, in NumPy, the reference's ambient-noise interferometry step that feeds
the RTM engine:

* ``cross_correlation``   tsw_rtm/interferometry.py:26-79 -- FFT cross-correlation
  ``irfft(conj(rfft(src)) * rfft(rec))`` at the input's precision (NumPy 2 computes
  the FFT of float32 data in float32), fftshift, rows ``[n_fft//2 - n_lags,
  n_fft//2 + n_lags + 1)`` with Python slice semantics;
* ``correlation_exact``   the same rows from a float64 direct sum (error statements);
* ``gradient_central``    interferometry.py:82-93 (``np.gradient``, float32);
* ``derivative_frequency`` interferometry.py:94-102;
* ``branch``              interferometry.py:112-163 (causal / anticausal / symmetric);
* ``resample_linear``     run_das_pipeline.py:48-55 (``interp1d`` linear, zero fill).

Only the tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU baseline use
this module; the product path is the CUDA library.
"""
from __future__ import annotations

from typing import List, Tuple

import numpy as np


def fft_size(nt: int) -> int:
    return int(2 ** np.ceil(np.log2(2 * nt - 1)))


def lag_rows(nt: int, max_lag_seconds: float, dt: float) -> Tuple[np.ndarray, np.ndarray]:
    """Lags (in samples) of the rows the reference keeps, and its returned lag axis.

    The kept rows are ``range(n_fft)[center - n_lags : center + n_lags + 1]`` of the
    fftshifted correlation (Python slice semantics, so a start below zero wraps),
    row i holding lag i - center.  The lag axis is ``arange(-n_lags, n_lags + 1) * dt``
    whatever rows were kept (interferometry.py:70-78)."""
    n_fft = fft_size(nt)
    n_lags = int(round(max_lag_seconds / dt))
    center = n_fft // 2
    rows = np.arange(n_fft)[center - n_lags:center + n_lags + 1]
    return rows - center, np.arange(-n_lags, n_lags + 1) * dt


def cross_correlation(data, source_channel_idx, max_lag_seconds, dt, receiver_indices=None):
    """interferometry.py:26-79 step for step."""
    nt, n_ch = data.shape
    if receiver_indices is None:
        receiver_indices = np.arange(n_ch)
    n_fft = fft_size(nt)
    n_lags = int(round(max_lag_seconds / dt))
    s = np.conjugate(np.fft.rfft(data[:, source_channel_idx], n=n_fft))
    r = np.fft.rfft(data[:, receiver_indices], n=n_fft, axis=0)
    cc = np.fft.fftshift(np.fft.irfft(s[:, None] * r, n=n_fft, axis=0), axes=0)
    c = n_fft // 2
    return cc[c - n_lags:c + n_lags + 1, :].astype(np.float32), np.arange(-n_lags, n_lags + 1) * dt


def correlation_exact(data, source_channel_idx, max_lag_seconds, dt, receiver_indices=None):
    """The reference's rows from a float64 direct sum sum_t s[t] r[t + lag]."""
    nt, n_ch = data.shape
    if receiver_indices is None:
        receiver_indices = np.arange(n_ch)
    lags, _ = lag_rows(nt, max_lag_seconds, dt)
    s = data[:, source_channel_idx].astype(np.float64)
    r = data[:, receiver_indices].astype(np.float64)
    out = np.zeros((len(lags), r.shape[1]))
    for i, l in enumerate(lags):
        if abs(l) >= nt:
            continue
        if l >= 0:
            out[i] = s[:nt - l] @ r[l:]
        else:
            out[i] = s[-l:] @ r[:nt + l]
    return out


def gradient_central(c: np.ndarray, dt: float) -> np.ndarray:
    """np.gradient(c, dt, axis=0) for float32 c: float32 differences divided by
    float32(2*dt) inside, one-sided (f[1]-f[0])/float32(dt) at the two ends."""
    c = np.asarray(c, np.float32)
    out = np.empty_like(c)
    out[1:-1] = (c[2:] - c[:-2]) / np.float32(2.0 * dt)
    out[0] = (c[1] - c[0]) / np.float32(dt)
    out[-1] = (c[-1] - c[-2]) / np.float32(dt)
    return out


def derivative_frequency(c: np.ndarray, dt: float) -> np.ndarray:
    """interferometry.py:94-102: i*omega*C(omega) at n_fft = 2^ceil(log2(nt))."""
    nt = c.shape[0]
    n_fft = int(2 ** np.ceil(np.log2(nt)))
    omega = 2.0 * np.pi * np.fft.rfftfreq(n_fft, d=dt)
    d = 1j * omega[:, None] * np.fft.rfft(c, n=n_fft, axis=0)
    return np.fft.irfft(d, n=n_fft, axis=0)[:nt, :].astype(np.float32)


def branch(processed: np.ndarray, lags: np.ndarray, which: str):
    """Causal rows from lag 0, anticausal rows reversed, or their float32 mean."""
    zero = int(np.argmin(np.abs(lags)))
    if which == "causal":
        return processed[zero:, :], lags[zero:]
    if which == "anticausal":
        return np.flip(processed[:zero + 1, :], axis=0), np.abs(lags[:zero + 1][::-1])
    if which == "symmetric":
        pos = processed[zero:, :]
        neg = np.flip(processed[:zero + 1, :], axis=0)
        m = min(pos.shape[0], neg.shape[0])
        return 0.5 * (pos[:m, :] + neg[:m, :]), lags[zero:zero + m]
    raise ValueError(f"Unknown branch option: {which}")


def resample_linear(gather: np.ndarray, dt_orig: float, dt_sim: float, target_nt: int):
    """Linear interpolation of each column from t = i*dt_orig to t = j*dt_sim with zero
    outside [0, (nt-1)*dt_orig]: the arithmetic of scipy's interp1d(kind='linear')
    (scipy 1.18): float64 weights (t - x_lo)/(x_hi - x_lo) and (x_hi - t)/(x_hi - x_lo),
    y_new = w_hi*y_hi + w_lo*y_lo in float64, then float32."""
    y = np.asarray(gather, np.float32)
    n = y.shape[0]
    x = np.arange(n) * dt_orig
    xn = np.arange(target_nt) * dt_sim
    hi = np.clip(np.searchsorted(x, xn), 1, n - 1)
    lo = hi - 1
    span = x[hi] - x[lo]
    out = ((xn - x[lo]) / span)[:, None] * y[hi] + ((x[hi] - xn) / span)[:, None] * y[lo]
    out[(xn < x[0]) | (xn > x[-1])] = 0.0
    return out.astype(np.float32)


def stack(ccfs: List[np.ndarray]) -> np.ndarray:
    """The pipeline's stack: float32 sum in file order, then division by the count."""
    acc = ccfs[0].copy()
    for c in ccfs[1:]:
        acc += c
    acc /= len(ccfs)
    return acc
