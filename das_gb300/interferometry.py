"""Drop-in for tsw_rtm/interferometry.py on the GB300, plus the pipeline's gather
resampling and a device-resident cross-correlation stack.

* ``VirtualShotGather``              interferometry.py:13-23
* ``compute_cross_correlation``      interferometry.py:26-79 (direct sum on the GPU,
  exact products accumulated in double-float arithmetic, same rows and lag axis)
* ``time_derivative_greens``         interferometry.py:82-102
* ``full_green_function``            interferometry.py:105-109
* ``build_virtual_shot_gather``      interferometry.py:112-163
* ``resample_gather_to_sim_dt``      run_das_pipeline.py:48-55
* ``CrossCorrelationStack``          the pipeline's window loop and stack
  (run_das_pipeline.py:202-213, :248-250) for many virtual sources at once, the
  stack kept in device memory.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Dict, Optional, Sequence, Tuple

import numpy as np

from . import _lib

__all__ = ["VirtualShotGather", "compute_cross_correlation", "time_derivative_greens",
           "full_green_function", "build_virtual_shot_gather", "resample_gather_to_sim_dt",
           "CrossCorrelationStack"]


@dataclass
class VirtualShotGather:
    source_idx: int
    source_channel: int
    source_coord_x: float
    receiver_channels: np.ndarray
    receiver_coords_x: np.ndarray
    offsets: np.ndarray
    time_axis: np.ndarray
    shot_gather: np.ndarray  # shape: (nt, n_receivers)
    dt: float


def _channels(idx, n_ch: int, what: str) -> np.ndarray:
    a = np.asarray(idx).reshape(-1)
    if a.size and not np.issubdtype(a.dtype, np.integer):
        raise IndexError(f"{what} must be integers")
    a = a.astype(np.int64)
    if np.any(a >= n_ch) or np.any(a < -n_ch):
        raise IndexError(f"{what} out of range for {n_ch} channels")
    return np.ascontiguousarray(np.where(a < 0, a + n_ch, a), dtype=np.int32)


class CrossCorrelationStack:
    """Cross-correlations of several virtual-source channels against a set of receiver
    channels, stacked over data windows on the device.

    ``add(window)`` takes one (nt_w, n_channels) float32 window with nt_w <= nt (host
    array, or a CUDA torch tensor through ``add_device``) whose correlation rows agree
    with the stack's (as NumPy's in-place sum requires); ``result()`` returns {source
    channel: (ccfs, lags)} exactly as the pipeline's stack after ``/= n_files``."""

    def __init__(self, nt: int, n_channels: int, source_channels: Sequence[int],
                 receiver_indices: Optional[Sequence[int]], max_lag_seconds: float, dt: float):
        self._lib = _lib.load()
        self.nt, self.n_channels, self.dt = int(nt), int(n_channels), float(dt)
        self.sources = _channels(source_channels, self.n_channels, "source channel")
        rec = np.arange(self.n_channels) if receiver_indices is None else receiver_indices
        self.receivers = _channels(rec, self.n_channels, "receiver_indices")
        self.n_lags = int(round(max_lag_seconds / dt))
        h = ctypes.c_void_p()
        _lib.check(self._lib.w2d_xcorr_create(ctypes.byref(h), self.nt, self.n_channels,
                                              self.sources.ctypes.data, len(self.sources),
                                              self.receivers.ctypes.data, len(self.receivers),
                                              self.n_lags))
        self._h = h
        lag0, rows = ctypes.c_int(), ctypes.c_int()
        _lib.check(self._lib.w2d_xcorr_shape(h, ctypes.byref(lag0), ctypes.byref(rows)))
        self.n_rows = rows.value
        self.lags = np.arange(-self.n_lags, self.n_lags + 1) * self.dt
        self.windows = 0

    def add(self, window: np.ndarray) -> None:
        w = np.ascontiguousarray(window, dtype=np.float32)
        if w.ndim != 2 or w.shape[1] != self.n_channels or not 1 <= w.shape[0] <= self.nt:
            raise ValueError(f"window shape {w.shape} does not fit (<= {self.nt}, "
                             f"{self.n_channels})")
        _lib.check(self._lib.w2d_xcorr_add(self._h, w.ctypes.data, w.shape[0]))
        self.windows += 1

    def add_device(self, window) -> None:
        """A CUDA tensor (nt, n_channels), float32, contiguous (synchronised first)."""
        import torch
        if window.dim() != 2 or window.shape[1] != self.n_channels or \
                not 1 <= window.shape[0] <= self.nt or window.dtype != torch.float32 \
                or not window.is_cuda or not window.is_contiguous():
            raise ValueError("expected a contiguous float32 CUDA tensor (nt_w, n_channels)")
        torch.cuda.current_stream().synchronize()
        _lib.check(self._lib.w2d_xcorr_add_device(self._h, window.data_ptr(),
                                                  int(window.shape[0])))
        self.windows += 1

    def result(self, divide: bool = True) -> Dict[int, Tuple[np.ndarray, np.ndarray]]:
        out = np.empty((len(self.sources), self.n_rows, len(self.receivers)), np.float32)
        _lib.check(self._lib.w2d_xcorr_read(self._h, out.ctypes.data if out.size else None,
                                            1 if divide else 0))
        return {int(s): (out[k], self.lags.copy()) for k, s in enumerate(self.sources)}

    def close(self):
        if getattr(self, "_h", None) is not None:
            self._lib.w2d_xcorr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def compute_cross_correlation(data: np.ndarray, source_channel_idx: int, max_lag_seconds: float,
                              dt: float, receiver_indices: Optional[np.ndarray] = None
                              ) -> Tuple[np.ndarray, np.ndarray]:
    """Cross-correlations of one source channel with the receiver channels
    (interferometry.py:26-79): (ccfs float32 (rows, n_receivers), lags in seconds)."""
    d = np.asarray(data)
    if d.ndim != 2:
        raise ValueError("data must be (nt, n_channels)")
    st = CrossCorrelationStack(d.shape[0], d.shape[1], [source_channel_idx], receiver_indices,
                               max_lag_seconds, dt)
    try:
        st.add(d)
        ccfs, lags = st.result(divide=False)[int(st.sources[0])]
    finally:
        st.close()
    return ccfs, lags


def time_derivative_greens(ccfs: np.ndarray, dt: float, scheme: str = "central") -> np.ndarray:
    """d(C_AB)/dt (interferometry.py:82-102): 'central' is np.gradient along axis 0
    (bit-identical), any other value the frequency-domain i*omega*C(omega)."""
    c = np.ascontiguousarray(ccfs, dtype=np.float32)
    if c.ndim != 2:
        raise ValueError("ccfs must be (n_lags, n_receivers)")
    out = np.empty_like(c)
    _lib.check(_lib.load().w2d_time_derivative(c.ctypes.data, c.shape[0], c.shape[1],
                                               float(dt), 0 if scheme == "central" else 1,
                                               out.ctypes.data))
    return out


def full_green_function(ccfs: np.ndarray, lags: np.ndarray) -> np.ndarray:
    """Green's function over the full lag axis (-T..+T), keeping the acausal branch."""
    return time_derivative_greens(ccfs, float(lags[1] - lags[0]))


_BRANCH = {"causal": 0, "anticausal": 1, "symmetric": 2}


def build_virtual_shot_gather(ccfs: np.ndarray, lags: np.ndarray, source_idx: int,
                              source_channel: int, channel_coords_x: np.ndarray,
                              receiver_indices: np.ndarray, branch: str = "causal",
                              take_derivative: bool = True) -> VirtualShotGather:
    """Virtual shot gather from CCFs (interferometry.py:112-163)."""
    if branch not in _BRANCH:
        raise ValueError(f"Unknown branch option: {branch}")
    dt = float(lags[1] - lags[0])
    zero_idx = int(np.argmin(np.abs(lags)))
    processed = time_derivative_greens(ccfs, dt) if take_derivative else \
        np.ascontiguousarray(ccfs, dtype=np.float32)
    n, nc = processed.shape
    if zero_idx >= n:
        raise IndexError("the lag axis is longer than the correlation rows")
    out = np.empty((n, nc), np.float32)
    m = ctypes.c_int()
    _lib.check(_lib.load().w2d_virtual_branch(processed.ctypes.data, n, nc, zero_idx,
                                              _BRANCH[branch], out.ctypes.data, ctypes.byref(m)))
    gather = out[:m.value]
    if branch == "causal":
        time_axis = lags[zero_idx:]
    elif branch == "anticausal":
        time_axis = np.abs(lags[:zero_idx + 1][::-1])
    else:
        time_axis = lags[zero_idx:zero_idx + m.value]
    src_x = float(channel_coords_x[source_channel])
    rec_x = channel_coords_x[receiver_indices]
    return VirtualShotGather(source_idx=source_idx, source_channel=source_channel,
                             source_coord_x=src_x, receiver_channels=receiver_indices,
                             receiver_coords_x=rec_x, offsets=np.abs(rec_x - src_x),
                             time_axis=time_axis, shot_gather=gather, dt=dt)


def resample_gather_to_sim_dt(gather: np.ndarray, dt_orig: float, dt_sim: float,
                              target_nt: int) -> np.ndarray:
    """Linear interpolation of the gather's time axis to the simulation step
    (run_das_pipeline.py:48-55), zero outside the recorded time span."""
    g = np.ascontiguousarray(gather, dtype=np.float32)
    if g.ndim != 2:
        raise ValueError("gather must be (nt, n_receivers)")
    out = np.empty((int(target_nt), g.shape[1]), np.float32)
    _lib.check(_lib.load().w2d_resample_linear(g.ctypes.data, g.shape[0], g.shape[1],
                                               float(dt_orig), float(dt_sim), int(target_nt),
                                               out.ctypes.data))
    return out
