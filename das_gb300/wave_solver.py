"""Drop-in for tsw_rtm/wave_solver.py backed by the GB300 CUDA engine.

Same names, arguments, return values and error behaviour as the reference
module (ll23002/DAS tsw_rtm/wave_solver.py):

* ``ricker_wavelet``            wave_solver.py:74-81
* ``WaveSolver2D.__init__``     wave_solver.py:89-117 (sponge built by the C ABI's
                                ``build_cerjan_sponge``, host ``expf``)
* ``check_stability``           wave_solver.py:119-126
* ``forward_propagate_acoustic``        wave_solver.py:128-186
* ``backward_propagate_and_correlate``  wave_solver.py:188-242

Where the reference crosses into C once per time step, here each method is one
call into ``libwave2d_cuda.so`` that runs the whole time loop on the device
(fused step kernels; injection, sampling, snapshots and imaging included).
"""
from __future__ import annotations

import ctypes
from typing import Optional, Tuple

import numpy as np

from . import _lib
from .geometry import normalize_index, normalize_indices

__all__ = ["ricker_wavelet", "WaveSolver2D"]


def ricker_wavelet(f0: float, dt: float, t_length: float) -> Tuple[np.ndarray, np.ndarray]:
    """Zero-phase Ricker wavelet: computed in float64, returned as float32."""
    nt = int(round(t_length / dt))
    t = np.arange(nt) * dt
    a = (np.pi * f0 * (t - 1.0 / f0)) ** 2
    w = (1.0 - 2.0 * a) * np.exp(-a)
    return w.astype(np.float32), t


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _is_cuda_tensor(a) -> bool:
    mod = type(a).__module__
    return mod.startswith("torch") and getattr(a, "is_cuda", False)


class WaveSolver2D:
    """2D wavefield propagator on one GB300 (sm_103a) GPU."""

    def __init__(self, nx: int, nz: int, dx: float, dz: float, dt: float, n_sponge: int = 30,
                 sponge_alpha: float = 0.0015, free_surface_top: bool = True,
                 solver_type: str = "acoustic"):
        self.nx = nx
        self.nz = nz
        self.dx = float(dx)
        self.dz = float(dz)
        self.dt = float(dt)
        self.n_sponge = n_sponge
        self.sponge_alpha = float(sponge_alpha)
        self.free_surface_top = free_surface_top
        self.solver_type = solver_type
        self._lib = _lib.load()
        self.sponge = np.ones((nz, nx), dtype=np.float32)
        self._lib.build_cerjan_sponge(self.sponge.ctypes.data, nx, nz, n_sponge, sponge_alpha,
                                      1 if free_surface_top else 0)
        self._sponge0 = self.sponge.copy()
        self._engine = None
        self._engine_sponge = None
        self.storage = "auto"
        self.tile = None  # (warps, rows_per_warp) or None for the default
        self.l2_hints = False  # L2 residency hints in the step kernel
        # step launch: one CTA per tile ("grid") or persistent CTAs ("persistent");
        # each optionally a programmatic dependent of the previous step (pdl)
        self.launch = ("grid", True)
        self.two_step = False  # two time steps per launch (grid launch mode; off by default)
        self.graphs = True  # migrations replay each pass as a captured CUDA graph

    def _default_sponge(self) -> np.ndarray:
        """The Cerjan sponge of this grid's (n_sponge, sponge_alpha) as built at creation."""
        return self._sponge0

    # -- engine handle -----------------------------------------------------------
    def _eng(self):
        sp = self.sponge
        if self._engine is not None and self._engine_sponge is not None and \
                (sp is None) == (self._engine_sponge is None) and \
                (sp is None or np.array_equal(sp, self._engine_sponge)):
            return self._engine
        self.close()
        h = ctypes.c_void_p()
        sp_c = None if sp is None else _f32(sp)
        _lib.check(self._lib.w2d_engine_create(ctypes.byref(h), self.nx, self.nz, self.dx, self.dz,
                                               self.dt, None if sp_c is None else sp_c.ctypes.data,
                                               1 if self.free_surface_top else 0))
        self._engine = h
        self._engine_sponge = None if sp_c is None else sp_c.copy()
        if self.tile is not None:
            _lib.check(self._lib.w2d_engine_set_tile(h, int(self.tile[0]), int(self.tile[1])))
        if self.l2_hints:
            _lib.check(self._lib.w2d_engine_set_l2_hints(h, 1))
        if self.launch != ("grid", True):
            self._apply_launch(h)
        if self.two_step is not False:
            v = 1 if self.two_step is True else int(self.two_step)
            _lib.check(self._lib.w2d_engine_set_two_step(h, v))
        if not self.graphs:
            _lib.check(self._lib.w2d_engine_set_graphs(h, 0))
        return h

    def set_graphs(self, on: bool = True) -> None:
        """Replay each migration pass as a captured CUDA graph (True, the default) or
        launch every step from the host (False).  Results are identical."""
        self.graphs = bool(on)
        if self._engine is not None:
            _lib.check(self._lib.w2d_engine_set_graphs(self._engine, 1 if on else 0))

    def _apply_launch(self, h):
        kind, pdl = self.launch
        if kind not in ("grid", "persistent"):
            raise ValueError("launch kind must be 'grid' or 'persistent'")
        _lib.check(self._lib.w2d_engine_set_launch(h, 1 if kind == "persistent" else 0,
                                                   1 if pdl else 0))

    def set_launch(self, kind: str = "grid", pdl: bool = True) -> None:
        """Choose how the step kernels launch (results are identical in every mode)."""
        self.launch = (kind, bool(pdl))
        if self._engine is not None:
            self._apply_launch(self._engine)

    def set_two_step(self, on=True) -> None:
        """Two time steps per launch (True, or an int 2..4: the tile's rows per warp) or
        one (False, the default: faster on sponge-framed grids).  Results are identical."""
        self.two_step = on if isinstance(on, bool) else int(on)
        if self._engine is not None:
            v = (1 if on else 0) if isinstance(on, bool) else int(on)
            _lib.check(self._lib.w2d_engine_set_two_step(self._engine, v))

    def set_checkpoint_segment(self, steps: int = 0) -> None:
        """Steps per checkpoint segment of the differentiable path (das_gb300.autograd):
        0 picks sqrt(3 nt); nt or more stores every forward state (no recomputation).
        The gradient is the same bit for bit either way."""
        _lib.check(self._lib.w2d_fwi_set_segment(self._eng(), int(steps)))

    def set_adjoint_form(self, form: str = "tiled") -> None:
        """Adjoint kernel of the differentiable path: "tiled" (vectorised, the default) or
        "cells" (the per-cell kernel it is checked against; the same to rounding)."""
        if form not in ("tiled", "cells"):
            raise ValueError("adjoint form must be 'tiled' or 'cells'")
        _lib.check(self._lib.w2d_fwi_set_adjoint_form(self._eng(), 1 if form == "cells" else 0))

    def close(self):
        if getattr(self, "_engine", None) is not None:
            self._lib.w2d_engine_destroy(self._engine)
            self._engine = None
            self._engine_sponge = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _set_velocity(self, slot: int, velocity_model) -> None:
        if _is_cuda_tensor(velocity_model):
            # a device-resident model (e.g. from generate_velocity_flood_models_on_device):
            # copied device to device, after the work that produced it on its stream
            import torch
            t = velocity_model.detach()
            if t.dtype != torch.float32:
                raise TypeError("a device velocity model must be float32")
            t = t.contiguous()
            if tuple(t.shape) != (self.nz, self.nx):
                raise ValueError(f"velocity model shape {tuple(t.shape)} != {(self.nz, self.nx)}")
            torch.cuda.current_stream(t.device).synchronize()
            _lib.check(self._lib.w2d_engine_set_velocity(self._eng(), slot, t.data_ptr()))
            return
        vel = _f32(velocity_model)
        if vel.shape != (self.nz, self.nx):
            raise ValueError(f"velocity model shape {vel.shape} != {(self.nz, self.nx)}")
        _lib.check(self._lib.w2d_engine_set_velocity(self._eng(), slot, vel.ctypes.data))

    def last_stats(self) -> dict:
        st, la, rc, ms = ctypes.c_int(), ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_float()
        _lib.check(self._lib.w2d_engine_last_stats(self._eng(), ctypes.byref(st), ctypes.byref(la),
                                                   ctypes.byref(rc), ctypes.byref(ms)))
        return {"storage": {0: "none", 1: "all", 2: "checkpoint"}.get(st.value, "?"),
                "step_launches": la.value, "recomputed_steps": rc.value, "device_ms": ms.value}

    # -- reference API ---------------------------------------------------------------
    def check_stability(self, max_vel: float, min_vel: float, max_freq: float) -> Tuple[bool, str]:
        """CFL and points-per-wavelength check (wave_solver.py:119-126)."""
        cfl = max_vel * self.dt * np.sqrt(1.0 / (self.dx ** 2) + 1.0 / (self.dz ** 2))
        grid_pts_per_wl = (min_vel / max_freq) / max(self.dx, self.dz)
        msg = (f"CFL number: {cfl:.3f} (target < 0.6). Grid pts per min wavelength: "
               f"{grid_pts_per_wl:.1f} (target >= 5).")
        stable = (cfl < 0.65) and (grid_pts_per_wl >= 4.0)
        return stable, msg

    def forward_propagate_acoustic(self, velocity_model: np.ndarray, source_ts: np.ndarray,
                                   source_ix: int, source_iz: int, receiver_ix: np.ndarray,
                                   receiver_iz: int = 2, save_wavefield: bool = False,
                                   snapshot_interval: int = 1
                                   ) -> Tuple[np.ndarray, Optional[np.ndarray]]:
        """Forward acoustic run: returns (traces (nt, n_rec), snapshots or None)."""
        w = _f32(source_ts).reshape(-1)
        nt = len(w)
        six = normalize_index(source_ix, self.nx, "source_ix")
        siz = normalize_index(source_iz, self.nz, "source_iz")
        rix = normalize_indices(receiver_ix, self.nx, "receiver_ix")
        riz = normalize_index(receiver_iz, self.nz, "receiver_iz")
        n_rec = len(rix)
        rec = np.zeros((nt, n_rec), dtype=np.float32)
        if nt == 0:
            return rec, (np.zeros((0, self.nz, self.nx), np.float32) if save_wavefield else None)
        if snapshot_interval <= 0:
            raise ZeroDivisionError("snapshot_interval must be positive")
        snaps = None
        if save_wavefield:
            snaps = np.empty(((nt - 1) // snapshot_interval + 1, self.nz, self.nx), np.float32)
        self._set_velocity(0, velocity_model)
        _lib.check(self._lib.w2d_forward(
            self._eng(), 0, w.ctypes.data, nt, six, siz, rix.ctypes.data, n_rec, riz,
            rec.ctypes.data, None if snaps is None else snaps.ctypes.data, int(snapshot_interval)))
        return rec, snaps

    def backward_propagate_and_correlate(self, velocity_model: np.ndarray,
                                         receiver_data: np.ndarray, receiver_ix: np.ndarray,
                                         receiver_iz: int, forward_wavefields: np.ndarray,
                                         image_out: np.ndarray, snapshot_interval: int = 1):
        """Back-propagate the time-reversed traces and correlate into image_out (in place)."""
        data = _f32(receiver_data)
        nt, n_rec = data.shape
        rix = normalize_indices(receiver_ix, self.nx, "receiver_ix")
        if len(rix) < n_rec:
            raise IndexError("fewer receiver indices than data columns")
        rix = rix[:n_rec]
        riz = normalize_index(receiver_iz, self.nz, "receiver_iz")
        if not (isinstance(image_out, np.ndarray) and image_out.dtype == np.float32 and
                image_out.flags.c_contiguous and image_out.shape == (self.nz, self.nx)):
            raise ValueError("image_out must be a C-contiguous float32 (nz, nx) array")
        if nt == 0:
            return
        fw = _f32(forward_wavefields)
        if fw.ndim != 3 or fw.shape[1:] != (self.nz, self.nx):
            raise ValueError("forward_wavefields must be (n_snaps, nz, nx)")
        n_snaps = fw.shape[0]
        # The reference only correlates while its snapshot counter, which starts at
        # (nt-1)//interval, indexes a snapshot that exists; with fewer snapshots it
        # never correlates (wave_solver.py:204,230).
        if n_snaps <= (nt - 1) // snapshot_interval:
            n_snaps = 0
        self._set_velocity(1, velocity_model)
        _lib.check(self._lib.w2d_backward_correlate(
            self._eng(), 1, data.ctypes.data, nt, rix.ctypes.data, n_rec, riz,
            fw.ctypes.data if n_snaps else None, n_snaps, image_out.ctypes.data,
            int(snapshot_interval)))
