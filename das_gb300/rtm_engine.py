"""Drop-in for tsw_rtm/rtm_engine.py backed by the GB300 CUDA engine.

* ``RTMResult``                        rtm_engine.py:16-24
* ``apply_laplacian_filter``           rtm_engine.py:27-38
* ``TSWRTMEngine.migrate_shot``        rtm_engine.py:49-104: forward modelling in the
  sediment-flood model with snapshots and illumination, then back-propagation in the
  rock-flood model with zero-lag imaging, in ONE call into the library; the forward
  wavefield never leaves the device (kept whole, or checkpointed and recomputed).
  The flood models may be host arrays or CUDA tensors already on the device (e.g.
  from ``generate_velocity_flood_models_on_device``).
* ``TSWRTMEngine.migrate_multiple_shots``  rtm_engine.py:106-171: the shot images are
  stacked on the device; sponge mute, illumination normalisation and the Laplacian
  run on the stacked image as the reference does.  On grids too small for one shot
  to fill the GPU the shots run as one batch (every launch advances all of them,
  das_gb300.batch); their images are stacked in shot order, so the result is the
  same bit for bit.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Tuple

import numpy as np

from . import _lib
from .geometry import normalize_index, normalize_indices
from .velocity_flood import FloodModels
from .wave_solver import WaveSolver2D, ricker_wavelet

__all__ = ["RTMResult", "apply_laplacian_filter", "TSWRTMEngine", "FloodModels", "WaveSolver2D",
           "ricker_wavelet"]

_STORAGE = {"auto": 0, "all": 1, "checkpoint": 2}
# below this many grid points one shot's step launch leaves most of the GPU idle
_BATCH_POINTS = 1 << 21


@dataclass
class RTMResult:
    raw_image: np.ndarray
    laplacian_image: np.ndarray
    normalized_image: np.ndarray
    grid_x: np.ndarray
    grid_z: np.ndarray
    dx: float
    dz: float


def apply_laplacian_filter(image: np.ndarray, dx: float, dz: float) -> np.ndarray:
    """3x3 Laplacian, 'same' output size, symmetric boundary (rtm_engine.py:27-38)."""
    from scipy import signal
    ix2, iz2 = 1.0 / (dx * dx), 1.0 / (dz * dz)
    kernel = np.array([[0.0, iz2, 0.0], [ix2, -2.0 * ix2 - 2.0 * iz2, ix2], [0.0, iz2, 0.0]],
                      dtype=np.float32)
    return signal.convolve2d(image, kernel, mode="same", boundary="symm")


class TSWRTMEngine:
    """Transmitted surface-wave reverse-time migration on one GB300."""

    def __init__(self, solver: WaveSolver2D, storage: str = "auto", batch: str = "auto"):
        if storage not in _STORAGE:
            raise ValueError(f"storage must be one of {sorted(_STORAGE)}")
        if batch not in ("auto", "on", "off"):
            raise ValueError("batch must be 'auto', 'on' or 'off'")
        self.solver = solver
        self.storage = storage
        self.batch = batch
        self._batch_engine = None
        self._batch_arena = 0

    def close(self):
        if self._batch_engine is not None:
            self._batch_engine.close()
            self._batch_engine = None
            self._batch_arena = 0

    def _prepare(self, flood_models, receiver_data, receiver_ix, receiver_iz, source_ts,
                 source_ix, source_iz):
        s = self.solver
        s._set_velocity(0, flood_models.sediment_flood)
        s._set_velocity(1, flood_models.rock_flood)
        return self._check(receiver_data, receiver_ix, receiver_iz, source_ts, source_ix,
                           source_iz)

    def _check(self, receiver_data, receiver_ix, receiver_iz, source_ts, source_ix, source_iz):
        s = self.solver
        w = np.ascontiguousarray(source_ts, dtype=np.float32).reshape(-1)
        data = np.ascontiguousarray(receiver_data, dtype=np.float32)
        if data.ndim != 2:
            raise ValueError("receiver_data must be (nt, n_receivers)")
        rix = normalize_indices(receiver_ix, s.nx, "receiver_ix")
        if len(rix) < data.shape[1]:
            raise IndexError("fewer receiver indices than data columns")
        rix = rix[: data.shape[1]]
        if data.shape[0] != len(w):
            raise ValueError("receiver_data and source_ts have different lengths")
        return (w, data, rix, normalize_index(receiver_iz, s.nz, "receiver_iz"),
                normalize_index(source_ix, s.nx, "source_ix"),
                normalize_index(source_iz, s.nz, "source_iz"))

    def migrate_shot(self, flood_models: FloodModels, source_ts: np.ndarray, source_ix: int,
                     source_iz: int, receiver_data: np.ndarray, receiver_ix: np.ndarray,
                     receiver_iz: int = 2, snapshot_interval: int = 2
                     ) -> Tuple[np.ndarray, np.ndarray]:
        """Migrate one virtual shot; returns (shot_image, illumination), both (nz, nx)."""
        s = self.solver
        w, data, rix, riz, six, siz = self._prepare(flood_models, receiver_data, receiver_ix,
                                                    receiver_iz, source_ts, source_ix, source_iz)
        image = np.empty((s.nz, s.nx), np.float32)
        illum = np.empty((s.nz, s.nx), np.float32)
        _lib.check(s._lib.w2d_migrate_shot(
            s._eng(), w.ctypes.data, len(w), six, siz, data.ctypes.data, rix.ctypes.data,
            data.shape[1], riz, int(snapshot_interval), _STORAGE[self.storage],
            image.ctypes.data, illum.ctypes.data))
        return image, illum

    def migrate_multiple_shots(self, flood_models: FloodModels, source_waveforms: List[np.ndarray],
                               source_coords_ix: List[int], source_coords_iz: List[int],
                               receiver_gathers: List[np.ndarray], receiver_ix: np.ndarray,
                               receiver_iz: int = 2, snapshot_interval: int = 2,
                               mute_sponge: bool = True) -> RTMResult:
        """Migrate and stack every shot, then mute, normalise and filter the stack."""
        s = self.solver
        eng = s._eng()
        _lib.check(s._lib.w2d_stack_reset(eng))
        if not (self._use_batch(len(source_coords_ix)) and self._migrate_batched(
                eng, flood_models, source_waveforms, source_coords_ix, source_coords_iz,
                receiver_gathers, receiver_ix, receiver_iz, snapshot_interval)):
            self._migrate_serial(eng, flood_models, source_waveforms, source_coords_ix,
                                 source_coords_iz, receiver_gathers, receiver_ix, receiver_iz,
                                 snapshot_interval)
        # mute, normalisation and Laplacian run on the device stack
        raw, lap, norm = (np.empty((s.nz, s.nx), np.float32) for _ in range(3))
        _lib.check(s._lib.w2d_post_stack(eng, 1 if mute_sponge else 0, raw.ctypes.data,
                                         lap.ctypes.data, norm.ctypes.data))
        return RTMResult(raw_image=raw, laplacian_image=lap, normalized_image=norm,
                         grid_x=np.arange(s.nx) * s.dx, grid_z=np.arange(s.nz) * s.dz,
                         dx=s.dx, dz=s.dz)

    def _use_batch(self, n_shots: int) -> bool:
        if self.batch == "off" or n_shots < 2:
            return False
        s = self.solver
        if s.sponge is not None and not np.array_equal(s.sponge, s._default_sponge()):
            return False  # a caller-modified sponge: the batch engine builds the Cerjan one
        if self.batch == "on":
            return True
        return self.storage == "auto" and s.nx * s.nz <= _BATCH_POINTS

    def _migrate_batched(self, eng, flood_models, source_waveforms, source_coords_ix,
                         source_coords_iz, receiver_gathers, receiver_ix, receiver_iz,
                         snapshot_interval) -> bool:
        """All shots as one batch; False (nothing done) when one shot does not fit."""
        from .batch import BatchEngine, ShotJob, new_model_key
        s = self.solver
        n_sp = s.n_sponge if s.sponge is not None else -1
        key = new_model_key()  # every shot migrates in the same flood models
        v_sed, v_rock = _host(flood_models.sediment_flood), _host(flood_models.rock_flood)
        jobs = []
        for k in range(len(source_coords_ix)):
            w, data, rix, riz, six, siz = self._check(receiver_gathers[k], receiver_ix,
                                                      receiver_iz, source_waveforms[k],
                                                      source_coords_ix[k], source_coords_iz[k])
            jobs.append(ShotJob(s.nx, s.nz, s.dx, s.dz, s.dt, v_sed, v_rock, w, data, rix, six,
                                siz, riz,
                                int(snapshot_interval), n_sp, s.sponge_alpha,
                                bool(s.free_surface_top), model_key=key))
        per = max(BatchEngine.shot_bytes(j) for j in jobs)
        free, _ = _lib.device_memory()
        arena = min(per * len(jobs), int(0.5 * free) + self._batch_arena)
        if arena < per:
            return False
        if self._batch_engine is None or self._batch_arena < arena:
            self.close()
            self._batch_engine = BatchEngine(arena_bytes=arena, max_shots=len(jobs), tile=(4, 4))
            self._batch_arena = arena
        results, _ = self._batch_engine.run(jobs)
        for img, ill in results:  # shot order, as the serial stack
            _lib.check(s._lib.w2d_stack_add(eng, img.ctypes.data, ill.ctypes.data))
        return True

    def _migrate_serial(self, eng, flood_models, source_waveforms, source_coords_ix,
                        source_coords_iz, receiver_gathers, receiver_ix, receiver_iz,
                        snapshot_interval):
        s = self.solver
        for k in range(len(source_coords_ix)):
            w, data, rix, riz, six, siz = self._prepare(
                flood_models, receiver_gathers[k], receiver_ix, receiver_iz, source_waveforms[k],
                source_coords_ix[k], source_coords_iz[k])
            _lib.check(s._lib.w2d_migrate_shot(
                eng, w.ctypes.data, len(w), six, siz, data.ctypes.data, rix.ctypes.data,
                data.shape[1], riz, int(snapshot_interval), _STORAGE[self.storage], None, None))


def _host(a):
    """A model as a host array (a device-resident CUDA tensor is copied back)."""
    if type(a).__module__.startswith("torch") and getattr(a, "is_cuda", False):
        return a.detach().float().contiguous().cpu().numpy()
    return a


def post_stack(solver: WaveSolver2D, stacked: np.ndarray, illum: np.ndarray,
               mute_sponge: bool = True) -> RTMResult:
    """Sponge mute (< 0.99), illumination normalisation, Laplacian (rtm_engine.py:145-171)."""
    if mute_sponge:
        mask = solver.sponge < 0.99
        stacked[mask] = 0.0
        illum[mask] = 0.0
    mx = np.max(illum)
    eps = 1e-4 * mx if mx > 0 else 1e-12
    normalized = stacked / (np.sqrt(illum) + eps)
    lap = apply_laplacian_filter(stacked, solver.dx, solver.dz)
    if mute_sponge:
        lap[mask] = 0.0
    return RTMResult(raw_image=stacked, laplacian_image=lap, normalized_image=normalized,
                     grid_x=np.arange(solver.nx) * solver.dx, grid_z=np.arange(solver.nz) * solver.dz,
                     dx=solver.dx, dz=solver.dz)
