"""Batched, continuously fed RTM on one GB300 (ctypes over the w2d_batch C ABI).

The reference migrates shots one after another (tsw_rtm/rtm_engine.py:125-143).
Here many shots -- each with its own grid size, length, models, wavelet and
receivers -- are admitted into a device memory arena while memory allows and
advanced together: by default one kernel launch per phase step covers every
active shot's tiles (form "grid"), or one persistent kernel per launch walks a
(step, shot, tile) work queue (form "queue"); finished shots leave and new ones
enter between two replays.  Each shot's result is bit-identical to
migrating it alone with ``TSWRTMEngine.migrate_shot``: the arithmetic of every
cell is the same fused step, independent of what else is in the batch.
"""
from __future__ import annotations

import ctypes
import itertools
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from .geometry import normalize_index, normalize_indices


_KEYS = itertools.count(1)


def new_model_key() -> int:
    """A model key no other job of this process has been given."""
    return next(_KEYS)


class _ShotDesc(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("nz", ctypes.c_int), ("dx", ctypes.c_float),
                ("dz", ctypes.c_float), ("dt", ctypes.c_double), ("free_surface", ctypes.c_int),
                ("n_sponge", ctypes.c_int), ("sponge_alpha", ctypes.c_float),
                ("nt", ctypes.c_int), ("snapshot_interval", ctypes.c_int), ("n_rec", ctypes.c_int),
                ("src_ix", ctypes.c_int), ("src_iz", ctypes.c_int), ("rec_iz", ctypes.c_int),
                ("vel_fwd", ctypes.c_void_p), ("vel_bwd", ctypes.c_void_p),
                ("wavelet", ctypes.c_void_p), ("data", ctypes.c_void_p),
                ("rec_ix", ctypes.c_void_p), ("model_key", ctypes.c_longlong)]


@dataclass
class ShotJob:
    """One shot's migration: the arguments of WaveSolver2D + TSWRTMEngine.migrate_shot."""
    nx: int
    nz: int
    dx: float
    dz: float
    dt: float
    vel_fwd: np.ndarray
    vel_bwd: np.ndarray
    wavelet: np.ndarray
    data: np.ndarray
    receiver_ix: np.ndarray
    source_ix: int
    source_iz: int
    receiver_iz: int = 2
    snapshot_interval: int = 2
    n_sponge: int = 30
    sponge_alpha: float = 0.0015
    free_surface_top: bool = True
    tag: object = None
    # nonzero: every job submitted with this key has identical models (the shots of one
    # survey); the engine keeps one device copy of them while any such job is admitted
    model_key: int = 0
    _keep: list = field(default_factory=list, repr=False)

    def desc(self) -> _ShotDesc:
        vf = np.ascontiguousarray(self.vel_fwd, dtype=np.float32)
        vb = np.ascontiguousarray(self.vel_bwd, dtype=np.float32)
        w = np.ascontiguousarray(self.wavelet, dtype=np.float32).reshape(-1)
        data = np.ascontiguousarray(self.data, dtype=np.float32)
        if vf.shape != (self.nz, self.nx) or vb.shape != (self.nz, self.nx):
            raise ValueError("velocity model shape does not match (nz, nx)")
        if data.ndim != 2 or data.shape[0] != len(w):
            raise ValueError("data must be (nt, n_receivers) with nt = len(wavelet)")
        rix = normalize_indices(self.receiver_ix, self.nx, "receiver_ix")[: data.shape[1]]
        if len(rix) < data.shape[1]:
            raise IndexError("fewer receiver indices than data columns")
        self._keep = [vf, vb, w, data, rix]
        return _ShotDesc(self.nx, self.nz, self.dx, self.dz, self.dt,
                         1 if self.free_surface_top else 0, int(self.n_sponge),
                         float(self.sponge_alpha), len(w), int(self.snapshot_interval),
                         data.shape[1], normalize_index(self.source_ix, self.nx, "source_ix"),
                         normalize_index(self.source_iz, self.nz, "source_iz"),
                         normalize_index(self.receiver_iz, self.nz, "receiver_iz"),
                         vf.ctypes.data, vb.ctypes.data, w.ctypes.data,
                         data.ctypes.data if data.size else None, rix.ctypes.data,
                         int(self.model_key))

    @property
    def counted_points(self) -> int:
        return 2 * self.nx * self.nz * len(self.wavelet)


@dataclass
class ModelJob:
    """One shot's forward modelling (WaveSolver2D.forward_propagate_acoustic with
    snapshots off): its result is the (nt, n_receivers) gather of p_next samples."""
    nx: int
    nz: int
    dx: float
    dz: float
    dt: float
    vel: np.ndarray
    wavelet: np.ndarray
    receiver_ix: np.ndarray
    source_ix: int
    source_iz: int
    receiver_iz: int = 2
    n_sponge: int = 30
    sponge_alpha: float = 0.0015
    free_surface_top: bool = True
    tag: object = None
    # nonzero: every job submitted with this key has identical models (the shots of one
    # survey); the engine keeps one device copy of them while any such job is admitted
    model_key: int = 0
    _keep: list = field(default_factory=list, repr=False)

    def desc(self) -> _ShotDesc:
        v = np.ascontiguousarray(self.vel, dtype=np.float32)
        w = np.ascontiguousarray(self.wavelet, dtype=np.float32).reshape(-1)
        if v.shape != (self.nz, self.nx):
            raise ValueError("velocity model shape does not match (nz, nx)")
        rix = normalize_indices(self.receiver_ix, self.nx, "receiver_ix")
        self._keep = [v, w, rix]
        return _ShotDesc(self.nx, self.nz, self.dx, self.dz, self.dt,
                         1 if self.free_surface_top else 0, int(self.n_sponge),
                         float(self.sponge_alpha), len(w), 1, len(rix),
                         normalize_index(self.source_ix, self.nx, "source_ix"),
                         normalize_index(self.source_iz, self.nz, "source_iz"),
                         normalize_index(self.receiver_iz, self.nz, "receiver_iz"),
                         v.ctypes.data, None, w.ctypes.data, None,
                         rix.ctypes.data if len(rix) else None, int(self.model_key))

    @property
    def n_receivers(self) -> int:
        return len(np.asarray(self.receiver_ix).reshape(-1))

    @property
    def counted_points(self) -> int:
        return self.nx * self.nz * len(self.wavelet)


class BatchEngine:
    """Persistent multi-shot RTM engine with admission by device-memory budget."""

    def __init__(self, arena_bytes: int = 0, max_shots: int = 1024, tile=(8, 4),
                 steps_per_launch: int = 16, launches_per_graph: int = 8, form: str = "grid"):
        self._lib = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(self._lib.w2d_batch_create(ctypes.byref(h), int(arena_bytes), int(max_shots)))
        self._h = h
        self.config = None
        self.set_config(tile, steps_per_launch, launches_per_graph)
        self.set_form(form)
        self.last_ms = 0.0
        self.last_points = 0.0

    def set_form(self, form: str) -> None:
        """'grid': one launch per phase step over every active shot (default);
        'queue': persistent kernel over a (step, shot, tile) queue.  Same results."""
        if form not in ("grid", "queue"):
            raise ValueError("form must be 'grid' or 'queue'")
        _lib.check(self._lib.w2d_batch_set_form(self._h, 1 if form == "grid" else 0))
        self.form = form

    def set_config(self, tile, steps_per_launch, launches_per_graph):
        _lib.check(self._lib.w2d_batch_set_config(self._h, int(tile[0]), int(tile[1]),
                                                  int(steps_per_launch), int(launches_per_graph)))
        self.config = (tuple(tile), int(steps_per_launch), int(launches_per_graph))

    def close(self):
        if getattr(self, "_h", None) is not None:
            self._lib.w2d_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def free_bytes(self) -> int:
        return int(self._lib.w2d_batch_free_bytes(self._h))

    @staticmethod
    def shot_bytes(job) -> int:
        """Device bytes a job occupies while admitted (upper bound)."""
        d = job.desc()
        fn = "w2d_batch_model_bytes" if isinstance(job, ModelJob) else "w2d_batch_shot_bytes"
        return int(getattr(_lib.load(), fn)(ctypes.byref(d)))

    def submit(self, job) -> Optional[int]:
        """Admit a ShotJob or ModelJob; None when it does not fit in device memory now."""
        d = job.desc()
        slot = ctypes.c_int(-1)
        fn = (self._lib.w2d_batch_submit_modelling if isinstance(job, ModelJob)
              else self._lib.w2d_batch_submit)
        rc = fn(self._h, ctypes.byref(d), ctypes.byref(slot))
        if rc == 3:  # W2D_ENOMEM: wait for running shots to leave
            return None
        _lib.check(rc)
        return slot.value

    def step(self) -> int:
        """Replay the captured time loop once; returns how many shots finished."""
        self.launch()
        return self.wait()

    def launch(self) -> None:
        """Start one replay; shots submitted meanwhile upload in parallel and join the next."""
        _lib.check(self._lib.w2d_batch_launch(self._h))

    def wait(self) -> int:
        """Finish the replay in flight; returns how many shots finished."""
        n = ctypes.c_int(0)
        _lib.check(self._lib.w2d_batch_wait(self._h, ctypes.byref(n)))
        na, ms, pts, la = ctypes.c_int(), ctypes.c_float(), ctypes.c_double(), ctypes.c_longlong()
        _lib.check(self._lib.w2d_batch_stats(self._h, ctypes.byref(na), ctypes.byref(ms),
                                             ctypes.byref(pts), ctypes.byref(la)))
        self.last_ms, self.last_points, self.last_launches = ms.value, pts.value, la.value
        self.n_active = na.value
        return n.value

    def finished(self, slot: int) -> bool:
        return self._lib.w2d_batch_is_finished(self._h, int(slot)) == 1

    def cancel(self, slot: int) -> None:
        """Drop an admitted job, running or finished, between replays (no replay in
        flight): its device memory returns to the arena, its slot is free again, and the
        other jobs continue with results unchanged."""
        _lib.check(self._lib.w2d_batch_cancel(self._h, int(slot)))

    def fetch(self, slot: int, nz: int, nx: int) -> Tuple[np.ndarray, np.ndarray]:
        img = np.empty((nz, nx), np.float32)
        ill = np.empty((nz, nx), np.float32)
        _lib.check(self._lib.w2d_batch_fetch(self._h, int(slot), img.ctypes.data, ill.ctypes.data))
        return img, ill

    def fetch_traces(self, slot: int, nt: int, n_rec: int) -> np.ndarray:
        tr = np.empty((nt, n_rec), np.float32)
        _lib.check(self._lib.w2d_batch_fetch_traces(self._h, int(slot),
                                                    tr.ctypes.data if tr.size else None))
        return tr

    def collect(self, slot: int, job):
        """Result of a finished job: (image, illumination) or the modelled gather."""
        if isinstance(job, ModelJob):
            return self.fetch_traces(slot, len(job.wavelet), job.n_receivers)
        return self.fetch(slot, job.nz, job.nx)

    def run(self, jobs: Sequence) -> Tuple[list, dict]:
        """Run every job (ShotJob or ModelJob, mixed freely; continuous admission);
        results in job order and statistics."""
        results: List[Optional[Tuple[np.ndarray, np.ndarray]]] = [None] * len(jobs)
        pending = list(range(len(jobs)))
        running: Dict[int, int] = {}
        dev_ms = 0.0
        pts = 0.0
        launches = 0
        max_active = 0

        def admit():
            while pending:
                slot = self.submit(jobs[pending[0]])
                if slot is None:
                    break
                running[slot] = pending.pop(0)

        admit()
        flying = False
        while running or pending:
            if not running:
                admit()
                if not running:
                    raise MemoryError("a shot does not fit in the arena even when it is empty")
            max_active = max(max_active, len(running))
            if not flying:
                self.launch()
            admit()  # uploads overlap the replay in flight; these shots join the next one
            self.wait()
            dev_ms += self.last_ms
            pts += self.last_points
            launches += self.last_launches
            fin = [s for s in running if self.finished(s)]
            # the next replay runs while the finished shots come back
            flying = len(fin) < len(running)
            if flying:
                self.launch()
            for slot in fin:
                j = running.pop(slot)
                results[j] = self.collect(slot, jobs[j])
        return results, {"device_ms": dev_ms, "counted_points": pts, "launches": launches,
                         "max_active": max_active}
