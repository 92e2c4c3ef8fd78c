"""Elastic (velocity-stress) modelling and its gradient on one GB300.

The reference ships the elastic step (tsw_rtm/c_engine/wave2d.c:95-212) but no
elastic time loop.  ``ElasticSolver2D`` runs that step (same arithmetic, same
staggered grid, free surface and sponge) with a vertical force source and
vertical-strain receivers -- the quantity a DAS fibre records -- and
``ElasticModeling`` puts the hand-written adjoint behind torch.autograd, so the
gradient of any loss on the traces with respect to lambda, mu and the
buoyancies (and, through ``gardner_parameters``, with respect to the shear
velocity) is available, the forward states being recomputed from checkpoints.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .geometry import normalize_index, normalize_indices


class ElasticSolver2D:
    def __init__(self, nx: int, nz: int, dx: float, dz: float, dt: float, n_sponge: int = 30,
                 sponge_alpha: float = 0.0015, free_surface_top: bool = True):
        self.nx, self.nz = nx, nz
        self.dx, self.dz, self.dt = float(dx), float(dz), float(dt)
        self.n_sponge, self.sponge_alpha = n_sponge, float(sponge_alpha)
        self.free_surface_top = free_surface_top
        self._lib = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(self._lib.w2d_elastic_create(ctypes.byref(h), nx, nz, self.dx, self.dz, self.dt,
                                                n_sponge, self.sponge_alpha,
                                                1 if free_surface_top else 0))
        self._h = h
        # a batch whose shots have identical models stores and reads one copy
        self.share_models = True

    def close(self):
        if getattr(self, "_h", None) is not None:
            self._lib.w2d_elastic_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def last_ms(self) -> float:
        return float(self._lib.w2d_elastic_last_ms(self._h))

    def set_tiles(self, step=(4, 2), adjoint=(4, 1)):
        """Tile shapes (warps, rows per warp) of the step kernels and the tiled adjoint
        passes; applies from the next forward call; results do not depend on them."""
        _lib.check(self._lib.w2d_elastic_set_tiles(self._h, int(step[0]), int(step[1]),
                                                   int(adjoint[0]), int(adjoint[1])))

    def set_pdl(self, on: bool = True):
        """Programmatic dependent launches between consecutive step and tiled-adjoint
        kernels (on by default); results are identical either way."""
        _lib.check(self._lib.w2d_elastic_set_pdl(self._h, 1 if on else 0))

    def set_adjoint(self, form: str = "tiled"):
        """How the adjoint passes run: "tiled" (TMA-tiled passes, the default) or
        "cells" (one thread per cell); both are exact adjoints of the step and agree
        to float32 rounding."""
        if form not in ("tiled", "cells"):
            raise ValueError("form must be 'tiled' or 'cells'")
        _lib.check(self._lib.w2d_elastic_set_adjoint(self._h, 1 if form == "tiled" else 0))


def gardner_parameters(vs: torch.Tensor, vp_over_vs: float = 1.73):
    """(lambda, mu, buo_x, buo_z) from the shear velocity: vp = 1.73 vs, Gardner's
    density rho = 310 vp^0.25 (kg/m^3, vp in m/s); differentiable in torch."""
    vp = vp_over_vs * vs
    rho = 310.0 * vp ** 0.25
    mu = rho * vs * vs
    lam = rho * vp * vp - 2.0 * mu
    b = 1.0 / rho
    return lam, mu, b, b


class ElasticModeling(torch.autograd.Function):
    """Traces of one shot (parameters (nz, nx), wavelet (nt,), scalar source) or of a
    batch of shots (parameters (S, nz, nx), wavelets (S, nt) or (nt,), source indices
    of length S), all shots advanced together; the backward pass returns one gradient
    per shot."""

    @staticmethod
    def forward(ctx, lam, mu, bx, bz, solver: ElasticSolver2D, wavelet, source_ix, source_iz,
                receiver_ix, receiver_iz):
        ps = [t.detach().to(torch.float32).contiguous() for t in (lam, mu, bx, bz)]
        batched = ps[0].dim() == 3
        S = ps[0].shape[0] if batched else 1
        for t in ps:
            if not t.is_cuda or tuple(t.shape[-2:]) != (solver.nz, solver.nx) or \
                    t.dim() != ps[0].dim() or (batched and t.shape[0] != S):
                raise ValueError("parameters must be CUDA tensors of shape (nz, nx) or "
                                 "(S, nz, nx)")
        w = np.ascontiguousarray(wavelet, dtype=np.float32)
        if w.ndim == 1:
            w = np.ascontiguousarray(np.broadcast_to(w, (S, w.shape[0])))
        if w.shape[0] != S:
            raise ValueError("one wavelet per shot")
        nt = w.shape[1]
        six = np.asarray([normalize_index(int(x), solver.nx, "source_ix")
                          for x in np.broadcast_to(np.asarray(source_ix), (S,))], dtype=np.int32)
        siz = np.asarray([normalize_index(int(x), solver.nz, "source_iz")
                          for x in np.broadcast_to(np.asarray(source_iz), (S,))], dtype=np.int32)
        rix = normalize_indices(receiver_ix, solver.nx, "receiver_ix")
        riz = normalize_index(receiver_iz, solver.nz, "receiver_iz")
        traces = torch.empty((S, nt, len(rix)), dtype=torch.float32, device=ps[0].device)
        # shots of one model (a job's shots, as in a survey): store and read it once
        shared = batched and S > 1 and solver.share_models and all(
            bool(torch.equal(t, t[:1].expand_as(t))) for t in ps)
        _lib.check(solver._lib.w2d_elastic_share_model(solver._h, 1 if shared else 0))
        torch.cuda.current_stream(ps[0].device).synchronize()
        _lib.check(solver._lib.w2d_elastic_forward_batch(
            solver._h, S, *[t.data_ptr() for t in ps], w.ctypes.data, nt, six.ctypes.data,
            siz.ctypes.data, rix.ctypes.data, len(rix), riz, traces.data_ptr()))
        ctx.solver = solver
        ctx.shape = tuple(ps[0].shape)
        ctx.device = ps[0].device
        return traces if batched else traces[0]

    @staticmethod
    def backward(ctx, grad_traces):
        g = grad_traces.detach().to(torch.float32).contiguous()
        outs = [torch.empty(ctx.shape, dtype=torch.float32, device=ctx.device) for _ in range(4)]
        torch.cuda.current_stream(ctx.device).synchronize()
        _lib.check(ctx.solver._lib.w2d_elastic_gradient_batch(ctx.solver._h, g.data_ptr(),
                                                              *[o.data_ptr() for o in outs]))
        return (*outs, None, None, None, None, None, None)


def elastic_traces(vs: torch.Tensor, solver: ElasticSolver2D, wavelet, source_ix, source_iz,
                   receiver_ix, receiver_iz=2):
    """Vertical-strain traces for a shear-velocity model; differentiable in vs.

    vs (nz, nx) with one source: traces (nt, n_rec).  vs (S, nz, nx) (one model per
    shot, possibly equal) with S sources and wavelets: traces (S, nt, n_rec), all shots
    advanced together."""
    return ElasticModeling.apply(*gardner_parameters(vs), solver, wavelet, source_ix, source_iz,
                                 receiver_ix, receiver_iz)


class ElasticExecutor:
    """Runs elastic migration jobs on worker threads, each with its own CUDA stream, so
    they overlap each other and the acoustic batch on the device.  A job's shots carry
    the shear velocity in ``vel_fwd`` and observed vertical-strain traces in ``data``;
    each shot's result is (dJ/dvs, None) for J = 0.5 * ||d(vs) - data||^2.  A job's
    shots run as batches (all shots of a batch advanced by the same launches), as many
    per batch as ``budget_gb`` of device memory holds; batches spread over the workers.
    A worker keeps the solver of the grid it ran last and drops it when the grid
    changes."""

    def __init__(self, workers: int = 3, budget_gb: float = 20.0):
        import queue
        import threading
        self._q = queue.Queue()
        self._done = []
        self._lock = threading.Lock()
        self._pending = 0
        self._jobs = {}  # job_id -> [request, results, shots left]
        self._solvers = {}
        self.busy_s = 0.0  # summed wall time of the workers' batches
        self.budget = int(budget_gb * (1 << 30))  # device bytes per worker for one batch
        # the creating thread's device: the CUDA device is per host thread and a new
        # thread starts on device 0, so each worker selects this one before any CUDA call
        self._device = torch.cuda.current_device() if torch.cuda.is_available() else None
        self._threads = [threading.Thread(target=self._loop, daemon=True)
                         for _ in range(max(1, int(workers)))]
        for t in self._threads:
            t.start()

    @staticmethod
    def _key(s):
        return (s.nx, s.nz, s.dx, s.dz, s.dt, s.n_sponge, s.sponge_alpha, s.free_surface_top)

    def _solver(self, s):
        """A solver for shot s kept by the calling thread's caller (used outside the workers)."""
        key = self._key(s)
        if key not in self._solvers:
            self._solvers[key] = ElasticSolver2D(s.nx, s.nz, s.dx, s.dz, s.dt, s.n_sponge,
                                                 s.sponge_alpha, s.free_surface_top)
        return self._solvers[key]

    @staticmethod
    def migrate_shot(solver, shot):
        return ElasticExecutor.migrate_shots(solver, [shot])[0]

    @staticmethod
    def migrate_shots(solver, shots):
        """Shots on one grid as one batch: per shot (dJ/dvs, None) for
        J = 0.5 * ||d(vs) - data||^2."""
        vs = torch.tensor(np.stack([np.asarray(s.vel_fwd, np.float32) for s in shots]),
                          device="cuda", requires_grad=True)
        d = elastic_traces(vs, solver, np.stack([np.asarray(s.wavelet, np.float32)
                                                 for s in shots]),
                           [s.source_ix for s in shots], [s.source_iz for s in shots],
                           shots[0].receiver_ix, shots[0].receiver_iz)
        obs = torch.tensor(np.stack([np.asarray(s.data, np.float32) for s in shots]),
                           device="cuda")
        J = 0.5 * torch.sum((d - obs) ** 2)
        J.backward()
        g = vs.grad.detach().cpu().numpy()
        return [(g[k], None) for k in range(len(shots))]

    def _batches(self, shots):
        """Consecutive runs of shots that share a grid, receivers and length, each at
        most as large as the per-worker memory budget allows."""
        out, cur = [], []
        for s in shots:
            same = cur and self._key(s) == self._key(cur[0]) and \
                len(s.wavelet) == len(cur[0].wavelet) and \
                np.array_equal(np.asarray(s.receiver_ix), np.asarray(cur[0].receiver_ix)) and \
                s.receiver_iz == cur[0].receiver_iz
            if cur and (not same or len(cur) >= self._cap(cur[0])):
                out.append(cur)
                cur = []
            cur.append(s)
        if cur:
            out.append(cur)
        return out

    def _cap(self, shot):
        per = int(_lib.load().w2d_elastic_shot_bytes(shot.nx, shot.nz, len(shot.wavelet),
                                                     len(np.asarray(shot.receiver_ix))))
        return max(1, min(64, self.budget // max(per, 1)))

    def _loop(self):
        import time
        if self._device is not None:
            torch.cuda.set_device(self._device)
            _lib.check(_lib.load().w2d_set_device(self._device))
        torch.cuda.set_stream(torch.cuda.Stream())
        key, solver = None, None
        while True:
            item = self._q.get()
            if item is None:
                if solver is not None:
                    solver.close()
                return
            jid, ks = item
            with self._lock:
                req = self._jobs[jid][0]
            shots = [req.shots[k] for k in ks]
            if self._key(shots[0]) != key:
                if solver is not None:
                    solver.close()
                key = self._key(shots[0])
                s0 = shots[0]
                solver = ElasticSolver2D(s0.nx, s0.nz, s0.dx, s0.dz, s0.dt, s0.n_sponge,
                                         s0.sponge_alpha, s0.free_surface_top)
            tb = time.perf_counter()
            res = self.migrate_shots(solver, shots)
            with self._lock:
                self.busy_s += time.perf_counter() - tb
                entry = self._jobs[jid]
                for k, r in zip(ks, res):
                    entry[1][k] = r
                entry[2] -= len(ks)
                if entry[2] == 0:
                    self._done.append((jid, entry[1], time.perf_counter()))
                    del self._jobs[jid]
                    self._pending -= 1

    def submit(self, req):
        with self._lock:
            self._pending += 1
            self._jobs[req.job_id] = [req, [None] * len(req.shots), len(req.shots)]
        k0 = 0
        for batch in self._batches(req.shots):
            self._q.put((req.job_id, list(range(k0, k0 + len(batch)))))
            k0 += len(batch)

    def pending(self) -> int:
        with self._lock:
            return self._pending

    def poll(self):
        with self._lock:
            out, self._done = self._done, []
        return out

    def close(self):
        for _ in self._threads:
            self._q.put(None)
        for t in self._threads:
            t.join()
        for sv in self._solvers.values():
            sv.close()
        self._solvers = {}
