"""RTM serving: continuous batching of migration jobs on one GB300.

A job is a list of shots (each a ``ShotJob``: grid, models, wavelet, data,
receivers) that arrives at some time.  The server keeps every admitted shot's
wavefields, snapshot store and inputs resident in the batched engine's device
arena; shots are admitted in arrival order whenever the arena (the HBM budget)
and a slot have room, so requests that arrive while others are running join
them on the device between two replays of the captured time loop; finished
shots leave at once, freeing memory for the next ones.  A job completes when its
last shot does; its latency is completion time minus arrival time.

Each shot's image and illumination are bit-identical to migrating it alone: the
persistent kernel applies the same fused step to each tile whatever else is in
the batch.  Elastic jobs go to ``elastic_executor`` (a callable taking a job
and returning its per-shot results) between replays when one is given.
"""
from __future__ import annotations

import collections
import time
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional, Sequence

import numpy as np

from .batch import BatchEngine, ShotJob, new_model_key


@dataclass
class RTMRequest:
    job_id: int
    shots: List[ShotJob]
    arrival: float          # seconds from the start of the trace
    kind: str = "acoustic"  # "acoustic" or "elastic"


@dataclass
class RTMResponse:
    job_id: int
    kind: str
    arrival: float
    finished: float
    results: List[tuple] = field(default_factory=list)

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


def percentile(xs: Sequence[float], q: float) -> float:
    return float(np.percentile(np.asarray(xs, dtype=np.float64), q)) if len(xs) else float("nan")


def share_models(shots) -> None:
    """Give the shots of one request that hold the same model arrays (the same objects)
    one model key, so the batch engine keeps a single device copy of those models while
    any of the shots is admitted.  Shots that already carry a key keep it."""
    groups = {}
    for sh in shots:
        if getattr(sh, "model_key", 0):
            continue
        ident = (id(getattr(sh, "vel_fwd", None)), id(getattr(sh, "vel_bwd", None)),
                 id(getattr(sh, "vel", None)))
        if ident not in groups:
            groups[ident] = new_model_key()
        sh.model_key = groups[ident]


class RTMServer:
    def __init__(self, engine: BatchEngine, elastic_executor: Optional[Callable] = None):
        self.engine = engine
        self.elastic_executor = elastic_executor

    def serve(self, trace: Sequence[RTMRequest], realtime: bool = True):
        """Run a trace of requests to completion; returns (responses, statistics).

        realtime: arrivals follow the wall clock (requests arriving while the GPU
        works wait in the queue).  Otherwise the clock is the device time of the
        replays, which makes a run independent of host speed (used by tests).
        """
        trace = sorted(trace, key=lambda r: r.arrival)
        eng = self.engine
        t_start = time.perf_counter()
        dev_clock = 0.0

        def now():
            return time.perf_counter() - t_start if realtime else dev_clock

        queue = collections.deque()  # (request, shot index)
        running: Dict[int, tuple] = {}
        responses: Dict[int, RTMResponse] = {}
        remaining: Dict[int, int] = {}
        i = 0
        pts = 0.0
        busy_ms = 0.0
        max_active = 0
        n_shots = 0
        def intake():
            nonlocal i
            t = now()
            while i < len(trace) and trace[i].arrival <= t:
                req = trace[i]
                responses[req.job_id] = RTMResponse(req.job_id, req.kind, req.arrival, float("nan"),
                                                    [None] * len(req.shots))
                remaining[req.job_id] = len(req.shots)
                if req.kind == "elastic" and self.elastic_executor is not None:
                    self.elastic_executor.submit(req)
                else:
                    share_models(req.shots)
                    for k in range(len(req.shots)):
                        queue.append((req, k))
                i += 1

        def admit():  # arrival order, by memory and slots
            while queue:
                req, k = queue[0]
                slot = eng.submit(req.shots[k])
                if slot is None:
                    break
                queue.popleft()
                running[slot] = (req, k)

        ex = self.elastic_executor

        def collect_elastic():
            nonlocal n_shots
            if ex is None:
                return
            for job_id, res, t_done in ex.poll():
                responses[job_id].results = list(res)
                responses[job_id].finished = t_done - t_start if realtime else dev_clock
                n_shots += len(res)
                remaining[job_id] = 0

        flying = False  # a replay launched and not yet waited for
        while i < len(trace) or queue or running or (ex is not None and ex.pending()):
            intake()
            admit()
            collect_elastic()
            if not running and not queue and ex is not None and ex.pending() and (
                    i >= len(trace) or trace[i].arrival > now()):
                time.sleep(0.002)  # only elastic work in flight
                continue
            if not running:
                if queue:
                    raise MemoryError(f"job {queue[0][0].job_id}: a shot does not fit the arena")
                if i < len(trace):
                    if realtime:
                        time.sleep(max(0.0, trace[i].arrival - now()))
                    else:
                        dev_clock = max(dev_clock, trace[i].arrival)
                continue
            max_active = max(max_active, len(running))
            if not flying:
                eng.launch()
            if realtime:  # requests arriving during the replay upload while it runs
                intake()
                admit()
            eng.wait()
            busy_ms += eng.last_ms
            pts += eng.last_points
            dev_clock += eng.last_ms / 1e3
            fin = [s for s in running if eng.finished(s)]
            # the next replay (the shots still running and those admitted meanwhile)
            # runs while the finished shots come back
            flying = len(fin) < len(running)
            if flying:
                eng.launch()
            for slot in fin:
                req, k = running.pop(slot)
                sh = req.shots[k]
                responses[req.job_id].results[k] = eng.fetch(slot, sh.nz, sh.nx)
                n_shots += 1
                remaining[req.job_id] -= 1
                if remaining[req.job_id] == 0:
                    responses[req.job_id].finished = now()
        collect_elastic()  # results that completed after the loop's last check
        makespan = now()
        out = [responses[r.job_id] for r in trace]
        lat = [r.latency for r in out]
        span_jobs = trace[-1].arrival - trace[0].arrival if len(trace) > 1 else 0.0
        # counted points (2 nz nx nt per shot) of every request, acoustic and elastic
        total_pts = float(sum(sh.counted_points for r in trace for sh in r.shots))
        stats = {"jobs": len(out), "shots": sum(len(r.shots) for r in trace),
                 "makespan_s": makespan, "p50_latency_s": percentile(lat, 50),
                 "p99_latency_s": percentile(lat, 99),
                 "shots_per_s": sum(len(r.shots) for r in trace) / makespan if makespan else 0.0,
                 # acoustic points advanced by the batch engine's replays
                 "gpts_per_s": pts / makespan / 1e9 if makespan else 0.0,
                 "device_busy_frac": busy_ms / 1e3 / makespan if makespan else 0.0,
                 "offered_jobs_per_s": (len(trace) - 1) / span_jobs if span_jobs > 0 else None,
                 # offered load (all requests' points over the arrival span) against the
                 # load served (the same points over the makespan)
                 "offered_gpts_per_s": total_pts / span_jobs / 1e9 if span_jobs > 0 else None,
                 "achieved_gpts_per_s": total_pts / makespan / 1e9 if makespan else 0.0,
                 "max_active_shots": max_active}
        for kind in sorted({r.kind for r in out}):
            lk = [r.latency for r in out if r.kind == kind]
            stats[kind] = {"jobs": len(lk), "p50_latency_s": percentile(lk, 50),
                           "p99_latency_s": percentile(lk, 99)}
        return out, stats


def poisson_trace(n_jobs: int, rate: float, make_job: Callable[[int, np.random.Generator], tuple],
                  seed: int = 0) -> List[RTMRequest]:
    """Requests with exponential inter-arrival times; make_job(i, rng) -> (kind, shots)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n_jobs):
        t += rng.exponential(1.0 / rate)
        kind, shots = make_job(i, rng)
        out.append(RTMRequest(i, shots, t, kind))
    return out
