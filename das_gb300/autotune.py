"""Autotuner for the launch configuration of the RTM kernels.

* ``tune_batch``: form of the batched engine (one launch per phase step, or the
  persistent queue kernel), tile shape, phase steps per launch and launches per
  replay, chosen by timing the batched engine on a sample of the workload's own
  shots (truncated in time).
* ``tune_plain``: tile shape of the per-shot step kernel for one grid, chosen by
  timing a short forward run.

Results are cached in a JSON file (``$DAS_GB300_TUNE_CACHE`` or
``~/.cache/das_gb300/tune.json``) keyed by a size signature, so a
configuration is measured once per machine and workload class.
"""
from __future__ import annotations

import json
import os
import time
from dataclasses import replace
from typing import List, Sequence, Tuple

import numpy as np


# (form, tile, steps per launch, launches per replay); in the grid form the last two
# only set how many phase steps a replay covers
BATCH_CANDIDATES = [("grid", (4, 4), 16, 16), ("grid", (8, 4), 16, 16), ("grid", (4, 8), 16, 16),
                    ("queue", (4, 4), 16, 16), ("queue", (4, 4), 32, 8), ("queue", (8, 4), 16, 16),
                    ("queue", (4, 4), 8, 32), ("queue", (8, 4), 32, 8), ("queue", (4, 8), 16, 16)]
PLAIN_TILES = [(4, 4), (8, 4), (4, 8), (8, 8)]


def _cache_path() -> str:
    return os.environ.get("DAS_GB300_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "das_gb300", "tune.json"))


def _load_cache() -> dict:
    try:
        with open(_cache_path()) as f:
            return json.load(f)
    except Exception:
        return {}


def _store_cache(key: str, value) -> None:
    d = _load_cache()
    d[key] = value
    try:
        os.makedirs(os.path.dirname(_cache_path()), exist_ok=True)
        with open(_cache_path(), "w") as f:
            json.dump(d, f, indent=1)
    except OSError:
        pass


def _truncate(job, nt):
    nt = max(8, min(nt, len(job.wavelet)))
    return replace(job, wavelet=job.wavelet[:nt], data=job.data[:nt], _keep=[])


def tune_batch(jobs: Sequence, candidates=None, sample_shots: int = 24, nt_sample: int = 256,
               arena_bytes: int = 0, use_cache: bool = True) -> Tuple[tuple, List[dict]]:
    """Best (tile, steps_per_launch, launches_per_graph, form) for this set of shots."""
    from .batch import BatchEngine
    pts = np.mean([j.nx * j.nz for j in jobs])
    key = f"batch2:{int(np.log2(max(pts, 1)))}:{len(jobs) >= 64}"
    cache = _load_cache() if use_cache else {}
    if key in cache:
        c = cache[key]["best"]
        return (tuple(c[0]), c[1], c[2], c[3]), cache[key]["table"]
    rng = np.random.default_rng(0)
    idx = rng.choice(len(jobs), size=min(sample_shots, len(jobs)), replace=False)
    sample = [_truncate(jobs[i], nt_sample) for i in idx]
    table = []
    for form, tile, spl, lpg in (candidates or BATCH_CANDIDATES):
        eng = BatchEngine(arena_bytes=arena_bytes, max_shots=len(sample) + 1, tile=tile,
                          steps_per_launch=spl, launches_per_graph=lpg, form=form)
        eng.run(sample[:2])  # graph capture and first touch
        _, st = eng.run(sample)
        eng.close()
        g = st["counted_points"] / max(st["device_ms"], 1e-6) / 1e6
        table.append({"form": form, "tile": list(tile), "steps_per_launch": spl,
                      "launches_per_graph": lpg, "device_gpts_per_s": g})
    best = max(table, key=lambda r: r["device_gpts_per_s"])
    cfg = (tuple(best["tile"]), best["steps_per_launch"], best["launches_per_graph"],
           best["form"])
    if use_cache:
        _store_cache(key, {"best": [list(cfg[0]), cfg[1], cfg[2], cfg[3]], "table": table})
    return cfg, table


def tune_plain(solver, vel, nt_sample: int = 200, tiles=None, use_cache: bool = True):
    """Best step-kernel tile shape for this solver's grid; sets it on the solver."""
    key = f"plain:{solver.nx}x{solver.nz}"
    cache = _load_cache() if use_cache else {}
    if key in cache:
        solver.tile = tuple(cache[key]["best"])
        solver.close()
        return solver.tile, cache[key]["table"]
    w = np.zeros(nt_sample, np.float32)
    w[0] = 1.0
    rix = np.arange(0, solver.nx, max(1, solver.nx // 64))
    table = []
    for t in (tiles or PLAIN_TILES):
        solver.tile = t
        solver.close()
        solver.forward_propagate_acoustic(vel, w[:16], solver.nx // 2, 2, rix, 2)
        solver.forward_propagate_acoustic(vel, w, solver.nx // 2, 2, rix, 2)
        ms = solver.last_stats()["device_ms"]
        table.append({"tile": list(t), "device_ms": ms,
                      "gpts_per_s": solver.nx * solver.nz * nt_sample / (ms / 1e3) / 1e9})
    best = min(table, key=lambda r: r["device_ms"])
    solver.tile = tuple(best["tile"])
    solver.close()
    if use_cache:
        _store_cache(key, {"best": best["tile"], "table": table})
    return solver.tile, table
