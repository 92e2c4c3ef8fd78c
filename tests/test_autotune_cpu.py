"""Host logic of the autotuner (no GPU): the candidate it picks, the sample it times and
the cache round trip, with stand-in engines whose device times are set by the test."""
import numpy as np

from das_gb300 import autotune
from das_gb300.batch import ShotJob


def _job(nz, nx, nt, tag):
    v = np.full((nz, nx), 2000.0, np.float32)
    return ShotJob(nx, nz, 5.0, 5.0, 5e-4, v, v, np.zeros(nt, np.float32),
                   np.zeros((nt, nx), np.float32), np.arange(nx), nx // 2, 2, 2, 2, 10, 0.0015,
                   True, tag=tag)


# device ms per counted point of each candidate; the grid form with 8 x 4 tiles is fastest
SPEED = {("grid", (4, 4)): 2.0, ("grid", (8, 4)): 1.0, ("grid", (4, 8)): 3.0,
         ("queue", (4, 4)): 4.0, ("queue", (8, 4)): 4.0, ("queue", (4, 8)): 4.0}


class StandInBatchEngine:
    made = []

    def __init__(self, arena_bytes, max_shots, tile, steps_per_launch, launches_per_graph, form):
        self.cfg = (form, tuple(tile), steps_per_launch, launches_per_graph)
        StandInBatchEngine.made.append(self)
        self.runs = []

    def run(self, jobs):
        self.runs.append(list(jobs))
        pts = sum(j.counted_points for j in jobs)
        ms = SPEED[self.cfg[:2]] * pts * 1e-9
        return [None] * len(jobs), {"counted_points": pts, "device_ms": ms}

    def close(self):
        pass


def test_tune_batch_picks_the_fastest_and_caches_it(tmp_path, monkeypatch):
    import das_gb300.batch as batch
    monkeypatch.setenv("DAS_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(batch, "BatchEngine", StandInBatchEngine)
    StandInBatchEngine.made = []
    jobs = [_job(100 + 5 * k, 200 + 7 * k, 1000 + 10 * k, k) for k in range(40)]
    cfg, table = autotune.tune_batch(jobs, sample_shots=12, nt_sample=64)
    assert cfg == ((8, 4), 16, 16, "grid")
    assert len(table) == len(autotune.BATCH_CANDIDATES)
    # every candidate timed on the same sample of 12 shots cut to 64 steps, after a
    # two-shot warm-up run
    for eng in StandInBatchEngine.made:
        warm, timed = eng.runs
        assert len(warm) == 2 and len(timed) == 12
        assert all(len(j.wavelet) == 64 and j.data.shape[0] == 64 for j in timed)
    tags = [j.tag for j in StandInBatchEngine.made[0].runs[1]]
    assert len(set(tags)) == 12
    assert all([j.tag for j in e.runs[1]] == tags for e in StandInBatchEngine.made)
    # second call: from the cache, nothing timed
    StandInBatchEngine.made = []
    cfg2, table2 = autotune.tune_batch(jobs, sample_shots=12, nt_sample=64)
    assert cfg2 == cfg and table2 == table and StandInBatchEngine.made == []


class StandInSolver:
    """Per tile shape a device time; records the tile of every forward run."""

    def __init__(self, nx, nz, ms_by_tile):
        self.nx, self.nz, self.tile = nx, nz, None
        self.ms_by_tile = ms_by_tile
        self.runs = []

    def close(self):
        pass

    def forward_propagate_acoustic(self, vel, w, six, siz, rix, riz):
        self.runs.append((self.tile, len(w)))

    def last_stats(self):
        return {"device_ms": self.ms_by_tile[self.tile]}


def test_tune_plain_sets_the_fastest_tile(tmp_path, monkeypatch):
    monkeypatch.setenv("DAS_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    ms = {(4, 4): 5.0, (8, 4): 6.0, (4, 8): 4.0, (8, 8): 7.0}
    s = StandInSolver(400, 150, ms)
    tile, table = autotune.tune_plain(s, np.zeros((150, 400), np.float32), nt_sample=50)
    assert tile == (4, 8) and s.tile == (4, 8)
    assert [r["tile"] for r in table] == [list(t) for t in autotune.PLAIN_TILES]
    # each tile: a 16-step warm-up, then the timed 50-step run
    assert s.runs == [(t, n) for t in autotune.PLAIN_TILES for n in (16, 50)]
    s2 = StandInSolver(400, 150, ms)
    tile2, _ = autotune.tune_plain(s2, np.zeros((150, 400), np.float32), nt_sample=50)
    assert tile2 == (4, 8) and s2.runs == []
