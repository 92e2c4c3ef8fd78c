"""Host logic of the continuous-batching server, on a stand-in engine (no GPU).

``RTMServer.serve`` decides what runs when: admission in arrival order by memory and
slots, replays while shots are in flight, results collected as shots finish, latency
per job, throughput and load statistics.  The stand-in engine advances each admitted
shot by a fixed number of phase steps per replay and charges a fixed device time, so
the schedule is exact and checkable; it returns each shot's own marker as its image,
so a result that went to the wrong job shows.
"""
import numpy as np
import pytest

from das_gb300.batch import ShotJob
from das_gb300.serving import RTMRequest, RTMServer, percentile

STEPS_PER_REPLAY = 50
MS_PER_REPLAY = 2.0


def _shot(nz, nx, nt, tag):
    v = np.full((nz, nx), 2000.0, np.float32)
    w = np.zeros(nt, np.float32)
    rix = np.arange(nx)
    return ShotJob(nx, nz, 5.0, 5.0, 5e-4, v, v, w, np.zeros((nt, nx), np.float32), rix,
                   nx // 2, 2, 2, 2, 10, 0.0015, True, tag=tag)


class FakeEngine:
    """Arena of `capacity` units (a shot costs nz * nx * nt), at most `slots` shots."""

    def __init__(self, capacity, slots):
        self.capacity, self.slots = capacity, slots
        self.used = 0
        self.running = {}  # slot -> [shot, phase steps done]
        self.next_slot = 0
        self.last_ms = 0.0
        self.last_points = 0.0
        self.max_used = 0
        self.admitted = []  # tags in admission order
        self.launches = 0

    @staticmethod
    def cost(sh):
        return sh.nz * sh.nx * len(sh.wavelet)

    def submit(self, sh):
        if self.cost(sh) > self.capacity:
            return None
        if len(self.running) >= self.slots or self.used + self.cost(sh) > self.capacity:
            return None
        slot = self.next_slot
        self.next_slot += 1
        self.running[slot] = [sh, 0]
        self.used += self.cost(sh)
        self.max_used = max(self.max_used, self.used)
        self.admitted.append(sh.tag)
        return slot

    def launch(self):
        self.launches += 1
        pts = 0.0
        for entry in self.running.values():
            sh, k = entry
            k_end = 2 * len(sh.wavelet)
            adv = min(STEPS_PER_REPLAY, k_end - k)
            entry[1] = k + adv
            pts += adv * sh.nz * sh.nx
        self.last_ms, self.last_points = MS_PER_REPLAY, pts

    def wait(self):
        pass

    def finished(self, slot):
        sh, k = self.running[slot]
        return k >= 2 * len(sh.wavelet)

    def fetch(self, slot, nz, nx):
        sh, _ = self.running.pop(slot)
        self.used -= self.cost(sh)
        assert (nz, nx) == (sh.nz, sh.nx)
        marker = np.full((nz, nx), float(sh.tag), np.float32)
        return marker, marker


class FakeElastic:
    """Finishes every submitted job at the next poll, with each shot's tag as its result."""

    def __init__(self):
        self.jobs = []
        self.submitted = []

    def submit(self, req):
        self.jobs.append(req)
        self.submitted.append(req.job_id)

    def pending(self):
        return len(self.jobs)

    def poll(self):
        out = [(r.job_id, [(float(s.tag), None) for s in r.shots], 0.0) for r in self.jobs]
        self.jobs = []
        return out


def _trace():
    # three jobs at t = 0, a burst at 0.010 s, a late one at 0.200 s (device clock)
    return [RTMRequest(0, [_shot(40, 80, 100, 1), _shot(40, 80, 100, 2)], 0.0),
            RTMRequest(1, [_shot(60, 60, 200, 3)], 0.0),
            RTMRequest(2, [_shot(30, 90, 60, 4)], 0.0),
            RTMRequest(3, [_shot(50, 50, 150, 5), _shot(50, 50, 150, 6),
                           _shot(50, 50, 150, 7)], 0.010),
            RTMRequest(4, [_shot(20, 40, 40, 8)], 0.200)]


def test_every_result_reaches_its_job_and_admission_is_fifo():
    trace = _trace()
    eng = FakeEngine(capacity=1_000_000, slots=3)
    out, st = RTMServer(eng).serve(trace, realtime=False)
    assert [r.job_id for r in out] == [0, 1, 2, 3, 4]
    for req, resp in zip(trace, out):
        assert len(resp.results) == len(req.shots)
        for sh, (img, ill) in zip(req.shots, resp.results):
            assert img.shape == (sh.nz, sh.nx) and np.all(img == sh.tag)
        assert resp.finished >= resp.arrival
    # arrival order, whatever the sizes
    assert eng.admitted == [1, 2, 3, 4, 5, 6, 7, 8]
    assert eng.max_used <= eng.capacity
    assert st["max_active_shots"] <= 3
    assert st["shots"] == 8 and st["jobs"] == 5


def test_memory_budget_limits_what_runs_together():
    trace = _trace()
    big = max(FakeEngine.cost(s) for r in trace for s in r.shots)
    eng = FakeEngine(capacity=big + 1, slots=8)  # room for one large shot at a time
    out, st = RTMServer(eng).serve(trace, realtime=False)
    assert eng.max_used <= big + 1
    assert all(len(r.results) == len(q.shots) for r, q in zip(out, trace))
    # with one shot at a time the replays run every shot's steps in turn: the makespan
    # is at least the sum over shots of their replays
    replays = sum(-(-2 * len(s.wavelet) // STEPS_PER_REPLAY) for r in trace for s in r.shots)
    assert st["makespan_s"] >= replays * MS_PER_REPLAY / 1e3 - 1e-9


def test_statistics_are_consistent():
    trace = _trace()
    eng = FakeEngine(capacity=1_000_000, slots=4)
    out, st = RTMServer(eng).serve(trace, realtime=False)
    lat = [r.finished - r.arrival for r in out]
    assert st["p50_latency_s"] == pytest.approx(percentile(lat, 50))
    assert st["p99_latency_s"] == pytest.approx(percentile(lat, 99))
    assert st["shots_per_s"] == pytest.approx(8 / st["makespan_s"])
    total = sum(s.counted_points for r in trace for s in r.shots)
    span = trace[-1].arrival - trace[0].arrival
    assert st["offered_gpts_per_s"] == pytest.approx(total / span / 1e9)
    assert st["achieved_gpts_per_s"] == pytest.approx(total / st["makespan_s"] / 1e9)
    # every counted point went through a replay of the stand-in engine
    assert st["gpts_per_s"] == pytest.approx(total / st["makespan_s"] / 1e9)
    # the device clock is the replays' time: busy all along except while idle before
    # the late job arrives
    assert 0.0 < st["device_busy_frac"] <= 1.0


def test_elastic_jobs_go_to_the_executor():
    trace = _trace()
    el = RTMRequest(5, [_shot(30, 30, 50, 9), _shot(30, 30, 50, 10)], 0.005, kind="elastic")
    trace.insert(3, el)
    eng = FakeEngine(capacity=1_000_000, slots=4)
    ex = FakeElastic()
    out, st = RTMServer(eng, elastic_executor=ex).serve(trace, realtime=False)
    assert ex.submitted == [5]
    assert 9 not in eng.admitted and 10 not in eng.admitted
    resp = {r.job_id: r for r in out}[5]
    assert [r[0] for r in resp.results] == [9.0, 10.0]
    assert st["elastic"]["jobs"] == 1 and st["acoustic"]["jobs"] == 5


def test_a_shot_larger_than_the_arena_is_refused():
    trace = [RTMRequest(0, [_shot(40, 80, 100, 1)], 0.0)]
    eng = FakeEngine(capacity=10, slots=2)
    with pytest.raises(MemoryError):
        RTMServer(eng).serve(trace, realtime=False)


def test_elastic_batches_split_by_grid_length_receivers_and_budget(monkeypatch):
    """ElasticExecutor groups consecutive shots that share grid, length and receivers,
    each group no larger than the per-worker budget allows (here three shots)."""
    from das_gb300.elastic import ElasticExecutor
    ex = object.__new__(ElasticExecutor)  # the grouping only: no worker threads
    monkeypatch.setattr(ElasticExecutor, "_cap", lambda self, shot: 3)
    a = [_shot(40, 80, 100, t) for t in range(5)]        # same grid and length
    b = [_shot(40, 80, 120, t) for t in range(5, 7)]     # another length
    c = [_shot(50, 80, 120, t) for t in range(7, 8)]     # another grid
    d = _shot(50, 80, 120, 8)
    d.receiver_ix = np.arange(0, 80, 2)                  # other receivers
    groups = ex._batches(a + b + c + [d])
    assert [[s.tag for s in g] for g in groups] == [[0, 1, 2], [3, 4], [5, 6], [7], [8]]
