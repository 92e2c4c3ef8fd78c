"""Batched / continuously fed engine: every shot's result equals migrating it alone.

The persistent (step, shot, tile) kernel runs the same fused tile-step as the
per-shot engine, so images and illuminations must be bit-identical to
``TSWRTMEngine.migrate_shot`` whatever else is in the batch, with shots of
different grid sizes, lengths, intervals, sponges and receiver layouts.
"""
import numpy as np
import pytest

from oracle import oracle as o

pytestmark = pytest.mark.gpu


def _job(seed, nz, nx, nt, interval=2, n_sponge=20, fs=True, tag=None):
    from das_gb300.batch import ShotJob
    from das_gb300.wave_solver import ricker_wavelet
    rng = np.random.default_rng(seed)
    dx, dt = 5.0, 5e-4
    v = rng.uniform(1500, 3200, (nz, nx)).astype(np.float32)
    w, _ = ricker_wavelet(rng.uniform(8, 14), dt, nt * dt)
    n_rec = int(rng.integers(nx // 3, nx))
    rix = np.sort(rng.integers(0, nx, size=n_rec))
    data = (rng.standard_normal((len(w), n_rec)) * 1e-7).astype(np.float32)
    return ShotJob(nx, nz, dx, dx, dt, v, v * 1.01, w, data, rix, int(rng.integers(0, nx)),
                   int(rng.integers(2, 5)), int(rng.integers(2, 5)), interval, n_sponge, 0.003, fs,
                   tag=tag)


def _alone(job):
    from das_gb300.rtm_engine import TSWRTMEngine
    from das_gb300.velocity_flood import FloodModels
    from das_gb300.wave_solver import WaveSolver2D
    s = WaveSolver2D(job.nx, job.nz, job.dx, job.dz, job.dt, job.n_sponge, job.sponge_alpha,
                     job.free_surface_top)
    fm = FloodModels(job.vel_fwd, job.vel_fwd, job.vel_bwd, 0, 0)
    return TSWRTMEngine(s, "all").migrate_shot(fm, job.wavelet, job.source_ix, job.source_iz,
                                               job.data, job.receiver_ix, job.receiver_iz,
                                               job.snapshot_interval)


@pytest.mark.parametrize("form", ["grid", "queue"])
@pytest.mark.parametrize("tile,steps", [((8, 4), 16), ((4, 4), 7), ((4, 8), 33)])
def test_batch_equals_single_shot(tile, steps, form):
    from das_gb300.batch import BatchEngine
    jobs = [_job(1, 90, 260, 150), _job(2, 40, 130, 97, interval=3),
            _job(3, 70, 400, 211, interval=1, fs=False), _job(4, 33, 77, 64, n_sponge=8),
            _job(5, 128, 300, 180, n_sponge=-1)]
    eng = BatchEngine(arena_bytes=1 << 30, max_shots=16, tile=tile, steps_per_launch=steps,
                      launches_per_graph=3, form=form)
    results, stats = eng.run(jobs)
    assert stats["counted_points"] == sum(j.counted_points for j in jobs)
    for j, (img, ill) in zip(jobs, results):
        ref_img, ref_ill = _alone(j)
        np.testing.assert_array_equal(img, ref_img)
        np.testing.assert_array_equal(ill, ref_ill)


def test_batch_memory_admission_and_mix_independence():
    """With room for ~2 shots at a time, shots queue, enter as others leave, and
    each result equals the same shot migrated alone in the batch engine."""
    from das_gb300.batch import BatchEngine
    from das_gb300 import _lib
    jobs = [_job(10 + k, 60, 200, 120 + 10 * k) for k in range(6)]
    per = max(BatchEngine.shot_bytes(j) for j in jobs)
    eng = BatchEngine(arena_bytes=2 * per + (1 << 16), max_shots=8, steps_per_launch=8,
                      launches_per_graph=4)
    mixed, stats = eng.run(jobs)
    assert stats["max_active"] == 2
    alone = BatchEngine(arena_bytes=1 << 28, max_shots=2, steps_per_launch=8, launches_per_graph=4)
    for j, (img, ill) in zip(jobs, mixed):
        (img1, ill1), = alone.run([j])[0]
        np.testing.assert_array_equal(img, img1)
        np.testing.assert_array_equal(ill, ill1)


def test_batch_golden_migrate_shot(golden):
    from das_gb300.batch import BatchEngine, ShotJob
    g = golden("loops")
    nx, nz, dx, dt, n, a, fs = g["grid"]
    job = ShotJob(int(nx), int(nz), float(dx), float(dx), float(dt), g["vsmooth"], g["vsmooth"],
                  g["wavelet"], g["fwd_rec"], np.arange(int(nx)), 20, 2, 2, 2, int(n), float(a),
                  bool(fs))
    (img, ill), = BatchEngine(arena_bytes=1 << 28, max_shots=4).run([job])[0]
    np.testing.assert_array_equal(img, g["ms_image"])
    np.testing.assert_array_equal(ill, g["ms_illum"])


def test_batch_modelling_golden_mixed_with_migration(golden):
    """Forward-modelling jobs (observed gathers) and migration jobs share one
    replay; each gather equals the reference's forward traces, including the
    edge-cell source, edge and duplicated receivers, receivers in free-surface
    row 1 and a grid without a free surface."""
    from das_gb300.batch import BatchEngine, ModelJob
    g = golden("loops")
    nx, nz, dx, dt, n, a, fs = g["grid"]
    nx, nz, n = int(nx), int(nz), int(n)
    dx, dt, a = float(dx), float(dt), float(a)
    w, rq, vt = g["wavelet"], g["q_rec_ix"], g["vtrue"]
    models = [ModelJob(nx, nz, dx, dx, dt, vt, w, np.arange(nx), 20, 2, 2, n, a, True),
              ModelJob(nx, nz, dx, dx, dt, vt, w[:120], rq, 0, 2, 2, n, a, True),
              ModelJob(nx, nz, dx, dx, dt, vt, w[:120], rq, 31, 1, 1, n, a, True),
              ModelJob(nx, nz, dx, dx, dt, vt, w, np.arange(nx), 33, 6, 4, n, a, False)]
    expect = [g["fwd_rec"], g["q_fwd_rec"], g["q_row1_rec"], g["nofs_rec"]]
    jobs = [models[0], _job(1, 90, 260, 150), models[1], models[2], _job(2, 40, 130, 97, 3),
            models[3]]
    for form in ("grid", "queue"):
        eng = BatchEngine(arena_bytes=1 << 30, max_shots=16, steps_per_launch=11,
                          launches_per_graph=3, form=form)
        results, stats = eng.run(jobs)
        _check_modelling_mix(jobs, results, stats, expect)
        eng.close()


def _check_modelling_mix(jobs, results, stats, expect):
    assert stats["counted_points"] == sum(j.counted_points for j in jobs)
    for k, e in zip((0, 2, 3, 5), expect):
        r = results[k]
        assert r.shape == e.shape
        np.testing.assert_array_equal(r, e)
    for k in (1, 4):
        img, ill = results[k]
        ref_img, ref_ill = _alone(jobs[k])
        np.testing.assert_array_equal(img, ref_img)
        np.testing.assert_array_equal(ill, ref_ill)


def test_batch_modelling_matches_engine_forward():
    """Random grids: the batched gather equals WaveSolver2D.forward_propagate_acoustic."""
    from das_gb300.batch import BatchEngine, ModelJob
    from das_gb300.wave_solver import WaveSolver2D
    jobs = []
    for k, (nz, nx, nt, ns, fs) in enumerate([(70, 300, 140, 20, True), (41, 97, 77, -1, True),
                                               (128, 520, 90, 12, False)]):
        base = _job(30 + k, nz, nx, nt, n_sponge=ns, fs=fs)
        jobs.append(ModelJob(nx, nz, base.dx, base.dz, base.dt, base.vel_fwd, base.wavelet,
                             base.receiver_ix, base.source_ix, base.source_iz, base.receiver_iz,
                             ns, base.sponge_alpha, fs))
    results, _ = BatchEngine(arena_bytes=1 << 29, max_shots=8, steps_per_launch=16,
                             launches_per_graph=2).run(jobs)
    for j, tr in zip(jobs, results):
        s = WaveSolver2D(j.nx, j.nz, j.dx, j.dz, j.dt, j.n_sponge, j.sponge_alpha,
                         j.free_surface_top)
        ref, _ = s.forward_propagate_acoustic(j.vel, j.wavelet, j.source_ix, j.source_iz,
                                              j.receiver_ix, j.receiver_iz, False)
        np.testing.assert_array_equal(tr, ref)


@pytest.mark.parametrize("form", ["grid", "queue"])
def test_shots_sharing_a_model_key(form):
    """Six shots of one survey (one model pair, one key) plus a modelling job and an
    unkeyed shot, in an arena that admits only part of them at a time: every result
    equals the shot migrated alone, the shared model block is released with its last
    shot (the arena is whole again), and a key reused for another grid is refused."""
    import dataclasses
    from das_gb300._lib import W2DError
    from das_gb300.batch import BatchEngine, ModelJob
    base = _job(11, 80, 300, 140)
    rng = np.random.default_rng(12)
    jobs = []
    for k in range(6):
        data = (rng.standard_normal(base.data.shape) * 1e-7).astype(np.float32)
        jobs.append(dataclasses.replace(base, data=data, source_ix=int(20 + 40 * k),
                                        model_key=77))
    jobs.append(ModelJob(base.nx, base.nz, base.dx, base.dz, base.dt, base.vel_fwd, base.wavelet,
                         base.receiver_ix, 150, 3, 2, base.n_sponge, base.sponge_alpha, True,
                         model_key=78))
    jobs.append(_job(13, 50, 200, 90))
    per = max(BatchEngine.shot_bytes(j) for j in jobs)
    eng = BatchEngine(arena_bytes=int(3.2 * per), max_shots=8, tile=(4, 4), form=form)
    whole = eng.free_bytes()
    results, _ = eng.run(jobs)
    for j, res in zip(jobs, results):
        if isinstance(j, ModelJob):
            from das_gb300.wave_solver import WaveSolver2D
            s = WaveSolver2D(j.nx, j.nz, j.dx, j.dz, j.dt, j.n_sponge, j.sponge_alpha, True)
            want, _ = s.forward_propagate_acoustic(j.vel, j.wavelet, j.source_ix, j.source_iz,
                                                   j.receiver_ix, j.receiver_iz)
            np.testing.assert_array_equal(res, want)
            s.close()
        else:
            ref_img, ref_ill = _alone(j)
            np.testing.assert_array_equal(res[0], ref_img)
            np.testing.assert_array_equal(res[1], ref_ill)
    assert eng.free_bytes() == whole
    bad = dataclasses.replace(_job(14, 60, 120, 50), model_key=77)
    slot = eng.submit(dataclasses.replace(jobs[0]))
    with pytest.raises(W2DError):
        eng.submit(bad)
    eng.wait()
    eng.close()
    assert slot is not None


def test_batch_shot_without_receivers_and_one_step():
    """A shot with no receivers (zero image) and a one-step shot beside an ordinary one:
    each equals the shot migrated alone."""
    import dataclasses
    from das_gb300.batch import BatchEngine
    a = _job(21, 40, 100, 60)
    b = dataclasses.replace(_job(22, 30, 90, 40), data=np.zeros((40, 0), np.float32),
                            receiver_ix=np.zeros(0, dtype=np.int64))
    c = _job(23, 25, 70, 1)
    eng = BatchEngine(arena_bytes=1 << 28, max_shots=4, tile=(4, 4))
    results, _ = eng.run([a, b, c])
    for j, (img, ill) in zip([a, b, c], results):
        ref_img, ref_ill = _alone(j)
        np.testing.assert_array_equal(img, ref_img)
        np.testing.assert_array_equal(ill, ref_ill)
    assert not results[1][0].any()
    eng.close()


def test_cancel_mid_run_leaves_the_others_unchanged():
    """A job cancelled between replays leaves the batch: its slot is free again, its
    memory returns to the arena, and the jobs still running finish with the results they
    have alone."""
    from das_gb300.batch import BatchEngine
    jobs = [_job(40, 50, 180, 150), _job(41, 60, 220, 170), _job(42, 45, 150, 130)]
    eng = BatchEngine(arena_bytes=1 << 28, max_shots=4, steps_per_launch=8, launches_per_graph=2)
    free0 = eng.free_bytes()
    slots = [eng.submit(j) for j in jobs]
    assert None not in slots
    eng.step()  # 16 phase steps of every job: all still running
    assert not any(eng.finished(s) for s in slots)
    eng.cancel(slots[1])
    assert eng._lib.w2d_batch_is_finished(eng._h, slots[1]) == -1
    left = {slots[0]: jobs[0], slots[2]: jobs[2]}
    out = {}
    for _ in range(1000):
        if len(out) == len(left):
            break
        eng.step()
        for s, j in left.items():
            if s not in out and eng.finished(s):
                out[s] = eng.fetch(s, j.nz, j.nx)
    assert len(out) == len(left)
    assert eng.free_bytes() == free0
    for s, j in left.items():
        ref_img, ref_ill = _alone(j)
        np.testing.assert_array_equal(out[s][0], ref_img)
        np.testing.assert_array_equal(out[s][1], ref_ill)
    eng.close()
