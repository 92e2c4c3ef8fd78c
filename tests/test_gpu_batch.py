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


@pytest.mark.parametrize("tile,steps", [((8, 4), 16), ((4, 4), 7), ((4, 8), 33)])
def test_batch_equals_single_shot(tile, steps):
    from das_gb300.batch import BatchEngine
    jobs = [_job(1, 90, 260, 150), _job(2, 40, 130, 97, interval=3),
            _job(3, 70, 400, 211, interval=1, fs=False), _job(4, 33, 77, 64, n_sponge=8),
            _job(5, 128, 300, 180, n_sponge=-1)]
    eng = BatchEngine(arena_bytes=1 << 30, max_shots=16, tile=tile, steps_per_launch=steps,
                      launches_per_graph=3)
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
