"""Continuous-batching server: every job's result is the same alone and in the mix.

Requests arrive while others are on the GPU (simulated clock = device time of
the replays, so the interleaving does not depend on host speed); shots are
admitted by arena memory and overlap on the device.  Each shot's image and
illumination must equal the per-shot engine's migrate_shot result.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _shot(rng, nz, nx, nt):
    from das_gb300.batch import ShotJob
    from das_gb300.wave_solver import ricker_wavelet
    dx, dt = 5.0, 5e-4
    v = rng.uniform(1500, 3000, (nz, nx)).astype(np.float32)
    w, _ = ricker_wavelet(rng.uniform(8, 14), dt, nt * dt)
    rix = np.arange(0, nx, 2)
    data = (rng.standard_normal((len(w), len(rix))) * 1e-7).astype(np.float32)
    return ShotJob(nx, nz, dx, dx, dt, v, v, w, data, rix, int(rng.integers(3, nx - 3)), 2, 2, 2,
                   20, 0.002, True)


def _alone(job):
    from das_gb300.rtm_engine import TSWRTMEngine
    from das_gb300.velocity_flood import FloodModels
    from das_gb300.wave_solver import WaveSolver2D
    s = WaveSolver2D(job.nx, job.nz, job.dx, job.dz, job.dt, job.n_sponge, job.sponge_alpha, True)
    return TSWRTMEngine(s, "all").migrate_shot(FloodModels(job.vel_fwd, job.vel_fwd, job.vel_bwd,
                                                           0, 0), job.wavelet, job.source_ix,
                                               job.source_iz, job.data, job.receiver_ix, 2, 2)


def test_served_mix_with_elastic_jobs():
    """Elastic jobs run on the executor's own stream while acoustic shots batch; each
    result equals the same computation alone."""
    import torch
    from das_gb300.batch import BatchEngine, ShotJob
    from das_gb300.elastic import ElasticExecutor, ElasticSolver2D
    from das_gb300.serving import RTMRequest, RTMServer
    from das_gb300.wave_solver import ricker_wavelet
    rng = np.random.default_rng(5)
    nz, nx, dt = 40, 96, 5e-4
    vs = (300.0 + 600.0 * np.arange(nz)[:, None] / nz + 0.0 * np.arange(nx)[None, :]).astype(
        np.float32)
    w, _ = ricker_wavelet(12.0, dt, 0.05)
    w = (w * 1e6).astype(np.float32)
    rix = np.arange(2, nx - 2)
    el_shots = [ShotJob(nx, nz, 5.0, 5.0, dt, vs, vs, w,
                        (rng.standard_normal((len(w), len(rix))) * 1e-3).astype(np.float32), rix,
                        s, 2, 2, 2, 10, 0.003, True) for s in (20, 60)]
    trace = [RTMRequest(0, [_shot(rng, 50, 150, 80)], 0.0),
             RTMRequest(1, el_shots, 0.0, kind="elastic"),
             RTMRequest(2, [_shot(rng, 60, 120, 90), _shot(rng, 60, 120, 70)], 0.001)]
    ex = ElasticExecutor()
    eng = BatchEngine(arena_bytes=1 << 28, max_shots=8, tile=(4, 4), steps_per_launch=8,
                      launches_per_graph=2)
    out, stats = RTMServer(eng, elastic_executor=ex).serve(trace, realtime=True)
    ex.close()
    assert stats["shots"] == 5 and all(np.isfinite(r.latency) for r in out)
    solver = ElasticSolver2D(nx, nz, 5.0, 5.0, dt, 10, 0.003, True)
    for shot, (g, _) in zip(el_shots, out[1].results):
        g_alone, _ = ElasticExecutor.migrate_shot(solver, shot)
        np.testing.assert_array_equal(g, g_alone)
        assert np.abs(g).max() > 0
    for req in (trace[0], trace[2]):
        for shot, (img, ill) in zip(req.shots, out[req.job_id].results):
            ref_img, ref_ill = _alone(shot)
            np.testing.assert_array_equal(img, ref_img)
    del torch


def test_served_results_equal_alone():
    from das_gb300.batch import BatchEngine
    from das_gb300.serving import RTMRequest, RTMServer
    rng = np.random.default_rng(2)
    trace = []
    for j in range(6):
        shots = [_shot(rng, int(rng.integers(40, 90)), int(rng.integers(100, 300)),
                       int(rng.integers(60, 160))) for _ in range(int(rng.integers(1, 4)))]
        trace.append(RTMRequest(j, shots, arrival=0.0005 * j))
    per = max(BatchEngine.shot_bytes(s) for r in trace for s in r.shots)
    eng = BatchEngine(arena_bytes=4 * per, max_shots=16, tile=(4, 4), steps_per_launch=8,
                      launches_per_graph=2)
    out, stats = RTMServer(eng).serve(trace, realtime=False)
    assert stats["max_active_shots"] > 1
    assert stats["p50_latency_s"] <= stats["p99_latency_s"]
    for req, resp in zip(trace, out):
        assert resp.job_id == req.job_id and resp.latency > 0
        for shot, (img, ill) in zip(req.shots, resp.results):
            ref_img, ref_ill = _alone(shot)
            np.testing.assert_array_equal(img, ref_img)
            np.testing.assert_array_equal(ill, ref_ill)
