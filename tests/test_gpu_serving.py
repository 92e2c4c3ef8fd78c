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
