"""Step launch modes: one CTA per tile or persistent CTAs over a tile counter, each
with or without programmatic dependent launch, give bit-identical results.

The persistent form draws tiles from a counter that is never reset between
launches (each launch draws exactly ntiles + grid indices); long runs with
checkpoint recomputation, forward and backward passes and many launches check
that the accounting holds.
"""
import numpy as np
import pytest

from oracle import oracle as o

pytestmark = pytest.mark.gpu

MODES = [("grid", False), ("persistent", False), ("persistent", True)]


def _solver(grid, tile, mode):
    from das_gb300.wave_solver import WaveSolver2D
    s = WaveSolver2D(grid.nx, grid.nz, grid.dx, grid.dz, grid.dt, grid.n_sponge,
                     grid.sponge_alpha, grid.free_surface_top)
    s.tile = tile
    s.set_launch(*mode)
    return s


def test_golden_in_every_mode(golden):
    from das_gb300.rtm_engine import TSWRTMEngine
    from das_gb300.velocity_flood import FloodModels
    g = golden("loops")
    nx, nz, dx, dt, n, a, fs = g["grid"]
    grid = o.Grid(int(nx), int(nz), float(dx), float(dx), float(dt), int(n), float(a), bool(fs))
    for mode in MODES:
        for tile in [(4, 4), (8, 4)]:
            s = _solver(grid, tile, mode)
            rec, snaps = s.forward_propagate_acoustic(g["vtrue"], g["wavelet"], 20, 2,
                                                      np.arange(s.nx), 2, True, 3)
            np.testing.assert_array_equal(rec, g["fwd_rec"], err_msg=str((mode, tile)))
            np.testing.assert_array_equal(snaps, g["fwd_snaps"], err_msg=str((mode, tile)))
            fm = FloodModels(g["vtrue"], g["vsmooth"], g["vsmooth"], 0, 0)
            img, ill = TSWRTMEngine(s).migrate_shot(fm, g["wavelet"], 20, 2, g["fwd_rec"],
                                                    np.arange(s.nx), 2, 2)
            np.testing.assert_array_equal(img, g["ms_image"], err_msg=str((mode, tile)))
            np.testing.assert_array_equal(ill, g["ms_illum"], err_msg=str((mode, tile)))
            s.close()


@pytest.mark.parametrize("shape", [(300, 1100, 40), (97, 389, 12), (1000, 1500, 30)])
def test_modes_identical_with_checkpoints(shape):
    """Migration with checkpoint recomputation (many passes and launches) and with full
    storage: every mode equals the default launch (one CTA per tile, PDL)."""
    from das_gb300.rtm_engine import TSWRTMEngine
    from das_gb300.velocity_flood import FloodModels
    nz, nx, nsp = shape
    rng = np.random.default_rng(nz + nx)
    grid = o.Grid(nx, nz, 5.0, 5.0, 5e-4, nsp, 0.0015, True)
    v = rng.uniform(1500, 3200, (nz, nx)).astype(np.float32)
    w, _ = o.ricker_wavelet(15.0, grid.dt, 0.1)
    rix = np.sort(rng.integers(0, nx, size=nx // 2))
    data = (rng.standard_normal((len(w), len(rix))) * 1e-7).astype(np.float32)
    fm = FloodModels(v, v, v * 1.02, 0, 0)
    results = {}
    for mode in [("grid", True)] + MODES:
        s = _solver(grid, (4, 4), mode)
        for storage in ("all", "checkpoint"):
            img, ill = TSWRTMEngine(s, storage).migrate_shot(fm, w, nx // 3, 2, data, rix, 2, 2)
            results[(mode, storage)] = (img, ill)
        s.close()
    ref_img, ref_ill = results[(("grid", True), "all")]
    for key, (img, ill) in results.items():
        np.testing.assert_array_equal(img, ref_img, err_msg=str(key))
        np.testing.assert_array_equal(ill, ref_ill, err_msg=str(key))


@pytest.mark.parametrize("fs,custom_sponge,rows", [(True, False, True), (False, False, 2),
                                                   (True, True, 4), (True, False, 2)])
def test_two_step_equals_one_step(fs, custom_sponge, rows):
    """Two time steps per launch (default) against one: traces, snapshots, image and
    illumination bit-identical, with an odd number of steps, receivers on the edge
    columns (cells the reference never writes, where injections accumulate), the
    source next to a corner, a caller-made sponge array, and checkpoint recomputation
    over segments of uneven length (the last one odd)."""
    from das_gb300.rtm_engine import TSWRTMEngine
    from das_gb300.velocity_flood import FloodModels
    from das_gb300.wave_solver import WaveSolver2D
    nz, nx = 83, 301
    rng = np.random.default_rng(17)
    grid = o.Grid(nx, nz, 5.0, 5.0, 5e-4, 14, 0.003, fs)
    v = rng.uniform(1500, 3200, (nz, nx)).astype(np.float32)
    w, _ = o.ricker_wavelet(18.0, grid.dt, 0.0905)  # 181 steps
    assert len(w) % 2 == 1
    rix = np.concatenate([[0, 1, 1], np.sort(rng.integers(2, nx - 2, size=60)), [nx - 2, nx - 1]])
    data = (rng.standard_normal((len(w), len(rix))) * 1e-6).astype(np.float32)
    fm = FloodModels(v, v, (v * 1.01).astype(np.float32), 0, 0)
    out = {}
    for two in (rows, False):
        s = WaveSolver2D(nx, nz, grid.dx, grid.dz, grid.dt, grid.n_sponge, grid.sponge_alpha, fs)
        if custom_sponge:
            s.sponge = (s.sponge * rng.uniform(0.9, 1.0, s.sponge.shape)).astype(np.float32) \
                if two is not False else out["sponge"]
            out["sponge"] = s.sponge
        s.set_two_step(two)
        rec, snaps = s.forward_propagate_acoustic(v, w, 3, 2 if fs else 3, rix, 2, True, 3)
        img = np.zeros((nz, nx), np.float32)
        s.backward_propagate_and_correlate(v, data, rix, 2, snaps, img, 3)
        res = [rec, snaps, img]
        for storage in ("all", "checkpoint"):
            res += list(TSWRTMEngine(s, storage).migrate_shot(fm, w, nx - 4, 2, data, rix, 2, 2))
        out[two] = res
        s.close()
    for a, b in zip(out[rows], out[False]):
        np.testing.assert_array_equal(a, b)
    assert np.abs(out[rows][2]).max() > 0


@pytest.mark.parametrize("storage", ["all", "checkpoint"])
def test_graph_replays_equal_direct_launches(storage):
    """Migrations replaying captured pass graphs (the default) equal migrations whose
    steps are launched one by one from the host, bit for bit, over a sequence of shots:
    the first shot captures, later shots with new sources, receivers' data and models
    replay the cached graphs, a shorter shot captures again, and the step counts the
    engine reports are the same."""
    from das_gb300.rtm_engine import TSWRTMEngine
    from das_gb300.velocity_flood import FloodModels
    from das_gb300.wave_solver import WaveSolver2D
    nz, nx = 180, 700
    rng = np.random.default_rng(5)
    grid = o.Grid(nx, nz, 5.0, 5.0, 5e-4, 30, 0.0015, True)
    w, _ = o.ricker_wavelet(12.0, grid.dt, 0.12)
    rix = np.arange(3, nx - 3, 3)
    shots = []
    for k, (six, nt) in enumerate([(100, len(w)), (350, len(w)), (620, len(w)), (40, len(w) - 37),
                                   (500, len(w))]):
        v = rng.uniform(1600, 3000, (nz, nx)).astype(np.float32)
        d = (rng.standard_normal((nt, len(rix))) * 1e-6).astype(np.float32)
        shots.append((FloodModels(v, v, (v * 1.01).astype(np.float32), 0, 0), w[:nt], six, d))
    out = {}
    for graphs in (True, False):
        s = WaveSolver2D(nx, nz, 5.0, 5.0, grid.dt, 30, 0.0015, True)
        s.set_graphs(graphs)
        eng = TSWRTMEngine(s, storage=storage)
        res = []
        for fm, wk, six, d in shots:
            img, ill = eng.migrate_shot(fm, wk, six, 2, d, rix, 2, 2)
            st = s.last_stats()
            res.append((img, ill, st["step_launches"], st["recomputed_steps"], st["storage"]))
        out[graphs] = res
        s.close()
    for k, (a, b) in enumerate(zip(out[True], out[False])):
        np.testing.assert_array_equal(a[0], b[0], err_msg=f"image, shot {k}")
        np.testing.assert_array_equal(a[1], b[1], err_msg=f"illumination, shot {k}")
        assert a[2:] == b[2:] and a[4] == storage, (k, a[2:], b[2:])
        assert np.abs(a[0]).max() > 0


def test_graph_replays_equal_direct_launches_modelling_and_correlation():
    """forward_propagate_acoustic (traces only, and traces with snapshots) and
    backward_propagate_and_correlate also replay cached pass graphs: over several calls
    with new sources, wavelets, receivers' data and images, and a change of length that
    captures again, every result equals the one-launch-per-step run bit for bit."""
    from das_gb300.wave_solver import WaveSolver2D
    nz, nx = 150, 520
    rng = np.random.default_rng(9)
    grid = o.Grid(nx, nz, 5.0, 5.0, 5e-4, 25, 0.0015, True)
    v = rng.uniform(1600, 3000, (nz, nx)).astype(np.float32)
    w, _ = o.ricker_wavelet(15.0, grid.dt, 0.1)
    rix = np.arange(2, nx - 2, 5)
    calls = []
    for k, (six, nt, snaps) in enumerate([(60, len(w), False), (300, len(w), False),
                                          (400, len(w), True), (90, len(w) - 11, True),
                                          (250, len(w), False)]):
        d = (rng.standard_normal((nt, len(rix))) * 1e-6).astype(np.float32)
        img0 = (rng.standard_normal((nz, nx)) * 1e-9).astype(np.float32)
        calls.append((six, w[:nt] * (1.0 + 0.1 * k), snaps, d, img0))
    out = {}
    for graphs in (True, False):
        s = WaveSolver2D(nx, nz, 5.0, 5.0, grid.dt, 25, 0.0015, True)
        s.set_graphs(graphs)
        res = []
        for six, wk, snaps, d, img0 in calls:
            rec, sn = s.forward_propagate_acoustic(v, wk.astype(np.float32), six, 2, rix, 2,
                                                   snaps, 2)
            res.append(rec)
            if snaps:
                res.append(sn)
                img = img0.copy()
                s.backward_propagate_and_correlate(v, d, rix, 2, sn, img, 2)
                res.append(img)
        out[graphs] = res
        s.close()
    assert len(out[True]) == len(out[False])
    for k, (a, b) in enumerate(zip(out[True], out[False])):
        np.testing.assert_array_equal(a, b, err_msg=f"result {k}")
