"""Parity of the CUDA engine against the reference's golden vectors and the CPU oracle.

Tolerances (stated by the engine's contract): wavefield snapshots and traces
within relative L2 1e-5, images within relative L2 1e-4, grid-index mapping
bit-exact.  The kernels evaluate every stencil in the reference's operation
order without FMA contraction, so in practice the float32 results are
bit-identical; the maximum absolute difference is asserted to be zero where
that holds so that any drift is seen at once.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as o

pytestmark = pytest.mark.gpu

SNAP_TOL = 1e-5
IMG_TOL = 1e-4


def _grid(g):
    nx, nz, dx, dt, n, a, fs = g["grid"]
    return o.Grid(int(nx), int(nz), float(dx), float(dx), float(dt), int(n), float(a), bool(fs))


def _solver(grid, **kw):
    from das_gb300.wave_solver import WaveSolver2D
    return WaveSolver2D(grid.nx, grid.nz, grid.dx, grid.dz, grid.dt, grid.n_sponge,
                        grid.sponge_alpha, grid.free_surface_top, **kw)


def _close(got, want, tol, exact=True, what=""):
    err = o.rel_l2(got, want)
    assert err <= tol, f"{what}: rel L2 {err:.3e} > {tol}"
    if exact:
        np.testing.assert_array_equal(got, want, err_msg=what)


# ---- reference-compatible per-step ABI ----------------------------------------------

def test_sponge_abi_bitwise(cuda_lib, golden):
    g = golden("sponge")
    for k in range(4):
        nx, nz, n, a, fs = g[f"sponge{k}_args"]
        out = np.ones((int(nz), int(nx)), np.float32)
        cuda_lib.build_cerjan_sponge(out.ctypes.data, int(nx), int(nz), int(n), float(a), int(fs))
        np.testing.assert_array_equal(out, g[f"sponge{k}"])


@pytest.mark.parametrize("fs", [0, 1])
@pytest.mark.parametrize("use_sponge", [0, 1])
def test_acoustic_step_abi(cuda_lib, golden, fs, use_sponge):
    g = golden("steps")
    nx, nz, dx, dz, dt = g["ac_args"]
    tag = f"ac_fs{fs}_sp{use_sponge}"
    out = g[f"{tag}_pn"].copy()
    sp = g[f"{tag}_sp"]
    rc = cuda_lib.w2d_acoustic_2d_step_status(
        g[f"{tag}_pc"].ctypes.data, g[f"{tag}_pp"].ctypes.data, out.ctypes.data,
        g[f"{tag}_vel"].ctypes.data, sp.ctypes.data if use_sponge else None, int(nx), int(nz),
        float(dx), float(dz), float(dt), fs)
    assert rc == 0, cuda_lib.w2d_last_error()
    _close(out, g[f"{tag}_out"], SNAP_TOL, what=tag)


@pytest.mark.parametrize("fs", [0, 1])
def test_elastic_step_abi(cuda_lib, golden, fs):
    g = golden("steps")
    nx, nz, dx, dz, dt = g["el_args"]
    tag = f"el_fs{fs}"
    f = [g[f"{tag}_{n}_in"].copy() for n in ("vx", "vz", "sxx", "szz", "sxz")]
    rc = cuda_lib.w2d_elastic_2d_step_status(
        *[a.ctypes.data for a in f], g[f"{tag}_lam"].ctypes.data, g[f"{tag}_mu"].ctypes.data,
        g[f"{tag}_bx"].ctypes.data, g[f"{tag}_bz"].ctypes.data, g[f"{tag}_sp"].ctypes.data,
        int(nx), int(nz), float(dx), float(dz), float(dt), fs)
    assert rc == 0, cuda_lib.w2d_last_error()
    for name, a in zip(("vx", "vz", "sxx", "szz", "sxz"), f):
        _close(a, g[f"{tag}_{name}_out"], SNAP_TOL, what=f"{tag} {name}")


def test_correlate_abi(cuda_lib, golden):
    g = golden("steps")
    out = g["corr_img"].copy()
    rc = cuda_lib.w2d_correlate_status(g["corr_src"].ctypes.data, g["corr_rec"].ctypes.data,
                                       out.ctypes.data, 31, 29, 2e-3)
    assert rc == 0
    _close(out, g["corr_out"], IMG_TOL, what="correlate")


def test_void_abi_symbols_run(cuda_lib, golden):
    """The reference-named void symbols run the same computation."""
    g = golden("steps")
    nx, nz, dx, dz, dt = g["ac_args"]
    tag = "ac_fs1_sp1"
    out = g[f"{tag}_pn"].copy()
    cuda_lib.acoustic_2d_step(g[f"{tag}_pc"].ctypes.data, g[f"{tag}_pp"].ctypes.data,
                              out.ctypes.data, g[f"{tag}_vel"].ctypes.data,
                              g[f"{tag}_sp"].ctypes.data, int(nx), int(nz), float(dx), float(dz),
                              float(dt), 1)
    np.testing.assert_array_equal(out, g[f"{tag}_out"])


# ---- whole-loop engine vs golden -------------------------------------------------------

def test_forward_golden(golden):
    g = golden("loops")
    s = _solver(_grid(g))
    rec, snaps = s.forward_propagate_acoustic(g["vtrue"], g["wavelet"], 20, 2, np.arange(s.nx), 2,
                                              True, 3)
    _close(rec, g["fwd_rec"], SNAP_TOL, what="traces")
    _close(snaps, g["fwd_snaps"], SNAP_TOL, what="snapshots")


def test_backward_golden(golden):
    g = golden("loops")
    s = _solver(_grid(g))
    rix = np.arange(s.nx)
    _, snaps = s.forward_propagate_acoustic(g["vsmooth"], g["wavelet"], 20, 2, rix, 2, True, 3)
    image = g["bwd_image0"].copy()
    s.backward_propagate_and_correlate(g["vsmooth"], g["fwd_rec"], rix, 2, snaps, image, 3)
    _close(image, g["bwd_image"], IMG_TOL, what="image")


def test_quirks_golden(golden):
    g = golden("loops")
    s = _solver(_grid(g))
    w = g["wavelet"][:120]
    rq = g["q_rec_ix"]
    rec, snaps = s.forward_propagate_acoustic(g["vtrue"], w, 0, 2, rq, 2, True, 1)
    _close(rec, g["q_fwd_rec"], SNAP_TOL, what="edge-source traces")
    _close(snaps[::7], g["q_fwd_snaps"], SNAP_TOL, what="edge-source snapshots")
    rec1, _ = s.forward_propagate_acoustic(g["vtrue"], w, 31, 1, rq, 1, False, 1)
    _close(rec1, g["q_row1_rec"], SNAP_TOL, what="row-1 traces")
    img = np.zeros((s.nz, s.nx), np.float32)
    s.backward_propagate_and_correlate(g["vsmooth"], rec, rq, 2, snaps, img, 1)
    _close(img, g["q_bwd_image"], IMG_TOL, what="duplicate-receiver image")


def test_no_free_surface_golden(golden):
    g = golden("loops")
    grid = _grid(g)
    grid.free_surface_top = False
    s = _solver(grid)
    rec, snaps = s.forward_propagate_acoustic(g["vtrue"], g["wavelet"], 33, 6, np.arange(s.nx), 4,
                                              True, 5)
    _close(rec, g["nofs_rec"], SNAP_TOL, what="traces")
    _close(snaps, g["nofs_snaps"], SNAP_TOL, what="snapshots")


@pytest.mark.parametrize("storage", ["all", "checkpoint"])
def test_migrate_shot_golden(golden, storage):
    from das_gb300.rtm_engine import TSWRTMEngine
    from das_gb300.velocity_flood import FloodModels
    g = golden("loops")
    s = _solver(_grid(g))
    eng = TSWRTMEngine(s, storage=storage)
    fm = FloodModels(g["vtrue"], g["vsmooth"], g["vsmooth"], 0, 0)
    img, ill = eng.migrate_shot(fm, g["wavelet"], 20, 2, g["fwd_rec"], np.arange(s.nx), 2, 2)
    assert s.last_stats()["storage"] == storage
    _close(img, g["ms_image"], IMG_TOL, what="image")
    _close(ill, g["ms_illum"], IMG_TOL, what="illumination")


@pytest.mark.parametrize("batch", ["off", "on"])
def test_migrate_multiple_golden(golden, batch):
    """The serial shot loop and the batched form (all shots advanced by the same
    launches, stacked in shot order), both against the reference's golden stack."""
    from das_gb300.rtm_engine import TSWRTMEngine
    from das_gb300.velocity_flood import FloodModels
    g = golden("loops")
    s = _solver(_grid(g))
    eng = TSWRTMEngine(s, batch=batch)
    fm = FloodModels(g["vtrue"], g["vsmooth"], g["vsmooth"], 0, 0)
    res = eng.migrate_multiple_shots(fm, [g["wavelet"]] * 3, list(g["mm_src_ix"]), [2] * 3,
                                     list(g["mm_gathers"]), np.arange(s.nx), 2, 2)
    _close(res.raw_image, g["mm_raw"], IMG_TOL, what="raw")
    _close(res.normalized_image, g["mm_norm"], IMG_TOL, what="normalized")
    # scipy's convolve2d (the reference's Laplacian, also used here) rounds
    # differently by an ulp between x86-64 and aarch64 builds: tolerance only
    _close(res.laplacian_image, g["mm_lap"], IMG_TOL, exact=False, what="laplacian")
    eng.close()


def test_migrate_multiple_batched_equals_serial():
    """Twelve shots with a caller-chosen interval and receivers on a row below the
    surface: the batched form's three images bit-identical to the serial loop's; a
    caller-modified sponge makes the batched form step aside (same result)."""
    from das_gb300.rtm_engine import TSWRTMEngine
    from das_gb300.velocity_flood import FloodModels
    from das_gb300.wave_solver import WaveSolver2D, ricker_wavelet
    nz, nx, dt = 90, 260, 1e-3
    rng = np.random.default_rng(12)
    vel = rng.uniform(1600, 2600, (nz, nx)).astype(np.float32)
    w, _ = ricker_wavelet(8.0, dt, 0.4)
    s = WaveSolver2D(nx, nz, 10.0, 10.0, dt, n_sponge=20)
    fm = FloodModels(vel, vel, (vel * 1.02).astype(np.float32), 0, 0)
    rix = np.arange(3, nx - 3, 2)
    gathers = [(rng.standard_normal((len(w), len(rix))) * 1e-3).astype(np.float32)
               for _ in range(12)]
    six = list(np.linspace(5, nx - 6, 12).astype(int))
    out = {}
    for mode in ("off", "on"):
        eng = TSWRTMEngine(s, batch=mode)
        out[mode] = eng.migrate_multiple_shots(fm, [w] * 12, six, [3] * 12, gathers, rix, 4, 3)
        eng.close()
    for f in ("raw_image", "laplacian_image", "normalized_image"):
        np.testing.assert_array_equal(getattr(out["on"], f), getattr(out["off"], f))
    assert np.abs(out["on"].raw_image).max() > 0
    s.sponge = s.sponge.copy()
    s.sponge[:, :5] *= 0.5
    eng = TSWRTMEngine(s, batch="on")
    assert not eng._use_batch(12)
    eng.close()


# ---- engine vs live oracle over shapes, tiles and intervals ----------------------------

CASES = [
    # nz, nx, n_sponge, fs, src (iz, ix), rec_iz, interval, tile
    (37, 53, 8, True, (2, 11), 2, 1, (8, 4)),
    (70, 300, 20, True, (3, 150), 3, 2, (4, 8)),
    (65, 129, 12, False, (5, 64), 7, 3, (8, 8)),
    (50, 200, 15, True, (2, 1), 2, 2, (4, 4)),
    (33, 131, 10, True, (2, 130), 2, 4, (8, 8)),
    (300, 700, 40, True, (2, 350), 2, 2, (8, 4)),
]


@pytest.mark.parametrize("case", CASES)
def test_forward_backward_vs_oracle(case):
    nz, nx, nsp, fs, (siz, six), riz, interval, tile = case
    rng = np.random.default_rng(nx * 7 + nz)
    grid = o.Grid(nx, nz, 7.5, 7.5, 8e-4, nsp, 0.003, fs)
    vel = rng.uniform(1500, 3200, (nz, nx)).astype(np.float32)
    w, _ = o.ricker_wavelet(12.0, grid.dt, 0.13)
    rix = np.sort(rng.integers(0, nx, size=nx // 3))
    s = _solver(grid)
    s.tile = tile
    rec, snaps = s.forward_propagate_acoustic(vel, w, six, siz, rix, riz, True, interval)
    rec_o, snaps_o = o.forward_propagate_acoustic(grid, vel, w, six, siz, rix, riz, True, interval)
    _close(rec, rec_o, SNAP_TOL, what="traces")
    _close(snaps, snaps_o, SNAP_TOL, what="snapshots")
    img = np.zeros((nz, nx), np.float32)
    img_o = np.zeros((nz, nx), np.float32)
    s.backward_propagate_and_correlate(vel, rec, rix, riz, snaps, img, interval)
    o.backward_propagate_and_correlate(grid, vel, rec_o, rix, riz, snaps_o, img_o, interval)
    _close(img, img_o, IMG_TOL, what="image")


def test_f64_error_statement():
    """Error of the float32 engine against a float64 run of the same stencil."""
    nz, nx = 60, 160
    grid = o.Grid(nx, nz, 10.0, 10.0, 1e-3, 15, 0.0015, True)
    rng = np.random.default_rng(3)
    vel = rng.uniform(1500, 3000, (nz, nx)).astype(np.float32)
    w, _ = o.ricker_wavelet(8.0, grid.dt, 0.4)
    rix = np.arange(nx)
    s = _solver(grid)
    rec, snaps = s.forward_propagate_acoustic(vel, w, 80, 2, rix, 2, True, 2)
    rec64, snaps64 = o.forward_propagate_acoustic(grid, vel, w, 80, 2, rix, 2, True, 2,
                                                  precision="f64")
    e_rec, e_snap = o.rel_l2(rec, rec64), o.rel_l2(snaps, snaps64)
    print(f"float32 engine vs float64 stencil: traces {e_rec:.2e}, snapshots {e_snap:.2e}")
    assert e_rec < 1e-4 and e_snap < 1e-4


def test_checkpoint_equals_full_storage_and_linearity():
    """Recomputation is exact, and the image is linear in the data."""
    from das_gb300.rtm_engine import TSWRTMEngine
    from das_gb300.velocity_flood import FloodModels
    nz, nx = 120, 400
    grid = o.Grid(nx, nz, 10.0, 10.0, 1e-3, 30, 0.0015, True)
    rng = np.random.default_rng(5)
    vel = rng.uniform(1500, 3000, (nz, nx)).astype(np.float32)
    w, _ = o.ricker_wavelet(6.0, grid.dt, 0.9)
    rix = np.arange(nx)
    s = _solver(grid)
    data, _ = s.forward_propagate_acoustic(vel * 1.02, w, 200, 2, rix, 2)
    fm = FloodModels(vel, vel, vel, 0, 0)
    img_a, ill_a = TSWRTMEngine(s, "all").migrate_shot(fm, w, 200, 2, data, rix, 2, 2)
    img_c, ill_c = TSWRTMEngine(s, "checkpoint").migrate_shot(fm, w, 200, 2, data, rix, 2, 2)
    assert s.last_stats()["recomputed_steps"] == len(w)
    np.testing.assert_array_equal(img_a, img_c)
    np.testing.assert_array_equal(ill_a, ill_c)
    # linear in the data: doubling is exact in float32 except where a product falls
    # into the subnormal range, which moves a rounding by an ulp here and there
    img_2, _ = TSWRTMEngine(s, "all").migrate_shot(fm, w, 200, 2, 2 * data, rix, 2, 2)
    assert o.rel_l2(img_2, 2 * img_a) < 1e-6


def test_errors_are_raised():
    from das_gb300._lib import W2DError
    grid = o.Grid(64, 48, 10.0, 10.0, 1e-3, 10, 0.0015, True)
    s = _solver(grid)
    vel = np.full((48, 64), 2000, np.float32)
    w = np.zeros(10, np.float32)
    with pytest.raises(IndexError):
        s.forward_propagate_acoustic(vel, w, 64, 2, np.arange(4), 2)
    with pytest.raises(IndexError):
        s.forward_propagate_acoustic(vel, w, 3, 2, np.array([0, 70]), 2)
    with pytest.raises(ValueError):
        s.forward_propagate_acoustic(np.zeros((10, 10), np.float32), w, 3, 2, np.arange(4), 2)
    # negative indices follow numpy semantics
    rec_neg, _ = s.forward_propagate_acoustic(vel, w + 1, -1, 2, np.array([-1, 0]), -46)
    rec_pos, _ = s.forward_propagate_acoustic(vel, w + 1, 63, 2, np.array([63, 0]), 2)
    np.testing.assert_array_equal(rec_neg, rec_pos)
    assert issubclass(W2DError, RuntimeError)


@pytest.mark.parametrize("nz,nx,nt,n_rec", [(5, 5, 1, 0), (5, 9, 7, 0), (6, 37, 13, 1), (41, 5, 9, 3)])
def test_degenerate_sizes_vs_oracle(nz, nx, nt, n_rec):
    """The smallest grids the engine takes, one-step runs and runs without receivers:
    traces, snapshots, image and illumination equal the oracle's (an empty receiver set
    gives (nt, 0) traces and a zero image)."""
    from das_gb300.rtm_engine import TSWRTMEngine
    from das_gb300.velocity_flood import FloodModels
    rng = np.random.default_rng(nz * 100 + nx)
    grid = o.Grid(nx, nz, 10.0, 10.0, 1e-3, 2, 0.01, True)
    vel = rng.uniform(1500, 2500, (nz, nx)).astype(np.float32)
    w = rng.standard_normal(nt).astype(np.float32)
    rix = np.sort(rng.integers(0, nx, size=n_rec))
    s = _solver(grid)
    rec, snaps = s.forward_propagate_acoustic(vel, w, nx // 2, 2, rix, 2, True, 1)
    rec_o, snaps_o = o.forward_propagate_acoustic(grid, vel, w, nx // 2, 2, rix, 2, True, 1)
    assert rec.shape == (nt, n_rec)
    np.testing.assert_array_equal(rec, rec_o)
    np.testing.assert_array_equal(snaps, snaps_o)
    data = (rng.standard_normal((nt, n_rec)) * 1e-3).astype(np.float32)
    fm = FloodModels(vel, vel, vel, 0, 0)
    img, ill = TSWRTMEngine(s).migrate_shot(fm, w, nx // 2, 2, data, rix, 2, 1)
    img_o, ill_o = o.migrate_shot(grid, vel, vel, w, nx // 2, 2, data, rix, 2, 1)
    np.testing.assert_array_equal(img, img_o)
    np.testing.assert_array_equal(ill, ill_o)
    if n_rec == 0:
        assert not img.any()
    s.close()
