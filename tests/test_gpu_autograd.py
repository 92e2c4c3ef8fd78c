"""Differentiable path: traces, finite-difference gradient check, relation to RTM.

The velocity gradient of J = 0.5 * ||d(v) - d_obs||^2 comes from the hand-written
adjoint kernel (acoustic_adjoint_kernel) behind torch.autograd; the forward
wavefield is recomputed from checkpoints.  Checked against central finite
differences of J evaluated by the float64 oracle on 16 random cells.
"""
import numpy as np
import pytest

from oracle import oracle as o

pytestmark = pytest.mark.gpu

NZ, NX, DX, DT = 50, 100, 10.0, 1e-3


def _setup():
    from das_gb300.wave_solver import WaveSolver2D, ricker_wavelet
    rng = np.random.default_rng(7)
    z = np.arange(NZ)[:, None]
    x = np.arange(NX)[None, :]
    v0 = (1800.0 + 15.0 * z + 0.0 * x).astype(np.float32)
    vt = v0.copy()
    vt[25:32, 30:70] += 250.0
    w, _ = ricker_wavelet(12.0, DT, 0.25)
    rix = np.arange(5, NX - 5)
    grid = o.Grid(NX, NZ, DX, DX, DT, 10, 0.0015, True)
    d_obs, _ = o.forward_propagate_acoustic(grid, vt, w, 50, 6, rix, 3, precision="f64")
    s = WaveSolver2D(NX, NZ, DX, DX, DT, n_sponge=10)
    return s, grid, v0, vt, w, rix, d_obs, rng


def test_traces_equal_forward_propagate():
    import torch
    from das_gb300.autograd import model_traces
    s, grid, v0, vt, w, rix, d_obs, _ = _setup()
    d = model_traces(torch.tensor(v0, device="cuda"), s, w, 50, 6, rix, 3).cpu().numpy()
    d_ref, _ = s.forward_propagate_acoustic(v0, w, 50, 6, rix, 3)
    np.testing.assert_array_equal(d, d_ref)


def test_gradient_matches_finite_differences():
    from das_gb300.autograd import misfit_and_gradient
    s, grid, v0, vt, w, rix, d_obs, rng = _setup()
    J, g = misfit_and_gradient(s, v0, w, 50, 6, rix, 3, d_obs.astype(np.float32))
    assert np.isfinite(g).all() and np.abs(g).max() > 0

    def J64(v):
        d, _ = o.forward_propagate_acoustic(grid, v, w, 50, 6, rix, 3, precision="f64")
        return 0.5 * np.sum((d - d_obs) ** 2)

    cells = [(int(rng.integers(8, 40)), int(rng.integers(12, 88))) for _ in range(16)]
    fd, an = [], []
    for iz, ix in cells:
        h = 1e-3 * float(v0[iz, ix])
        vp = v0.astype(np.float64).copy()
        vm = vp.copy()
        vp[iz, ix] += h
        vm[iz, ix] -= h
        fd.append((J64(vp) - J64(vm)) / (2 * h))
        an.append(float(g[iz, ix]))
    fd, an = np.array(fd), np.array(an)
    err = np.linalg.norm(an - fd) / np.linalg.norm(fd)
    print(f"gradient vs central differences on 16 cells: rel-L2 {err:.2e}")
    assert err < 1e-3, (an, fd)


def test_gradient_relates_to_rtm_image():
    """The adjoint-state gradient and the zero-lag RTM image of the residual share
    their structure (the gradient correlates p_adj with d2p/dt2 instead of p)."""
    from das_gb300.autograd import misfit_and_gradient
    from das_gb300.rtm_engine import TSWRTMEngine
    from das_gb300.velocity_flood import FloodModels
    s, grid, v0, vt, w, rix, d_obs, rng = _setup()
    d0, _ = s.forward_propagate_acoustic(v0, w, 50, 6, rix, 3)
    resid = (d0 - d_obs).astype(np.float32)
    _, g = misfit_and_gradient(s, v0, w, 50, 6, rix, 3, d_obs.astype(np.float32))
    img, _ = TSWRTMEngine(s).migrate_shot(FloodModels(v0, v0, v0, 0, 0), w, 50, 6, resid, rix, 3, 1)
    m = (slice(8, 40), slice(12, 88))
    c = np.corrcoef(g[m].ravel(), img[m].ravel())[0, 1]
    print(f"correlation(gradient, RTM image of the residual) = {c:.3f}")
    assert c < -0.8  # d2/dt2 ~ -omega^2: anti-correlated with the zero-lag image


@pytest.mark.parametrize("nz,nx,fs,layout", [
    (50, 100, True, "line"),       # one partial tile column, receivers on row 3
    (70, 300, True, "gaps"),       # receivers every third column (the CSR lookup)
    (90, 520, False, "line"),      # no free surface: the sponge on all four sides
    (130, 700, True, "shuffled"),  # receivers in no column order, some columns twice
])
def test_vectorised_adjoint_equals_per_cell_adjoint(nz, nx, fs, layout):
    """The vectorised adjoint kernel (float4 lanes, register window, plain tiles stored
    as float4) against the per-cell kernel on grids with frame tiles, partial tiles,
    the receiver row, the free-surface fold and the sponge: the same gradient to float32
    rounding (they differ only in the compiler's contraction choices)."""
    from das_gb300.autograd import misfit_and_gradient
    from das_gb300.wave_solver import WaveSolver2D, ricker_wavelet
    rng = np.random.default_rng(nz + nx)
    z = np.arange(nz)[:, None]
    v = (1800.0 + 12.0 * z + 40.0 * rng.standard_normal((nz, nx))).astype(np.float32)
    w, _ = ricker_wavelet(15.0, DT, 0.2)
    if layout == "line":
        rix = np.arange(2, nx - 2)
    elif layout == "gaps":
        rix = np.arange(2, nx - 2, 3)
    else:
        rix = rng.permutation(np.concatenate([np.arange(2, nx - 2, 2), np.arange(5, 60, 7)]))
    riz = 2 if fs else 3
    d_obs = (1e-9 * rng.standard_normal((len(w), len(rix)))).astype(np.float32)
    s = WaveSolver2D(nx, nz, DX, DX, DT, n_sponge=12, free_surface_top=fs)
    grads = {}
    for form in ("cells", "tiled"):
        s.set_adjoint_form(form)
        J, g = misfit_and_gradient(s, v, w, nx // 3, 6, rix, riz, d_obs)
        grads[form] = g
    s.close()
    a, b = grads["tiled"].astype(np.float64), grads["cells"].astype(np.float64)
    assert np.abs(b).max() > 0
    rel = np.linalg.norm(a - b) / np.linalg.norm(b)
    print(f"{nz} x {nx} ({layout}, free surface {fs}): vectorised vs per-cell rel L2 {rel:.2e}")
    assert rel < 1e-5


def test_gradient_of_8000_steps_on_the_large_grid():
    """An 8000-step shot on the 1000 x 4000 grid.  By default the forward states come
    back from checkpoints (about sqrt(3 nt) steps per segment, one segment of states
    stored at a time), so the gradient fits in a few GB of HBM.  The same gradient
    with every forward state stored by the forward pass itself (8000 planes, 128 GB:
    nothing recomputed) must be equal bit for bit, because the recomputation replays
    the same kernels on the same inputs."""
    import time
    from das_gb300.autograd import misfit_and_gradient
    from das_gb300.wave_solver import WaveSolver2D, ricker_wavelet
    nz, nx, dx, dt, nt = 1000, 4000, 2.5, 2.5e-4, 8000
    v = (1500.0 + 1.5 * np.arange(nz)[:, None] + 0.0 * np.arange(nx)[None, :]).astype(np.float32)
    w, _ = ricker_wavelet(6.0, dt, nt * dt)
    rix = np.arange(2, nx - 2, 4)
    d_obs = np.zeros((len(w), len(rix)), np.float32)
    s = WaveSolver2D(nx, nz, dx, dx, dt, n_sponge=30)
    t0 = time.perf_counter()
    J, g = misfit_and_gradient(s, v, w, nx // 2, 2, rix, 2, d_obs)
    el = time.perf_counter() - t0
    st = s.last_stats()
    assert np.isfinite(J) and J > 0
    assert np.isfinite(g).all() and np.abs(g).max() > 0
    assert st["recomputed_steps"] == nt  # each segment recomputed once from its checkpoint
    s.set_checkpoint_segment(nt)
    t0 = time.perf_counter()
    J_full, g_full = misfit_and_gradient(s, v, w, nx // 2, 2, rix, 2, d_obs)
    el_full = time.perf_counter() - t0
    assert s.last_stats()["recomputed_steps"] == 0
    s.close()
    print(f"8000-step gradient on 1000 x 4000: checkpointed {el:.2f} s "
          f"({st['recomputed_steps']} steps recomputed), all states stored {el_full:.2f} s")
    assert J_full == J
    np.testing.assert_array_equal(g_full, g)


def test_device_arguments_refuse_host_memory():
    """A DEVICE argument that is host memory is refused on the host with W2D_EINVAL
    before any launch, and the handle stays usable.  The host memory is page-locked,
    which the device can read through its mapping, so no launch could fault on it even
    if the check let it through."""
    import torch
    from das_gb300 import _lib
    from das_gb300.elastic import ElasticSolver2D
    from das_gb300.pinned import pinned_array
    s, grid, v0, vt, w, rix, d_obs, _ = _setup()
    lib = _lib.load()
    w32 = np.ascontiguousarray(w, dtype=np.float32)
    r = np.ascontiguousarray(rix, dtype=np.int32)
    host_vel = pinned_array(v0.shape)
    host_vel[...] = v0
    traces = torch.empty((len(w32), len(r)), dtype=torch.float32, device="cuda")

    def msg():
        m = lib.w2d_last_error()
        return m.decode() if isinstance(m, bytes) else str(m)

    rc = lib.w2d_fwi_forward(s._eng(), host_vel.ctypes.data, w32.ctypes.data, len(w32), 50, 6,
                             r.ctypes.data, len(r), 3, traces.data_ptr())
    assert rc == 1 and "not device memory" in msg(), msg()
    vel = torch.tensor(v0, device="cuda")
    torch.cuda.synchronize()
    assert lib.w2d_fwi_forward(s._eng(), vel.data_ptr(), w32.ctypes.data, len(w32), 50, 6,
                               r.ctypes.data, len(r), 3, traces.data_ptr()) == 0
    torch.cuda.synchronize()
    d_ref, _ = s.forward_propagate_acoustic(v0, w, 50, 6, rix, 3)
    np.testing.assert_array_equal(traces.cpu().numpy(), d_ref)

    es = ElasticSolver2D(64, 32, 2.0, 2.0, 2e-4, 8, 0.0015, True)
    try:
        lam = pinned_array((32, 64))
        lam[...] = 1.0
        dev = torch.ones((32, 64), dtype=torch.float32, device="cuda")
        etr = torch.empty((1, 20, 60), dtype=torch.float32, device="cuda")
        ew = np.zeros((1, 20), np.float32)
        six, siz = np.array([32], np.int32), np.array([10], np.int32)
        erix = np.arange(2, 62, dtype=np.int32)
        rc = lib.w2d_elastic_forward_batch(es._h, 1, lam.ctypes.data, dev.data_ptr(),
                                           dev.data_ptr(), dev.data_ptr(), ew.ctypes.data, 20,
                                           six.ctypes.data, siz.ctypes.data, erix.ctypes.data,
                                           len(erix), 2, etr.data_ptr())
        assert rc == 1 and "lam" in msg() and "not device memory" in msg(), msg()
    finally:
        es.close()
