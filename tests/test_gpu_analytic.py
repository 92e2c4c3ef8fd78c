"""Analytic known-answer checks of the scheme and directional-derivative checks of the
adjoints.

* Dispersion: a standing wave cos(kx) cos(wt) is an exact solution of the discrete
  scheme (4th-order Laplacian, leapfrog) when cos(w dt) = 1 + v^2 dt^2 L(k) / 2 with
  L(k) = (c0 + 2 c1 cos(k dx) + 2 c2 cos(2 k dx)) / dx^2; one step of the GPU engine
  must reproduce it, and the implied phase velocity must differ from v by the
  scheme's known dispersion error.
* Travel time: in a homogeneous medium the arrival-time difference between two
  receivers on a line through the source is their distance difference over v.
* Adjoints: <dJ/dm, dm> against a float64 central difference of J along a random
  smooth direction dm (acoustic velocity and elastic shear velocity).
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as o

pytestmark = pytest.mark.gpu

C0, C1, C2 = -2.5, 4.0 / 3.0, -1.0 / 12.0


@pytest.mark.parametrize("ppw", [40.0, 10.0, 5.0, 3.0])
def test_standing_wave_is_exact_for_the_discrete_scheme(cuda_lib, ppw):
    nx, nz, dx, dt, v = 257, 9, 10.0, 1e-3, 2000.0
    k = 2.0 * np.pi / (ppw * dx)
    L = (C0 + 2 * C1 * np.cos(k * dx) + 2 * C2 * np.cos(2 * k * dx)) / dx ** 2
    c = 1.0 + (v * dt) ** 2 * L / 2.0  # cos(w dt) of the discrete scheme
    x = np.arange(nx) * dx
    row = np.cos(k * x)
    p_curr = np.ascontiguousarray(np.broadcast_to(row, (nz, nx)), dtype=np.float32)
    p_prev = np.ascontiguousarray(np.broadcast_to(row * c, (nz, nx)), dtype=np.float32)
    p_next = np.zeros((nz, nx), np.float32)
    vel = np.full((nz, nx), v, np.float32)
    rc = cuda_lib.w2d_acoustic_2d_step_status(p_curr.ctypes.data, p_prev.ctypes.data,
                                              p_next.ctypes.data, vel.ctypes.data, None, nx, nz,
                                              ctypes.c_float(dx), ctypes.c_float(dx),
                                              ctypes.c_float(dt), 0)
    assert rc == 0
    # interior rows/columns are updated; z is uniform so only the x operator acts
    got = p_next[2:nz - 2, 2:nx - 2].astype(np.float64)
    want = (row * c)[2:nx - 2][None, :]
    assert np.max(np.abs(got - want)) < 5e-6
    # phase velocity of the scheme against the continuum: the 4th-order stencil's
    # relative error at `ppw` points per wavelength
    w_num = np.arccos(c) / dt
    err = w_num / (v * k) - 1.0
    print(f"{ppw} points per wavelength: phase velocity error {err:+.2e}")
    # the known behaviour of the scheme: negligible at 10 or more points per
    # wavelength, a few percent at 3-5
    assert abs(err) < {40.0: 1e-4, 10.0: 1e-3, 5.0: 2e-2, 3.0: 1e-1}[ppw]


def test_homogeneous_travel_time():
    """Two receivers 100 and 300 cells from a buried source in a 2000 m/s medium: the
    lag between their direct arrivals is 200 dx / v within two samples.  The grid keeps
    the sponge's reflections out of the windows (the Cerjan sponge of the scheme
    reflects low frequencies noticeably), and no free surface."""
    from das_gb300.wave_solver import WaveSolver2D, ricker_wavelet
    nz, nx, dx, dt, v = 400, 900, 5.0, 5e-4, 2000.0
    s = WaveSolver2D(nx, nz, dx, dx, dt, n_sponge=40, free_surface_top=False)
    w, _ = ricker_wavelet(15.0, dt, 1.0)
    src = (200, 150)  # (iz, ix)
    rix = np.array([src[1] + 100, src[1] + 300])
    rec, _ = s.forward_propagate_acoustic(np.full((nz, nx), v, np.float32), w, src[1], src[0], rix,
                                          src[0])
    # direct arrivals: near at 0.25 s + the wavelet delay, far at 0.75 s + it; the first
    # sponge reflection reaches the near receiver after 0.8 s and the far one after 1.1 s
    a = rec[: int(0.6 / dt), 0].astype(np.float64)
    b = rec[:, 1].astype(np.float64)
    cc = np.correlate(b, a, mode="full")
    lag = (np.argmax(cc) - (len(a) - 1)) * dt
    want = 200 * dx / v
    print(f"arrival lag {lag * 1e3:.2f} ms, expected {want * 1e3:.2f} ms")
    assert abs(lag - want) <= 2 * dt


def _smooth_direction(rng, nz, nx, sigma=3.0):
    from scipy.ndimage import gaussian_filter
    d = gaussian_filter(rng.standard_normal((nz, nx)), sigma)
    return d / np.max(np.abs(d))


def test_acoustic_gradient_directional_derivative():
    import torch
    from das_gb300.autograd import model_traces
    from das_gb300.wave_solver import WaveSolver2D, ricker_wavelet
    nz, nx, dx, dt = 50, 120, 10.0, 1e-3
    rng = np.random.default_rng(21)
    v0 = (1800.0 + 12.0 * np.arange(nz)[:, None] + 0.0 * np.arange(nx)[None, :]).astype(np.float32)
    w, _ = ricker_wavelet(12.0, dt, 0.25)
    rix = np.arange(5, nx - 5)
    R = rng.standard_normal((len(w), len(rix)))
    s = WaveSolver2D(nx, nz, dx, dx, dt, n_sponge=10)
    v = torch.tensor(v0, device="cuda", requires_grad=True)
    J = (model_traces(v, s, w, 60, 5, rix, 3) * torch.tensor(R, dtype=torch.float32,
                                                             device="cuda")).sum()
    J.backward()
    g = v.grad.cpu().numpy().astype(np.float64)
    grid = o.Grid(nx, nz, dx, dx, dt, 10, 0.0015, True)
    dm = _smooth_direction(rng, nz, nx) * 5.0  # m/s

    def J64(m):
        d, _ = o.forward_propagate_acoustic(grid, m, w, 60, 5, rix, 3, precision="f64")
        return float(np.sum(d * R))

    h = 1.0
    fd = (J64(v0 + h * dm) - J64(v0 - h * dm)) / (2 * h)
    an = float(np.sum(g * dm))
    err = abs(an - fd) / abs(fd)
    print(f"acoustic <grad, dm> {an:.6e} vs central difference {fd:.6e}: rel {err:.2e}")
    assert err < 2e-3


def test_elastic_gradient_directional_derivative():
    import torch
    from das_gb300.elastic import ElasticSolver2D, elastic_traces, gardner_parameters
    from das_gb300.wave_solver import ricker_wavelet
    nz, nx, dx, dt = 40, 80, 5.0, 5e-4
    rng = np.random.default_rng(22)
    vs0 = (300.0 + 900.0 * np.arange(nz)[:, None] / (nz - 1) + 0.0 * np.arange(nx)[None, :]
           ).astype(np.float32)
    w, _ = ricker_wavelet(12.0, dt, 0.15)
    w = (w * 1e6).astype(np.float32)
    rix = np.arange(4, nx - 4)
    R = rng.standard_normal((len(w), len(rix)))
    solver = ElasticSolver2D(nx, nz, dx, dx, dt, n_sponge=10, sponge_alpha=0.003)
    v = torch.tensor(vs0, device="cuda", requires_grad=True)
    J = (elastic_traces(v, solver, w, 40, 3, rix, 2) *
         torch.tensor(R, dtype=torch.float32, device="cuda")).sum()
    J.backward()
    g = v.grad.cpu().numpy().astype(np.float64)
    grid = o.Grid(nx, nz, dx, dx, dt, 10, 0.003, True)
    dm = _smooth_direction(rng, nz, nx) * 3.0  # m/s

    def J64(m):
        lam, mu, bx, bz = o.gardner_parameters(m, precision="f64")
        d = o.elastic_forward(grid, lam, mu, bx, bz, w, 40, 3, rix, 2, precision="f64")
        return float(np.sum(d * R))

    h = 1.0
    fd = (J64(vs0 + h * dm) - J64(vs0 - h * dm)) / (2 * h)
    an = float(np.sum(g * dm))
    err = abs(an - fd) / abs(fd)
    print(f"elastic <grad, dm> {an:.6e} vs central difference {fd:.6e}: rel {err:.2e}")
    assert err < 2e-3
