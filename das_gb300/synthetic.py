"""Seeded synthetic workloads for the RTM engine's benchmark configurations.

The reference publishes no dataset for this path; these generators stand in
with the shapes, sizes and value ranges of the benchmark configurations:

* ``plain_small``  150 x 400 grid, dx = 10 m, vp 1500 -> 3000 m/s with depth, a 200 m
  +400 m/s layer at 700 m cut by a 60-degree fault with 100 m throw; migration model
  Gaussian-smoothed (sigma 5 cells); 20 sources, 400 receivers; 3 Hz Ricker,
  dt 1 ms, nt 2000; sponge 40 cells.
* ``plain_large``  1000 x 4000 grid, dx = 2.5 m; the same model scaled to depth plus two
  faults of random dip in [45, 75] degrees; 200 sources, 4000 receivers; 6 Hz Ricker,
  dt 0.25 ms, nt 8000.
* ``batched_gathers``  uneven sub-grids (nx in [400, 2000], nz in [200, 600], dx 5 m),
  smoothed layered models with 1-3 faults (vp 1500-3500 m/s), 3-5 Hz Ricker,
  nt in [1500, 4000].

Sources and receivers sit on grid row 2 (the reference drivers use rows 2 or 3:
run_das_pipeline.py:352,371; run_synthetic_benchmarks.py:52-53).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List

import numpy as np

from .wave_solver import ricker_wavelet

SURFACE_IZ = 2


@dataclass
class Survey:
    name: str
    nz: int
    nx: int
    dx: float
    dz: float
    dt: float
    nt: int
    f0: float
    n_sponge: int
    sponge_alpha: float
    vel_true: np.ndarray
    vel_mig: np.ndarray
    src_ix: np.ndarray
    src_iz: int
    rec_ix: np.ndarray
    rec_iz: int
    wavelet: np.ndarray
    meta: dict = field(default_factory=dict)

    @property
    def points(self) -> int:
        return self.nz * self.nx

    def counted_points_per_shot(self) -> int:
        """Point-updates of one RTM shot: forward + backward, 2 * nz * nx * nt."""
        return 2 * self.nz * self.nx * self.nt


def _layered_faulted(nz, nx, dx, dz, layer_top, layer_thick, throw, faults, v0=1500.0, v1=3000.0,
                     dv_layer=400.0):
    """Velocity rising linearly with depth plus a fast layer offset by normal faults.

    faults: list of (surface_x_m, dip_deg, throw_m); the layer on the hanging-wall
    side (x greater than the fault trace at that depth) is shifted down by throw_m.
    """
    z = (np.arange(nz) * dz)[:, None]
    x = (np.arange(nx) * dx)[None, :]
    zmax = (nz - 1) * dz
    v = v0 + (v1 - v0) * z / zmax + 0.0 * x
    top = np.full((nz, nx), layer_top)
    for xs, dip, th in faults:
        trace = xs + z / np.tan(np.deg2rad(dip))
        top = top + np.where(x > trace, th, 0.0)
    v = v + np.where((z >= top) & (z < top + layer_thick), dv_layer, 0.0)
    return v.astype(np.float32)


def plain_small(seed: int = 0, nt: int = 2000) -> Survey:
    from scipy.ndimage import gaussian_filter
    nz, nx, d = 150, 400, 10.0
    faults = [(0.5 * (nx - 1) * d, 60.0, 100.0)]
    vt = _layered_faulted(nz, nx, d, d, 700.0, 200.0, 100.0, faults)
    vm = gaussian_filter(vt.astype(np.float64), 5.0).astype(np.float32)
    dt = 1e-3
    w, _ = ricker_wavelet(3.0, dt, nt * dt)
    return Survey("plain 2D acoustic RTM 150x400, nt=2000, 20 shots x 400 receivers", nz, nx, d, d,
                  dt, len(w), 3.0, 40, 0.0015, vt, vm, np.arange(20) * 20 + 10, SURFACE_IZ,
                  np.arange(nx), SURFACE_IZ, w, {"seed": seed})


def plain_large(seed: int = 0, nt: int = 8000, n_shots: int = 200) -> Survey:
    from scipy.ndimage import gaussian_filter
    rng = np.random.default_rng(seed)
    nz, nx, d = 1000, 4000, 2.5
    scale = ((nz - 1) * d) / (149 * 10.0)  # the small model scaled to this depth
    faults = [(0.5 * (nx - 1) * d, 60.0, 100.0 * scale)]
    for _ in range(2):
        faults.append((rng.uniform(0.15, 0.85) * (nx - 1) * d, rng.uniform(45.0, 75.0),
                       rng.uniform(0.5, 1.0) * 100.0 * scale * rng.choice([-1.0, 1.0])))
    vt = _layered_faulted(nz, nx, d, d, 700.0 * scale, 200.0 * scale, 100.0 * scale, faults)
    vm = gaussian_filter(vt.astype(np.float64), 5.0).astype(np.float32)
    dt = 2.5e-4
    w, _ = ricker_wavelet(6.0, dt, nt * dt)
    src = (np.arange(n_shots) * nx) // n_shots + nx // (2 * n_shots)
    return Survey(f"large plain 2D acoustic RTM 1000x4000, nt={len(w)}, 4000 receivers", nz, nx, d,
                  d, dt, len(w), 6.0, 40, 0.0015, vt, vm, src, SURFACE_IZ, np.arange(nx),
                  SURFACE_IZ, w, {"seed": seed, "faults": faults})


def plain_large_window(n_steps: int = 240, first_sample: int = 560, seed: int = 0) -> Survey:
    """The 1000 x 4000 survey cut to ``n_steps`` time steps for checks that a CPU
    restatement must finish in seconds: the same grid, models, sponge, receivers and
    sources, with the 6 Hz Ricker taken from ``first_sample`` on (its main lobe, which
    peaks at sample 667, falls inside the window instead of after it)."""
    sv = plain_large(seed=seed, nt=8000)
    w = np.ascontiguousarray(sv.wavelet[first_sample:first_sample + n_steps])
    sv.name = (f"large plain 2D acoustic RTM 1000x4000 cut to {len(w)} steps "
               f"(Ricker from sample {first_sample}), 4000 receivers")
    sv.wavelet = w
    sv.nt = len(w)
    sv.meta = dict(sv.meta, first_sample=first_sample)
    return sv


@dataclass
class Gather:
    nz: int
    nx: int
    dx: float
    dt: float
    nt: int
    f0: float
    vel: np.ndarray
    src_ix: int
    wavelet: np.ndarray


def batched_gathers(n: int = 256, seed: int = 0, dt: float = 5e-4, nt_range=(1500, 4000),
                    nx_range=(400, 2000), nz_range=(200, 600)) -> List[Gather]:
    """Uneven virtual-source gathers; dt 0.5 ms keeps CFL <= 0.5 at 3500 m/s and dx 5 m."""
    from scipy.ndimage import gaussian_filter
    rng = np.random.default_rng(seed)
    out = []
    d = 5.0
    for _ in range(n):
        nx = int(rng.integers(nx_range[0], nx_range[1] + 1))
        nz = int(rng.integers(nz_range[0], nz_range[1] + 1))
        nt = int(rng.integers(nt_range[0], nt_range[1] + 1))
        f0 = float(rng.uniform(3.0, 5.0))
        zmax = (nz - 1) * d
        faults = [(rng.uniform(0.2, 0.8) * (nx - 1) * d, rng.uniform(45.0, 80.0),
                   rng.uniform(-0.08, 0.08) * zmax) for _ in range(int(rng.integers(1, 4)))]
        v = _layered_faulted(nz, nx, d, d, rng.uniform(0.3, 0.6) * zmax,
                             rng.uniform(0.08, 0.2) * zmax, 0.0, faults,
                             v0=1500.0, v1=float(rng.uniform(2600.0, 3100.0)), dv_layer=400.0)
        v = np.clip(gaussian_filter(v.astype(np.float64), 4.0), 1500.0, 3500.0).astype(np.float32)
        w, _ = ricker_wavelet(f0, dt, nt * dt)
        out.append(Gather(nz, nx, d, dt, len(w), f0, v, int(rng.integers(40, nx - 40)), w))
    return out


def elastic_fault_zone(nz: int = 1024, nx: int = 2048, dx: float = 2.0, vs_top: float = 300.0,
                       vs_bottom: float = 1200.0, zone_width_m: float = 20.0, dip_deg: float = 70.0,
                       zone_factor: float = 0.7) -> np.ndarray:
    """Shear velocity rising linearly with depth, cut by a low-velocity fault zone of
    the given width dipping at dip_deg from the middle of the surface."""
    z = (np.arange(nz) * dx)[:, None]
    x = (np.arange(nx) * dx)[None, :]
    vs = vs_top + (vs_bottom - vs_top) * z / ((nz - 1) * dx) + 0.0 * x
    x0 = 0.5 * (nx - 1) * dx
    # distance to the plane through (x0, 0) dipping dip_deg
    th = np.deg2rad(dip_deg)
    dist = np.abs((x - x0) * np.sin(th) - z * np.cos(th))
    vs = np.where(dist <= 0.5 * zone_width_m, vs * zone_factor, vs)
    return vs.astype(np.float32)
