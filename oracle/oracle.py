"""CPU oracle for the 2D RTM engine.  TEST INFRASTRUCTURE ONLY.

Restates, with numpy loops over the per-step C operators of
``oracle/wave2d_oracle.c``, what ll23002/DAS computes on its RTM path:

* ``ricker_wavelet``                      tsw_rtm/wave_solver.py:74-81
* ``cerjan_sponge``                       tsw_rtm/c_engine/wave2d.c:237-265 (called at wave_solver.py:112-117)
* ``forward_propagate_acoustic``          tsw_rtm/wave_solver.py:128-186
* ``backward_propagate_and_correlate``    tsw_rtm/wave_solver.py:188-242
* ``migrate_shot``                        tsw_rtm/rtm_engine.py:49-104
* ``migrate_multiple_shots``              tsw_rtm/rtm_engine.py:106-171
* ``apply_laplacian_filter``              tsw_rtm/rtm_engine.py:27-38
* ``generate_velocity_flood_models``      tsw_rtm/velocity_flood.py:24-94

Every function has a ``precision`` argument: ``"f32"`` follows the reference's
float32 arithmetic step for step (injection products are float32 x float32
exactly as NumPy 2 evaluates ``float32_scalar * python_float``); ``"f64"`` runs
the same algorithm in float64 to state the error of a float32 result.

Only tests, the smoke check and the CPU-baseline leg of bench.py import this
module; the product path (package ``das_gb300``) never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass
from typing import Optional, Sequence, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIBS = {}


def build(native: bool = True) -> None:
    """Compile the oracle libraries (and the reference library when its source is present)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def _load(name: str = "liboracle.so") -> ctypes.CDLL:
    if name in _LIBS:
        return _LIBS[name]
    path = os.path.join(HERE, name)
    if not os.path.exists(path):
        build()
    lib = ctypes.CDLL(path)
    f32p = ctypes.c_void_p
    i = ctypes.c_int
    f = ctypes.c_float
    d = ctypes.c_double
    lib.oracle_acoustic_step_f32.argtypes = [f32p] * 5 + [i, i, f, f, f, i]
    lib.oracle_acoustic_step_f64.argtypes = [f32p] * 5 + [i, i, d, d, d, i]
    lib.oracle_elastic_step_f32.argtypes = [f32p] * 10 + [i, i, f, f, f, i]
    lib.oracle_elastic_step_f64.argtypes = [f32p] * 10 + [i, i, d, d, d, i]
    lib.oracle_correlate_f32.argtypes = [f32p] * 3 + [i, i, f]
    lib.oracle_correlate_f64.argtypes = [f32p] * 3 + [i, i, d]
    lib.oracle_cerjan_sponge.argtypes = [f32p, i, i, i, f, i]
    lib.oracle_num_threads.restype = ctypes.c_int
    lib.oracle_set_num_threads.argtypes = [i]
    lib.oracle_set_num_threads.restype = None
    for fn in ("oracle_acoustic_step_f32", "oracle_acoustic_step_f64", "oracle_elastic_step_f32",
               "oracle_elastic_step_f64", "oracle_correlate_f32", "oracle_correlate_f64",
               "oracle_cerjan_sponge"):
        getattr(lib, fn).restype = None
    _LIBS[name] = lib
    return lib


def lib(native: bool = False) -> ctypes.CDLL:
    return _load("liboracle_native.so" if native else "liboracle.so")


REF_LIB = os.path.join(HERE, "_ref", "libwave2d.so")


def reference_available() -> bool:
    """True where oracle/_ref holds the reference's wave2d.c compiled here from source."""
    return os.path.exists(REF_LIB)


def ref_lib() -> ctypes.CDLL:
    """The reference library itself (same symbols and argument types as its ctypes binding)."""
    if "ref" in _LIBS:
        return _LIBS["ref"]
    L = ctypes.CDLL(REF_LIB)
    p, i, f = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
    L.acoustic_2d_step.argtypes = [p] * 5 + [i, i, f, f, f, i]
    L.correlate_imaging_condition.argtypes = [p] * 3 + [i, i, f]
    L.acoustic_2d_step.restype = None
    L.correlate_imaging_condition.restype = None
    _LIBS["ref"] = L
    return L


# float32 step backend for the time loops: "port" (this restatement, -ffp-contract=off),
# "native" (the restatement with the reference's own compiler flags) or "reference"
# (oracle/_ref/libwave2d.so).  Used by the CPU-baseline timing.
_BACKEND = "port"


def set_backend(name: str) -> None:
    global _BACKEND
    if name not in ("port", "native", "reference"):
        raise ValueError(name)
    if name == "reference" and not reference_available():
        raise RuntimeError("oracle/_ref/libwave2d.so is not built")
    _BACKEND = name


def backend() -> str:
    return _BACKEND


def num_threads(native: bool = False) -> int:
    return int(lib(native).oracle_num_threads())


def set_num_threads(n: int) -> None:
    """Threads of the later parallel regions (the port, the native build and the
    reference library share the process's OpenMP runtime)."""
    lib(False).oracle_set_num_threads(int(n))
    lib(True).oracle_set_num_threads(int(n))


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


def _dtype(precision: str):
    if precision not in ("f32", "f64"):
        raise ValueError(precision)
    return np.float32 if precision == "f32" else np.float64


# --------------------------------------------------------------------------- operators

def ricker_wavelet(f0: float, dt: float, t_length: float) -> Tuple[np.ndarray, np.ndarray]:
    """Zero-phase Ricker wavelet in float64, returned as float32 (wave_solver.py:74-81)."""
    nt = int(round(t_length / dt))
    t = np.arange(nt) * dt
    arg = (np.pi * f0 * (t - 1.0 / f0)) ** 2
    w = (1.0 - 2.0 * arg) * np.exp(-arg)
    return w.astype(np.float32), t


def cerjan_sponge(nx: int, nz: int, n_sponge: int = 30, alpha: float = 0.0015,
                  free_surface_top: bool = True) -> np.ndarray:
    out = np.ones((nz, nx), dtype=np.float32)
    lib().oracle_cerjan_sponge(_ptr(out), nx, nz, n_sponge, alpha, 1 if free_surface_top else 0)
    return out


def acoustic_step(p_curr, p_prev, p_next, vel, sponge, nx, nz, dx, dz, dt, free_surface_top,
                  precision="f32", native=False):
    if precision == "f32" and _BACKEND == "reference":
        ref_lib().acoustic_2d_step(_ptr(p_curr), _ptr(p_prev), _ptr(p_next), _ptr(vel),
                                   _ptr(sponge), nx, nz, dx, dz, dt, 1 if free_surface_top else 0)
        return
    L = lib(native or _BACKEND == "native")
    fn = L.oracle_acoustic_step_f32 if precision == "f32" else L.oracle_acoustic_step_f64
    fn(_ptr(p_curr), _ptr(p_prev), _ptr(p_next), _ptr(vel), _ptr(sponge), nx, nz, dx, dz, dt,
       1 if free_surface_top else 0)


def elastic_step(vx, vz, sxx, szz, sxz, lam, mu, bx, bz, sponge, nx, nz, dx, dz, dt,
                 free_surface_top, precision="f32"):
    fn = lib().oracle_elastic_step_f32 if precision == "f32" else lib().oracle_elastic_step_f64
    fn(*[_ptr(a) for a in (vx, vz, sxx, szz, sxz, lam, mu, bx, bz, sponge)], nx, nz, dx, dz, dt,
       1 if free_surface_top else 0)


def correlate(src, rec, image, nx, nz, dt, precision="f32"):
    if precision == "f32" and _BACKEND == "reference":
        ref_lib().correlate_imaging_condition(_ptr(src), _ptr(rec), _ptr(image), nx, nz, dt)
        return
    fn = lib().oracle_correlate_f32 if precision == "f32" else lib().oracle_correlate_f64
    fn(_ptr(src), _ptr(rec), _ptr(image), nx, nz, dt)


# --------------------------------------------------------------------------- time loops

@dataclass
class Grid:
    nx: int
    nz: int
    dx: float
    dz: float
    dt: float
    n_sponge: int = 30
    sponge_alpha: float = 0.0015
    free_surface_top: bool = True

    def sponge(self) -> np.ndarray:
        return cerjan_sponge(self.nx, self.nz, self.n_sponge, self.sponge_alpha,
                             self.free_surface_top)


def _inject_scale(dt: float, precision: str):
    # wave_solver.py:159 and :213 multiply a float32 sample by the Python float dt**2;
    # under NumPy 2 the Python float is cast to float32 first.
    return np.float32(dt ** 2) if precision == "f32" else float(dt) ** 2


def forward_propagate_acoustic(g: Grid, velocity_model, source_ts, source_ix, source_iz,
                               receiver_ix, receiver_iz=2, save_wavefield=False,
                               snapshot_interval=1, precision="f32", sponge=None, native=False):
    """wave_solver.py:128-186, step for step."""
    dt_ = _dtype(precision)
    sp = (g.sponge() if sponge is None else sponge).astype(dt_)
    nt = len(source_ts)
    vel = np.ascontiguousarray(velocity_model, dtype=dt_)
    bufs = [np.zeros((g.nz, g.nx), dtype=dt_) for _ in range(3)]
    prev, curr, nxt = bufs
    rix = np.asarray(receiver_ix)
    rec = np.zeros((nt, len(rix)), dtype=dt_)
    snaps = [] if save_wavefield else None
    scale = _inject_scale(g.dt, precision)
    w = np.asarray(source_ts, dtype=np.float32).astype(dt_)
    dtc = g.dt
    for it in range(nt):
        curr[source_iz, source_ix] += w[it] * scale
        acoustic_step(curr, prev, nxt, vel, sp, g.nx, g.nz, g.dx, g.dz, dtc, g.free_surface_top,
                      precision, native)
        rec[it, :] = nxt[receiver_iz, rix]
        if save_wavefield and it % snapshot_interval == 0:
            snaps.append(curr.copy())
        prev, curr, nxt = curr, nxt, prev
    return rec, (np.array(snaps) if save_wavefield else None)


def backward_propagate_and_correlate(g: Grid, velocity_model, receiver_data, receiver_ix,
                                     receiver_iz, forward_wavefields, image_out,
                                     snapshot_interval=1, precision="f32", sponge=None,
                                     native=False):
    """wave_solver.py:188-242, step for step (receivers injected one at a time)."""
    dt_ = _dtype(precision)
    sp = (g.sponge() if sponge is None else sponge).astype(dt_)
    nt, n_rec = receiver_data.shape
    vel = np.ascontiguousarray(velocity_model, dtype=dt_)
    prev, curr, nxt = (np.zeros((g.nz, g.nx), dtype=dt_) for _ in range(3))
    scale = _inject_scale(g.dt, precision)
    data = np.asarray(receiver_data).astype(dt_)
    rix = [int(r) for r in receiver_ix]
    snap_idx = (nt - 1) // snapshot_interval
    dcorr = g.dt * snapshot_interval
    for it in range(nt - 1, -1, -1):
        row = data[it]
        for ir in range(n_rec):
            curr[receiver_iz, rix[ir]] += row[ir] * scale
        acoustic_step(curr, prev, nxt, vel, sp, g.nx, g.nz, g.dx, g.dz, g.dt, g.free_surface_top,
                      precision, native)
        if it % snapshot_interval == 0 and 0 <= snap_idx < len(forward_wavefields):
            fw = np.ascontiguousarray(forward_wavefields[snap_idx], dtype=dt_)
            correlate(fw, curr, image_out, g.nx, g.nz, dcorr, precision)
            snap_idx -= 1
        prev, curr, nxt = curr, nxt, prev


def migrate_shot(g: Grid, vel_fwd, vel_bwd, source_ts, source_ix, source_iz, receiver_data,
                 receiver_ix, receiver_iz=2, snapshot_interval=2, precision="f32", sponge=None,
                 native=False):
    """rtm_engine.py:49-104: forward with snapshots, illumination, backward + imaging."""
    dt_ = _dtype(precision)
    _, snaps = forward_propagate_acoustic(g, vel_fwd, source_ts, source_ix, source_iz,
                                          receiver_ix, receiver_iz, True, snapshot_interval,
                                          precision, sponge, native)
    scale = np.float32(g.dt * snapshot_interval) if precision == "f32" else g.dt * snapshot_interval
    illum = np.sum(snaps ** 2, axis=0) * scale
    image = np.zeros((g.nz, g.nx), dtype=dt_)
    backward_propagate_and_correlate(g, vel_bwd, receiver_data, receiver_ix, receiver_iz, snaps,
                                     image, snapshot_interval, precision, sponge, native)
    return image, illum


def apply_laplacian_filter(image: np.ndarray, dx: float, dz: float) -> np.ndarray:
    """rtm_engine.py:27-38: 3x3 Laplacian, 'same' size, symmetric boundary (scipy)."""
    from scipy import signal
    ix2, iz2 = 1.0 / (dx * dx), 1.0 / (dz * dz)
    k = np.array([[0.0, iz2, 0.0], [ix2, -2.0 * ix2 - 2.0 * iz2, ix2], [0.0, iz2, 0.0]],
                 dtype=np.float32)
    return signal.convolve2d(image, k, mode="same", boundary="symm")


@dataclass
class RTMResult:
    raw_image: np.ndarray
    laplacian_image: np.ndarray
    normalized_image: np.ndarray
    grid_x: np.ndarray
    grid_z: np.ndarray
    dx: float
    dz: float


def post_stack(g: Grid, stacked: np.ndarray, illum: np.ndarray, mute_sponge=True,
               sponge=None) -> RTMResult:
    """rtm_engine.py:145-171: sponge mute (< 0.99), illumination normalisation, Laplacian."""
    sp = g.sponge() if sponge is None else sponge
    stacked = stacked.copy()
    illum = illum.copy()
    if mute_sponge:
        mask = sp < 0.99
        stacked[mask] = 0.0
        illum[mask] = 0.0
    mx = np.max(illum)
    eps = 1e-4 * mx if mx > 0 else 1e-12
    normalized = stacked / (np.sqrt(illum) + eps)
    lap = apply_laplacian_filter(stacked, g.dx, g.dz)
    if mute_sponge:
        lap[mask] = 0.0
    return RTMResult(stacked, lap, normalized, np.arange(g.nx) * g.dx, np.arange(g.nz) * g.dz,
                     g.dx, g.dz)


def migrate_multiple_shots(g: Grid, vel_fwd, vel_bwd, source_waveforms: Sequence[np.ndarray],
                           source_ix: Sequence[int], source_iz: Sequence[int],
                           receiver_gathers: Sequence[np.ndarray], receiver_ix, receiver_iz=2,
                           snapshot_interval=2, mute_sponge=True, precision="f32",
                           native=False) -> RTMResult:
    """rtm_engine.py:106-171: serial shot loop, stack, post-stack."""
    dt_ = _dtype(precision)
    stacked = np.zeros((g.nz, g.nx), dtype=dt_)
    illum = np.zeros((g.nz, g.nx), dtype=dt_)
    for s in range(len(source_ix)):
        img, ill = migrate_shot(g, vel_fwd, vel_bwd, source_waveforms[s], source_ix[s],
                                source_iz[s], receiver_gathers[s], receiver_ix, receiver_iz,
                                snapshot_interval, precision, native=native)
        stacked += img
        illum += ill
    return post_stack(g, stacked, illum, mute_sponge)


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    """||a - b|| / ||b|| in float64 (0 when both are zero)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    na = np.linalg.norm(a - b)
    if nb == 0.0:
        return 0.0 if na == 0.0 else float("inf")
    return float(na / nb)


# --------------------------------------------------------------------------- elastic loop

def elastic_forward(g: Grid, lam, mu, bx, bz, source_ts, source_ix, source_iz, receiver_ix,
                    receiver_iz, precision="f32"):
    """Elastic modelling around the reference step (wave2d.c:95-212), which has no time
    loop of its own in the reference: before step n, vz[src] += w[n] * dt; after it,
    the vertical strain Dz- vz (4th-order staggered, the stress update's operator)
    is sampled at (receiver_iz, receiver_ix).  Row -1 reads zero."""
    dt_ = _dtype(precision)
    nz, nx = g.nz, g.nx
    f = [np.zeros((nz, nx), dtype=dt_) for _ in range(5)]
    vx, vz, sxx, szz, sxz = f
    P = [np.ascontiguousarray(a, dtype=dt_) for a in (lam, mu, bx, bz)]
    sp = g.sponge().astype(dt_)
    w = np.asarray(source_ts, dtype=np.float32).astype(dt_)
    dtv = dt_(g.dt) if precision == "f32" else g.dt
    rix = np.asarray(receiver_ix, dtype=np.int64)
    k1, k2 = dt_(9.0 / 8.0), dt_(-1.0 / 24.0)
    rdz = dt_(1.0) / dt_(g.dz)
    out = np.zeros((len(w), len(rix)), dtype=dt_)
    r = receiver_iz

    def row(a, i):
        return a[i] if i >= 0 else np.zeros(nx, dtype=dt_)

    for n in range(len(w)):
        vz[source_iz, source_ix] += w[n] * dtv
        elastic_step(vx, vz, sxx, szz, sxz, *P, sp, nx, nz, g.dx, g.dz, g.dt, g.free_surface_top,
                     precision)
        d = k1 * (row(vz, r) - row(vz, r - 1)) + k2 * (row(vz, r + 1) - row(vz, r - 2))
        out[n] = d[rix] * rdz
    return out


def gardner_parameters(vs, vp_over_vs=1.73, precision="f64"):
    dt_ = _dtype(precision)
    vs = np.asarray(vs, dtype=dt_)
    vp = dt_(vp_over_vs) * vs
    rho = dt_(310.0) * vp ** dt_(0.25)
    mu = rho * vs * vs
    lam = rho * vp * vp - dt_(2.0) * mu
    b = dt_(1.0) / rho
    return lam, mu, b, b


# --------------------------------------------------------------------------- flood models

def generate_velocity_flood_models(base_model, fault_x_idx, sediment_is_left=True,
                                   flood_offset_cells=15, perturb_sediment=0.0,
                                   perturb_rock=0.0):
    """tsw_rtm/velocity_flood.py:24-94 step for step: slice copies, then the per-column
    fill loops (Python indexing: a negative flood line counts from the end), then the
    fractional perturbations.  Returns (sediment_flood, rock_flood, line_sed, line_rock)."""
    base = np.asarray(base_model)
    nz, nx = base.shape
    sed = np.zeros_like(base)
    rock = np.zeros_like(base)
    if sediment_is_left:
        ls = min(nx - 1, fault_x_idx - flood_offset_cells)
        lr = max(0, fault_x_idx + flood_offset_cells)
        sed[:, :ls] = base[:, :ls]
        for ix in range(ls, nx):
            sed[:, ix] = base[:, ls]
        rock[:, lr:] = base[:, lr:]
        for ix in range(0, lr):
            rock[:, ix] = base[:, lr]
    else:
        ls = max(0, fault_x_idx + flood_offset_cells)
        lr = min(nx - 1, fault_x_idx - flood_offset_cells)
        sed[:, ls:] = base[:, ls:]
        for ix in range(0, ls):
            sed[:, ix] = base[:, ls]
        rock[:, :lr] = base[:, :lr]
        for ix in range(lr, nx):
            rock[:, ix] = base[:, lr]
    if perturb_sediment != 0.0:
        sed = sed * (1.0 + perturb_sediment)
    if perturb_rock != 0.0:
        rock = rock * (1.0 + perturb_rock)
    return sed.astype(np.float32), rock.astype(np.float32), ls, lr

