"""Generate ``golden_interferometry.npz`` by running the reference's own code.

``tsw_rtm/interferometry.py`` (cross-correlation, time-derivative Green's function,
virtual shot gathers) is executed from its source file, unchanged.  The gather
resampling helper ``resample_gather_to_sim_dt`` lives in ``run_das_pipeline.py``,
whose imports (HDF5 reader, plotting, report builder) are not installed here, so
that one function definition is taken out of the script's syntax tree and
executed alone with the names it uses (``np``, ``interp1d``).

The inputs are seeded synthetic stand-ins for preprocessed DAS windows: band-
limited noise with a few coherent arrivals moving along the cable.

Run from the repository root (needs the reference tree, which only this
development container has):

    python tests/golden/make_golden_interferometry.py
"""
from __future__ import annotations

import ast
import os
import sys
import types

import numpy as np
from scipy.interpolate import interp1d
from scipy.ndimage import gaussian_filter1d

OUT = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(OUT))
# the reference checkout: DAS_REFERENCE_ROOT, else a sibling folder "reference" beside the repo
REF_ROOT = os.environ.get("DAS_REFERENCE_ROOT", os.path.join(os.path.dirname(REPO), "reference"))


def load_interferometry():
    path = os.path.join(REF_ROOT, "tsw_rtm", "interferometry.py")
    with open(path, "r", encoding="utf-8") as fh:
        code = compile(fh.read(), path, "exec")
    mod = types.ModuleType("tsw_rtm.interferometry")
    mod.__file__ = path
    sys.modules[mod.__name__] = mod
    exec(code, mod.__dict__)
    return mod


def load_resample():
    path = os.path.join(REF_ROOT, "run_das_pipeline.py")
    with open(path, "r", encoding="utf-8") as fh:
        tree = ast.parse(fh.read(), path)
    fn = [n for n in tree.body
          if isinstance(n, ast.FunctionDef) and n.name == "resample_gather_to_sim_dt"]
    if len(fn) != 1:
        raise SystemExit("resample_gather_to_sim_dt not found in run_das_pipeline.py")
    mod = ast.Module(body=fn, type_ignores=[])
    ns = {"np": np, "interp1d": interp1d}
    exec(compile(mod, path, "exec"), ns)
    return ns["resample_gather_to_sim_dt"]


def das_window(rng, nt, n_ch, dt, dx):
    """Band-limited noise plus coherent arrivals crossing the cable (float32)."""
    x = rng.standard_normal((nt, n_ch))
    x = gaussian_filter1d(x, 2.0, axis=0)
    t = np.arange(nt) * dt
    pos = np.arange(n_ch) * dx
    for _ in range(6):
        t0, v = rng.uniform(0, nt * dt), rng.choice([-1, 1]) * rng.uniform(800, 3000)
        f = rng.uniform(1.0, 4.0)
        tau = t[:, None] - t0 - pos[None, :] / v
        x += 3.0 * np.exp(-(tau * f) ** 2) * np.cos(2 * np.pi * f * tau)
    return x.astype(np.float32)


def main():
    itf = load_interferometry()
    resample = load_resample()
    rng = np.random.default_rng(11)
    dt, dx, n_ch = 0.02, 4.0, 96
    files = [das_window(rng, 1500, n_ch, dt, dx), das_window(rng, 1500, n_ch, dt, dx),
             das_window(rng, 1111, n_ch, dt, dx)]
    src = np.array([20, 27, 35])
    rec = np.arange(32, n_ch - 4, 4)
    max_lag = 3.5
    g = {"dt": np.array(dt), "dx": np.array(dx), "max_lag": np.array(max_lag), "src": src,
         "rec": rec}
    for k, d in enumerate(files):
        g[f"data{k}"] = d
    # per-file correlations and the pipeline's float32 stack (run_das_pipeline.py:202-213,
    # :248-250): stacked = ccf of file 0, += the others, then /= number of files
    for s in src:
        stacked = None
        for k, d in enumerate(files):
            ccf, lags = itf.compute_cross_correlation(d, int(s), max_lag, dt, rec)
            g[f"ccf_s{s}_f{k}"] = ccf
            stacked = ccf.copy() if stacked is None else stacked + ccf
        stacked /= len(files)
        g[f"stack_s{s}"] = stacked
    g["lags"] = lags
    # default receivers (all channels), a short window and a lag longer than the window
    ccf_all, lags_all = itf.compute_cross_correlation(files[2][:300], 5, 0.5, dt)
    g.update(ccf_all=ccf_all, lags_all=lags_all)
    ccf_long, lags_long = itf.compute_cross_correlation(files[2][:120], 7, 3.0, dt, rec[:5])
    g.update(ccf_long=ccf_long, lags_long=lags_long)
    # Green's functions and virtual gathers from the stacked CCFs of the first source
    st = g[f"stack_s{src[0]}"]
    g["green_central"] = itf.time_derivative_greens(st, dt, "central")
    g["green_freq"] = itf.time_derivative_greens(st, dt, "frequency")
    g["green_full"] = itf.full_green_function(st, lags)
    coords = np.arange(n_ch) * dx
    for branch in ("causal", "anticausal", "symmetric"):
        for deriv in (True, False):
            vs = itf.build_virtual_shot_gather(st, lags, 0, int(src[0]), coords, rec, branch, deriv)
            tag = f"{branch}_{int(deriv)}"
            g[f"vs_{tag}_gather"] = vs.shot_gather
            g[f"vs_{tag}_time"] = vs.time_axis
            g[f"vs_{tag}_offsets"] = vs.offsets
            g[f"vs_{tag}_dt"] = np.array(vs.dt)
    # resampling to the simulation step (run_das_pipeline.py:48-55, used at :342-355)
    gat = g["vs_causal_1_gather"]
    for k, (dt_sim, nt_sim) in enumerate([(0.0015, int(round(max_lag / 0.0015))),
                                          (0.007, 600), (0.02, 176), (0.05, 40)]):
        g[f"rs{k}_args"] = np.array([dt_sim, nt_sim])
        g[f"rs{k}_out"] = resample(gat, dt_orig=dt, dt_sim=dt_sim, target_nt=nt_sim)
    np.savez_compressed(os.path.join(OUT, "golden_interferometry.npz"), **g)
    print("golden_interferometry.npz", os.path.getsize(os.path.join(OUT, "golden_interferometry.npz")))


if __name__ == "__main__":
    main()
