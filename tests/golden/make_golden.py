"""Generate the golden fixtures in this folder by running the reference itself.

The reference Python modules (tsw_rtm/wave_solver.py, tsw_rtm/velocity_flood.py,
tsw_rtm/rtm_engine.py) are executed from their source files, unchanged, with the
ctypes load of ``libwave2d.so`` redirected to the library that ``oracle/Makefile``
compiles from the reference's own ``wave2d.c`` into ``oracle/_ref/``.  The
prebuilt binary shipped inside the reference tree and its ``__pycache__`` are
never loaded: each module is compiled here from its ``.py`` source.

Run from the repository root (needs the reference tree, which only this
development container has):

    make -C oracle && python tests/golden/make_golden.py

Outputs ``golden_*.npz``; each array is small so the fixtures stay a few MB.
"""
from __future__ import annotations

import ctypes
import os
import sys
import types

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
# the reference checkout: DAS_REFERENCE_ROOT, else a sibling folder "reference" beside the repo
REF_ROOT = os.environ.get("DAS_REFERENCE_ROOT", os.path.join(os.path.dirname(REPO), "reference"))
OUT = os.path.dirname(os.path.abspath(__file__))
REF_LIB = os.path.join(REPO, "oracle", "_ref", "libwave2d.so")


def load_reference():
    """Execute the reference modules from source with the library load redirected."""
    if not os.path.exists(REF_LIB):
        raise SystemExit("oracle/_ref/libwave2d.so missing: run `make -C oracle` first")
    pkg = types.ModuleType("tsw_rtm")
    pkg.__path__ = []  # nothing is imported implicitly from the reference tree
    sys.modules["tsw_rtm"] = pkg
    real_cdll = ctypes.CDLL

    def cdll(name, *a, **k):
        if str(name).endswith("libwave2d.so"):
            name = REF_LIB
        return real_cdll(name, *a, **k)

    mods = {}
    ctypes.CDLL = cdll
    try:
        for name in ("wave_solver", "velocity_flood", "rtm_engine"):
            path = os.path.join(REF_ROOT, "tsw_rtm", name + ".py")
            with open(path, "r", encoding="utf-8") as fh:
                code = compile(fh.read(), path, "exec")
            mod = types.ModuleType("tsw_rtm." + name)
            mod.__file__ = path
            mod.__package__ = "tsw_rtm"
            sys.modules["tsw_rtm." + name] = mod
            exec(code, mod.__dict__)
            mods[name] = mod
    finally:
        ctypes.CDLL = real_cdll
    return mods


def layered_fault_model(nz, nx, dz, dx, seed=0):
    """Small smoothed gradient + layer + dipping fault model for the fixtures."""
    from scipy.ndimage import gaussian_filter
    z = np.arange(nz)[:, None] * dz
    x = np.arange(nx)[None, :] * dx
    zmax = (nz - 1) * dz
    v = 1500.0 + 1500.0 * z / zmax + 0.0 * x
    xf = 0.5 * (nx - 1) * dx + z / np.tan(np.deg2rad(60.0))
    top = 0.45 * zmax + np.where(x > xf, 0.08 * zmax, 0.0)
    v = v + np.where((z >= top) & (z < top + 0.15 * zmax), 400.0, 0.0)
    return v.astype(np.float32), gaussian_filter(v, 3.0).astype(np.float32)


def main():
    ref = load_reference()
    ws, re, vf = ref["wave_solver"], ref["rtm_engine"], ref["velocity_flood"]
    lib = ws._lib
    rng = np.random.default_rng(20240611)

    # --- sponge tables (wave2d.c:237-265 via WaveSolver2D.__init__) -------------
    sp = {}
    for k, (nx, nz, n, a, fs) in enumerate([(400, 150, 40, 0.0015, True), (64, 48, 10, 0.0015, True),
                                            (53, 37, 8, 0.004, False), (20, 12, 15, 0.0015, True)]):
        s = ws.WaveSolver2D(nx=nx, nz=nz, dx=10.0, dz=10.0, dt=1e-3, n_sponge=n,
                            sponge_alpha=a, free_surface_top=fs)
        sp[f"sponge{k}"] = s.sponge
        sp[f"sponge{k}_args"] = np.array([nx, nz, n, a, int(fs)], dtype=np.float64)
    np.savez_compressed(os.path.join(OUT, "golden_sponge.npz"), **sp)

    # --- single steps --------------------------------------------------------------
    st = {}
    nz, nx = 37, 53
    for fs in (0, 1):
        for use_sponge in (0, 1):
            tag = f"ac_fs{fs}_sp{use_sponge}"
            pc = rng.standard_normal((nz, nx)).astype(np.float32)
            pp = rng.standard_normal((nz, nx)).astype(np.float32)
            pn = rng.standard_normal((nz, nx)).astype(np.float32)
            vel = rng.uniform(1500, 3500, (nz, nx)).astype(np.float32)
            spg = rng.uniform(0.5, 1.0, (nz, nx)).astype(np.float32)
            out = pn.copy()
            lib.acoustic_2d_step(pc.ctypes.data, pp.ctypes.data, out.ctypes.data, vel.ctypes.data,
                                 spg.ctypes.data if use_sponge else None, nx, nz,
                                 ctypes.c_float(7.5), ctypes.c_float(5.0), ctypes.c_float(6e-4), fs)
            st.update({f"{tag}_pc": pc, f"{tag}_pp": pp, f"{tag}_pn": pn, f"{tag}_vel": vel,
                       f"{tag}_sp": spg, f"{tag}_out": out})
    st["ac_args"] = np.array([nx, nz, 7.5, 5.0, 6e-4])

    # elastic: two zero guard rows in front of row 0 (the reference reads row -1
    # of sxz and vz when the free surface is on).
    nz, nx = 33, 47
    guard = 2
    for fs in (0, 1):
        tag = f"el_fs{fs}"
        fields = [rng.standard_normal((nz, nx)).astype(np.float32) * 1e-3 for _ in range(5)]
        vp = rng.uniform(1500, 3000, (nz, nx)).astype(np.float32)
        vs = (vp / 1.73).astype(np.float32)
        rho = rng.uniform(1800, 2600, (nz, nx)).astype(np.float32)
        mu = (rho * vs * vs).astype(np.float32)
        lam = (rho * vp * vp - 2 * mu).astype(np.float32)
        bx = (1.0 / rho).astype(np.float32)
        bz = (1.0 / rho).astype(np.float32)
        spg = rng.uniform(0.7, 1.0, (nz, nx)).astype(np.float32)
        padded = []
        for f in fields:
            p = np.zeros((nz + guard, nx), dtype=np.float32)
            p[guard:] = f
            padded.append(p)
        ptrs = [p.ctypes.data + guard * nx * 4 for p in padded]
        lib.elastic_2d_step(*ptrs, lam.ctypes.data, mu.ctypes.data, bx.ctypes.data,
                            bz.ctypes.data, spg.ctypes.data, nx, nz, ctypes.c_float(2.0),
                            ctypes.c_float(2.5), ctypes.c_float(2e-4), fs)
        for name, f, p in zip(("vx", "vz", "sxx", "szz", "sxz"), fields, padded):
            st[f"{tag}_{name}_in"] = f
            st[f"{tag}_{name}_out"] = p[guard:].copy()
            assert not p[:guard].any()
        st.update({f"{tag}_lam": lam, f"{tag}_mu": mu, f"{tag}_bx": bx, f"{tag}_bz": bz,
                   f"{tag}_sp": spg})
    st["el_args"] = np.array([nx, nz, 2.0, 2.5, 2e-4])

    src = rng.standard_normal((29, 31)).astype(np.float32)
    rec = rng.standard_normal((29, 31)).astype(np.float32)
    img = rng.standard_normal((29, 31)).astype(np.float32)
    out = img.copy()
    lib.correlate_imaging_condition(src.ctypes.data, rec.ctypes.data, out.ctypes.data, 31, 29,
                                    ctypes.c_float(2e-3))
    st.update(corr_src=src, corr_rec=rec, corr_img=img, corr_out=out)
    np.savez_compressed(os.path.join(OUT, "golden_steps.npz"), **st)

    # --- Ricker wavelet and index mapping --------------------------------------------
    rk = {}
    for k, (f0, dt, T) in enumerate([(3.0, 1e-3, 2.0), (6.0, 2.5e-4, 2.0), (5.0, 2e-4, 0.3)]):
        w, t = ws.ricker_wavelet(f0, dt, T)
        rk[f"w{k}"], rk[f"t{k}"] = w, t
        rk[f"args{k}"] = np.array([f0, dt, T])
    # source/receiver grid-index mapping used by the reference drivers
    # (run_synthetic_benchmarks.py:50-51, run_das_pipeline.py:350-351)
    rk["map_src"] = np.linspace(35, 200 - 15, 7, dtype=int)
    rk["map_rec"] = np.linspace(200 + 15, 400 - 35, 50, dtype=int)
    half = np.arange(0, 81)
    rk["map_half_in"] = half
    rk["map_half"] = np.array([int(round(s / 2)) for s in half])
    np.savez_compressed(os.path.join(OUT, "golden_ricker.npz"), **rk)

    # --- time loops ------------------------------------------------------------------
    lp = {}
    nz, nx, dx, dt = 48, 64, 10.0, 1e-3
    vtrue, vsmooth = layered_fault_model(nz, nx, dx, dx)
    w, _ = ws.ricker_wavelet(8.0, dt, 0.3)
    nt = len(w)
    rec_ix = np.arange(nx)
    solver = ws.WaveSolver2D(nx=nx, nz=nz, dx=dx, dz=dx, dt=dt, n_sponge=10)
    rec, snaps = solver.forward_propagate_acoustic(vtrue, w, 20, 2, rec_ix, 2, True, 3)
    lp.update(vtrue=vtrue, vsmooth=vsmooth, wavelet=w, fwd_rec=rec, fwd_snaps=snaps)
    lp["grid"] = np.array([nx, nz, dx, dt, 10, 0.0015, 1])

    # backward + imaging into a non-zero image (the image is accumulated in place)
    _, snaps_s = solver.forward_propagate_acoustic(vsmooth, w, 20, 2, rec_ix, 2, True, 3)
    image0 = rng.standard_normal((nz, nx)).astype(np.float32) * 1e-20
    image = image0.copy()
    solver.backward_propagate_and_correlate(vsmooth, rec, rec_ix, 2, snaps_s, image, 3)
    lp.update(bwd_image0=image0, bwd_image=image)

    # parity quirks: source in a never-written edge cell, receivers at the edges,
    # duplicated receivers, receivers in free-surface row 1
    rq = np.array([0, 1, 5, 5, 62, 63, 30, 0], dtype=int)
    rec_q, snaps_q = solver.forward_propagate_acoustic(vtrue, w[:120], 0, 2, rq, 2, True, 1)
    lp.update(q_rec_ix=rq, q_fwd_rec=rec_q, q_fwd_snaps=snaps_q[::7])
    rec_r1, _ = solver.forward_propagate_acoustic(vtrue, w[:120], 31, 1, rq, 1, False, 1)
    lp.update(q_row1_rec=rec_r1)
    img_q = np.zeros((nz, nx), dtype=np.float32)
    solver.backward_propagate_and_correlate(vsmooth, rec_q, rq, 2, snaps_q, img_q, 1)
    lp.update(q_bwd_image=img_q)

    # no free surface
    s2 = ws.WaveSolver2D(nx=nx, nz=nz, dx=dx, dz=dx, dt=dt, n_sponge=10, free_surface_top=False)
    rec_nf, snaps_nf = s2.forward_propagate_acoustic(vtrue, w, 33, 6, rec_ix, 4, True, 5)
    lp.update(nofs_rec=rec_nf, nofs_snaps=snaps_nf)

    # migrate_shot and migrate_multiple_shots
    eng = re.TSWRTMEngine(solver)
    fm = vf.FloodModels(true_model=vtrue, sediment_flood=vsmooth, rock_flood=vsmooth,
                        flood_line_sed=0, flood_line_rock=0)
    img1, ill1 = eng.migrate_shot(fm, w, 20, 2, rec, rec_ix, 2, 2)
    lp.update(ms_image=img1, ms_illum=ill1)
    six = [12, 32, 52]
    gathers = [solver.forward_propagate_acoustic(vtrue, w, s, 2, rec_ix, 2)[0] for s in six]
    res = eng.migrate_multiple_shots(fm, [w] * 3, six, [2] * 3, gathers, rec_ix, 2, 2, True)
    lp.update(mm_src_ix=np.array(six), mm_gathers=np.stack(gathers), mm_raw=res.raw_image,
              mm_lap=res.laplacian_image, mm_norm=res.normalized_image)
    # flood-model construction consumed by migrate_shot (velocity_flood.py:24-94)
    fl = vf.generate_velocity_flood_models(vtrue, 30, True, 6, 0.1, -0.05)
    lp.update(flood_sed=fl.sediment_flood, flood_rock=fl.rock_flood)
    np.savez_compressed(os.path.join(OUT, "golden_loops.npz"), **lp)
    for f in sorted(os.listdir(OUT)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(OUT, f)))


if __name__ == "__main__":
    main()
