"""Pin the CPU oracle against golden vectors produced by the reference itself.

The fixtures in tests/golden were made by tests/golden/make_golden.py, which runs
the reference's unchanged wave_solver.py / rtm_engine.py over its wave2d.c
compiled from source.  The float32 oracle must reproduce them bit for bit.
"""
import numpy as np
import pytest

from oracle import oracle as o


def test_sponge_bitwise(golden):
    g = golden("sponge")
    for k in range(4):
        nx, nz, n, a, fs = g[f"sponge{k}_args"]
        got = o.cerjan_sponge(int(nx), int(nz), int(n), float(a), bool(fs))
        np.testing.assert_array_equal(got, g[f"sponge{k}"])


@pytest.mark.parametrize("fs", [0, 1])
@pytest.mark.parametrize("use_sponge", [0, 1])
def test_acoustic_step_bitwise(golden, fs, use_sponge):
    g = golden("steps")
    nx, nz, dx, dz, dt = g["ac_args"]
    tag = f"ac_fs{fs}_sp{use_sponge}"
    out = g[f"{tag}_pn"].copy()
    o.acoustic_step(g[f"{tag}_pc"], g[f"{tag}_pp"], out, g[f"{tag}_vel"],
                    g[f"{tag}_sp"] if use_sponge else None, int(nx), int(nz), float(dx), float(dz),
                    float(dt), fs)
    np.testing.assert_array_equal(out, g[f"{tag}_out"])


@pytest.mark.parametrize("fs", [0, 1])
def test_elastic_step_bitwise(golden, fs):
    g = golden("steps")
    nx, nz, dx, dz, dt = g["el_args"]
    tag = f"el_fs{fs}"
    f = [g[f"{tag}_{n}_in"].copy() for n in ("vx", "vz", "sxx", "szz", "sxz")]
    o.elastic_step(*f, g[f"{tag}_lam"], g[f"{tag}_mu"], g[f"{tag}_bx"], g[f"{tag}_bz"],
                   g[f"{tag}_sp"], int(nx), int(nz), float(dx), float(dz), float(dt), fs)
    for name, a in zip(("vx", "vz", "sxx", "szz", "sxz"), f):
        np.testing.assert_array_equal(a, g[f"{tag}_{name}_out"], err_msg=name)


def test_correlate_bitwise(golden):
    g = golden("steps")
    out = g["corr_img"].copy()
    o.correlate(g["corr_src"], g["corr_rec"], out, 31, 29, 2e-3)
    np.testing.assert_array_equal(out, g["corr_out"])


def test_ricker_and_index_mapping(golden):
    g = golden("ricker")
    for k in range(3):
        f0, dt, T = g[f"args{k}"]
        w, t = o.ricker_wavelet(f0, dt, T)
        np.testing.assert_array_equal(w, g[f"w{k}"])
        np.testing.assert_array_equal(t, g[f"t{k}"])
    from das_gb300 import geometry
    np.testing.assert_array_equal(geometry.linspace_indices(35, 185, 7), g["map_src"])
    np.testing.assert_array_equal(geometry.linspace_indices(215, 365, 50), g["map_rec"])
    np.testing.assert_array_equal(geometry.halve_indices(g["map_half_in"]), g["map_half"])


def _grid(g):
    nx, nz, dx, dt, n, a, fs = g["grid"]
    return o.Grid(int(nx), int(nz), float(dx), float(dx), float(dt), int(n), float(a), bool(fs))


def test_forward_loop_bitwise(golden):
    g = golden("loops")
    grid = _grid(g)
    rec, snaps = o.forward_propagate_acoustic(grid, g["vtrue"], g["wavelet"], 20, 2,
                                              np.arange(grid.nx), 2, True, 3)
    np.testing.assert_array_equal(rec, g["fwd_rec"])
    np.testing.assert_array_equal(snaps, g["fwd_snaps"])


def test_backward_loop_bitwise(golden):
    g = golden("loops")
    grid = _grid(g)
    rix = np.arange(grid.nx)
    _, snaps = o.forward_propagate_acoustic(grid, g["vsmooth"], g["wavelet"], 20, 2, rix, 2,
                                            True, 3)
    image = g["bwd_image0"].copy()
    o.backward_propagate_and_correlate(grid, g["vsmooth"], g["fwd_rec"], rix, 2, snaps, image, 3)
    np.testing.assert_array_equal(image, g["bwd_image"])


def test_quirk_cases_bitwise(golden):
    g = golden("loops")
    grid = _grid(g)
    w = g["wavelet"][:120]
    rq = g["q_rec_ix"]
    rec, snaps = o.forward_propagate_acoustic(grid, g["vtrue"], w, 0, 2, rq, 2, True, 1)
    np.testing.assert_array_equal(rec, g["q_fwd_rec"])
    np.testing.assert_array_equal(snaps[::7], g["q_fwd_snaps"])
    rec1, _ = o.forward_propagate_acoustic(grid, g["vtrue"], w, 31, 1, rq, 1, False, 1)
    np.testing.assert_array_equal(rec1, g["q_row1_rec"])
    img = np.zeros((grid.nz, grid.nx), np.float32)
    _, snaps_s = o.forward_propagate_acoustic(grid, g["vtrue"], w, 0, 2, rq, 2, True, 1)
    o.backward_propagate_and_correlate(grid, g["vsmooth"], rec, rq, 2, snaps_s, img, 1)
    np.testing.assert_array_equal(img, g["q_bwd_image"])


def test_no_free_surface_bitwise(golden):
    g = golden("loops")
    grid = _grid(g)
    grid.free_surface_top = False
    rec, snaps = o.forward_propagate_acoustic(grid, g["vtrue"], g["wavelet"], 33, 6,
                                              np.arange(grid.nx), 4, True, 5)
    np.testing.assert_array_equal(rec, g["nofs_rec"])
    np.testing.assert_array_equal(snaps, g["nofs_snaps"])


def test_migrate_bitwise(golden):
    g = golden("loops")
    grid = _grid(g)
    rix = np.arange(grid.nx)
    img, ill = o.migrate_shot(grid, g["vsmooth"], g["vsmooth"], g["wavelet"], 20, 2,
                              g["fwd_rec"], rix, 2, 2)
    np.testing.assert_array_equal(img, g["ms_image"])
    np.testing.assert_array_equal(ill, g["ms_illum"])
    res = o.migrate_multiple_shots(grid, g["vsmooth"], g["vsmooth"], [g["wavelet"]] * 3,
                                   list(g["mm_src_ix"]), [2] * 3, list(g["mm_gathers"]), rix, 2, 2)
    np.testing.assert_array_equal(res.raw_image, g["mm_raw"])
    np.testing.assert_array_equal(res.laplacian_image, g["mm_lap"])
    np.testing.assert_array_equal(res.normalized_image, g["mm_norm"])


def test_f64_close_to_f32(golden):
    """The float64 run of the same loop agrees with the float32 golden to float32 accuracy."""
    g = golden("loops")
    grid = _grid(g)
    rec, snaps = o.forward_propagate_acoustic(grid, g["vtrue"], g["wavelet"], 20, 2,
                                              np.arange(grid.nx), 2, True, 3, precision="f64")
    assert o.rel_l2(g["fwd_rec"], rec) < 1e-4
    assert o.rel_l2(g["fwd_snaps"], snaps) < 1e-4


def test_flood_models_bitwise(golden):
    """The oracle's flood construction (velocity_flood.py:24-94, its loops restated)
    against the reference's own output, and the package's host port against the oracle
    over both sides, negative flood lines and zero perturbations."""
    g = golden("loops")
    sed, rock, _, _ = o.generate_velocity_flood_models(g["vtrue"], 30, True, 6, 0.1, -0.05)
    np.testing.assert_array_equal(sed, g["flood_sed"])
    np.testing.assert_array_equal(rock, g["flood_rock"])
    from das_gb300.velocity_flood import generate_velocity_flood_models
    base = g["vtrue"]
    for args in [(30, True, 6, 0.1, -0.05), (30, False, 6, 0.0, 0.2), (3, True, 10, -0.1, 0.0),
                 (60, False, 2, 0.05, 0.05), (0, False, 0, 0.0, 0.0), (5, True, 9, 0.0, 0.0)]:
        fl = generate_velocity_flood_models(base, *args)
        sed, rock, ls, lr = o.generate_velocity_flood_models(base, *args)
        np.testing.assert_array_equal(fl.sediment_flood, sed, err_msg=str(args))
        np.testing.assert_array_equal(fl.rock_flood, rock, err_msg=str(args))
        assert (fl.flood_line_sed, fl.flood_line_rock) == (ls, lr)
