"""Velocity-flood models built on the device (velocity_flood.py:24-94).

``generate_velocity_flood_models_on_device`` writes both flood models from a base
model already in device memory.  Checked bit for bit against the reference's own
output (golden) and against the oracle's restatement of its column loops over both
sides, negative flood lines and zero perturbations; a flood line past the model's
columns raises IndexError as the reference does.  A migration whose flood models
stay on the device equals the one that uploads them from the host, bit for bit.
"""
import numpy as np
import pytest

from oracle import oracle as o

pytestmark = pytest.mark.gpu

CASES = [(30, True, 6, 0.1, -0.05), (30, False, 6, 0.0, 0.2), (3, True, 10, -0.1, 0.0),
         (60, False, 2, 0.05, 0.05), (0, False, 0, 0.0, 0.0), (5, True, 9, 0.0, 0.0)]


def test_device_flood_models_bitwise(golden):
    import torch
    from das_gb300.velocity_flood import generate_velocity_flood_models_on_device
    g = golden("loops")
    base = torch.tensor(g["vtrue"], device="cuda")
    fl = generate_velocity_flood_models_on_device(base, 30, True, 6, 0.1, -0.05)
    np.testing.assert_array_equal(fl.sediment_flood.cpu().numpy(), g["flood_sed"])
    np.testing.assert_array_equal(fl.rock_flood.cpu().numpy(), g["flood_rock"])
    for args in CASES:
        fl = generate_velocity_flood_models_on_device(base, *args)
        sed, rock, ls, lr = o.generate_velocity_flood_models(g["vtrue"], *args)
        np.testing.assert_array_equal(fl.sediment_flood.cpu().numpy(), sed, err_msg=str(args))
        np.testing.assert_array_equal(fl.rock_flood.cpu().numpy(), rock, err_msg=str(args))
        assert (fl.flood_line_sed, fl.flood_line_rock) == (ls, lr)
        assert torch.equal(fl.true_model, base)
    with pytest.raises(IndexError):
        o.generate_velocity_flood_models(g["vtrue"], 90, True, 6)  # the reference's behaviour
    with pytest.raises(IndexError):
        generate_velocity_flood_models_on_device(base, 90, True, 6)


def test_migration_with_device_resident_models(golden):
    import torch
    from das_gb300.rtm_engine import TSWRTMEngine
    from das_gb300.velocity_flood import (generate_velocity_flood_models,
                                          generate_velocity_flood_models_on_device)
    from das_gb300.wave_solver import WaveSolver2D
    g = golden("loops")
    nx, nz, dx, dt, n, a, fs = g["grid"]
    s = WaveSolver2D(int(nx), int(nz), float(dx), float(dx), float(dt), int(n), float(a), bool(fs))
    eng = TSWRTMEngine(s)
    host = generate_velocity_flood_models(g["vsmooth"], 30, True, 6, 0.02, -0.03)
    dev = generate_velocity_flood_models_on_device(torch.tensor(g["vsmooth"], device="cuda"), 30,
                                                   True, 6, 0.02, -0.03)
    args = (g["wavelet"], 20, 2, g["fwd_rec"], np.arange(s.nx), 2, 2)
    img_h, ill_h = eng.migrate_shot(host, *args)
    img_d, ill_d = eng.migrate_shot(dev, *args)
    np.testing.assert_array_equal(img_d, img_h)
    np.testing.assert_array_equal(ill_d, ill_h)
    assert np.abs(img_h).max() > 0
    res_h = eng.migrate_multiple_shots(host, [g["wavelet"]] * 3, list(g["mm_src_ix"]), [2] * 3,
                                       list(g["mm_gathers"]), np.arange(s.nx), 2, 2)
    res_d = eng.migrate_multiple_shots(dev, [g["wavelet"]] * 3, list(g["mm_src_ix"]), [2] * 3,
                                       list(g["mm_gathers"]), np.arange(s.nx), 2, 2)
    np.testing.assert_array_equal(res_d.raw_image, res_h.raw_image)
    eng.close()
    s.close()
