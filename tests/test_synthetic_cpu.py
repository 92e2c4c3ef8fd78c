"""The seeded synthetic inputs stand in for the benchmark configurations: their grids,
models, acquisition and wavelets must have the stated shapes, sizes and values (CPU).

* 150 x 400, dx 10 m: vp 1500 m/s at the surface rising linearly to 3000 m/s at depth,
  a 200 m +400 m/s layer at 700 m, offset by 100 m across a 60-degree fault; migration
  model the true one smoothed with sigma 5 cells; 20 sources every 20 columns, 400
  receivers; 3 Hz Ricker, dt 1 ms, nt 2000; 40-cell sponge.
* 1000 x 4000, dx 2.5 m: the same model scaled to depth plus two faults of dip in
  [45, 75] degrees; 200 sources evenly spaced, 4000 receivers; 6 Hz Ricker, dt 0.25 ms,
  nt 8000; reproducible from the seed.
"""
import numpy as np
import pytest

from das_gb300.synthetic import plain_large, plain_small


def test_small_configuration():
    sv = plain_small()
    assert (sv.nz, sv.nx, sv.dx, sv.dz, sv.dt, sv.nt) == (150, 400, 10.0, 10.0, 1e-3, 2000)
    assert (sv.n_sponge, sv.f0, sv.src_iz, sv.rec_iz) == (40, 3.0, 2, 2)
    assert list(sv.src_ix) == list(range(10, 400, 20)) and list(sv.rec_ix) == list(range(400))
    v = sv.vel_true.astype(np.float64)
    z = np.arange(150) * 10.0
    background = 1500.0 + 1500.0 * z / z[-1]
    # far from the layer the model is the linear gradient, 1500 at the top, 3000 at depth
    assert np.allclose(v[:, 0][z < 600], background[z < 600], atol=1e-3)
    assert v[0, 0] == pytest.approx(1500.0) and v[-1, 0] == pytest.approx(3000.0)
    # the +400 layer: 200 m thick from 700 m on the footwall (left), 100 m deeper on the
    # hanging wall (right of the 60-degree fault through the middle of the line)
    anomaly = v - background[:, None]
    left, right = anomaly[:, 5], anomaly[:, 395]
    assert np.allclose(left[(z >= 700) & (z < 900)], 400.0, atol=1e-3)
    assert np.allclose(left[(z < 700) | (z >= 900)], 0.0, atol=1e-3)
    assert np.allclose(right[(z >= 800) & (z < 1000)], 400.0, atol=1e-3)
    assert np.allclose(right[(z < 800) | (z >= 1000)], 0.0, atol=1e-3)
    # the fault dips 60 degrees: the layer's offset column moves by dz / tan(60) per metre
    xs = 0.5 * 399 * 10.0
    # (rows 70-79: the layer on the footwall only; rows 90-99: on the hanging wall only)
    for iz, left_v, right_v in ((70, 400.0, 0.0), (75, 400.0, 0.0), (90, 0.0, 400.0),
                                (95, 0.0, 400.0)):
        x_fault = xs + z[iz] / np.tan(np.deg2rad(60.0))
        ix = int(np.floor(x_fault / 10.0))
        assert anomaly[iz, ix - 1] == pytest.approx(left_v, abs=1e-3)
        assert anomaly[iz, ix + 2] == pytest.approx(right_v, abs=1e-3)
    # the migration model is the true one smoothed: same mean, smaller variation
    assert sv.vel_mig.dtype == np.float32 and sv.vel_mig.shape == (150, 400)
    assert abs(sv.vel_mig.mean() - v.mean()) < 1.0
    assert np.abs(np.diff(sv.vel_mig, axis=0)).max() < np.abs(np.diff(v, axis=0)).max()
    # 3 Hz Ricker: peak at t0 = 1 / f0
    assert int(np.argmax(sv.wavelet)) == round(1.0 / 3.0 / 1e-3)


def test_large_configuration_and_seed():
    sv = plain_large(nt=8000)
    assert (sv.nz, sv.nx, sv.dx, sv.dt, sv.nt) == (1000, 4000, 2.5, 2.5e-4, 8000)
    assert (sv.n_sponge, sv.f0, len(sv.src_ix), len(sv.rec_ix)) == (40, 6.0, 200, 4000)
    assert np.all(np.diff(sv.src_ix) == 20) and sv.src_ix[0] == 10
    v = sv.vel_true
    assert v.min() >= 1500.0 - 1e-3 and v.max() <= 3400.0 + 1e-3
    faults = sv.meta["faults"]
    assert len(faults) == 3 and faults[0][1] == 60.0
    assert all(45.0 <= f[1] <= 75.0 for f in faults[1:])
    again = plain_large(nt=8000)
    np.testing.assert_array_equal(again.vel_true, v)
    assert again.meta["faults"] == faults
    other = plain_large(seed=1, nt=8000)
    assert other.meta["faults"] != faults
    assert int(np.argmax(sv.wavelet)) == round(1.0 / 6.0 / 2.5e-4)


def test_batched_gathers_configuration():
    """256 uneven gathers: nx in [400, 2000], nz in [200, 600], dx 5 m, nt in [1500, 4000],
    3-5 Hz Ricker, smoothed layered models with 1-3 faults within vp 1500-3500 m/s; dt
    0.5 ms keeps the CFL number at or below 0.5."""
    from das_gb300.synthetic import batched_gathers
    gs = batched_gathers(256, seed=0)
    assert len(gs) == 256
    for g in gs:
        assert 400 <= g.nx <= 2000 and 200 <= g.nz <= 600 and 1500 <= g.nt <= 4000
        assert g.dx == 5.0 and g.dt == 5e-4 and 3.0 <= g.f0 <= 5.0
        assert g.vel.shape == (g.nz, g.nx) and g.vel.dtype == np.float32
        assert g.vel.min() >= 1500.0 and g.vel.max() <= 3500.0
        assert 40 <= g.src_ix < g.nx - 40
        cfl = float(g.vel.max()) * g.dt * np.sqrt(2.0) / g.dx
        assert cfl <= 0.5
    # uneven, and reproducible from the seed
    assert len({(g.nz, g.nx, g.nt) for g in gs}) > 200
    again = batched_gathers(256, seed=0)
    assert all(np.array_equal(a.vel, b.vel) for a, b in zip(gs[:8], again[:8]))


def test_elastic_fault_zone_configuration():
    """1024 x 2048, dx 2 m: vs 300 -> 1200 m/s with depth, a 20 m low-velocity zone dipping
    70 degrees; vp = 1.73 vs and density from Gardner's relation (rho = 310 vp^0.25)."""
    torch = pytest.importorskip("torch")
    from das_gb300.elastic import gardner_parameters
    from das_gb300.synthetic import elastic_fault_zone
    vs = elastic_fault_zone()
    assert vs.shape == (1024, 2048) and vs.dtype == np.float32
    assert vs[0, 0] == pytest.approx(300.0) and vs[-1, 0] == pytest.approx(1200.0)
    z = np.arange(1024) * 2.0
    background = 300.0 + 900.0 * z / z[-1]
    slow = vs < background[:, None] - 1e-3
    # the zone: 70 % of the background, about 20 m wide across the dip
    assert np.allclose(vs[slow], 0.7 * np.broadcast_to(background[:, None], vs.shape)[slow],
                       rtol=1e-6)
    widths = slow.sum(axis=1) * 2.0 * np.sin(np.deg2rad(70.0))
    assert np.all((widths[:900] > 14.0) & (widths[:900] < 26.0))
    # it dips 70 degrees: its centre moves by dz / tan(70) to the right per metre of depth
    cols = [np.mean(np.nonzero(slow[iz])[0]) for iz in (100, 500, 900)]
    slope = (cols[2] - cols[0]) * 2.0 / (z[900] - z[100])
    assert slope == pytest.approx(1.0 / np.tan(np.deg2rad(70.0)), rel=0.02)
    lam, mu, bx, bz = gardner_parameters(torch.tensor(vs[:4, :4].astype(np.float64)))[:4]
    vp = 1.73 * vs[:4, :4].astype(np.float64)
    rho = 310.0 * vp ** 0.25
    np.testing.assert_allclose(mu.numpy(), rho * vs[:4, :4] ** 2, rtol=1e-6)
    np.testing.assert_allclose(lam.numpy(), rho * vp * vp - 2.0 * rho * vs[:4, :4] ** 2, rtol=1e-6)
