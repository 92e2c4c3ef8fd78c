"""Elastic modelling and its adjoint gradient.

The elastic time loop, its vertical-force source, its vertical-strain receivers
and the gradient have no counterpart in the reference (it ships the elastic step
only), so they are checked against the oracle's loop around the reference step
(traces) and against central finite differences of the float64 oracle
(gradient with respect to the shear velocity, 16 random cells).
"""
import numpy as np
import pytest

from oracle import oracle as o

pytestmark = pytest.mark.gpu

NZ, NX, DX, DT = 40, 80, 5.0, 5e-4


def _model():
    z = np.arange(NZ)[:, None] + 0.0 * np.arange(NX)[None, :]
    vs = (300.0 + 900.0 * z / (NZ - 1)).astype(np.float32)
    vs_true = vs.copy()
    vs_true[18:24, 25:55] *= 0.8  # low-velocity zone
    return vs, vs_true


def _setup():
    import torch
    from das_gb300.elastic import ElasticSolver2D
    from das_gb300.wave_solver import ricker_wavelet
    w, _ = ricker_wavelet(12.0, DT, 0.15)
    # a unit force gives strains of ~1e-12 here, whose products with the adjoint
    # fields fall below float32's normal range; the modelling is linear in the
    # source, so scale it
    w = (w * 1e6).astype(np.float32)
    rix = np.arange(4, NX - 4)
    grid = o.Grid(NX, NZ, DX, DX, DT, 10, 0.003, True)
    solver = ElasticSolver2D(NX, NZ, DX, DX, DT, n_sponge=10, sponge_alpha=0.003)
    return torch, solver, grid, w, rix


def test_elastic_traces_match_oracle_loop():
    from das_gb300.elastic import elastic_traces
    torch, solver, grid, w, rix = _setup()
    vs, _ = _model()
    d = elastic_traces(torch.tensor(vs, device="cuda"), solver, w, 40, 3, rix, 2).cpu().numpy()
    lam, mu, bx, bz = (a.astype(np.float32) for a in o.gardner_parameters(vs, precision="f32"))
    ref = o.elastic_forward(grid, lam, mu, bx, bz, w, 40, 3, rix, 2)
    err = o.rel_l2(d, ref)
    print(f"elastic traces vs oracle loop: rel-L2 {err:.2e}")
    assert err < 1e-5


def test_elastic_gradient_matches_finite_differences():
    """dJ/dvs for J = sum(R * d(vs)) with fixed random weights R: the adjoint applied
    to R, compared with central differences of the float64 oracle (a misfit whose
    residual sat at float32 rounding level would test rounding, not the adjoint)."""
    from das_gb300.elastic import elastic_traces
    torch, solver, grid, w, rix = _setup()
    vs, _ = _model()
    R = np.random.default_rng(9).standard_normal((len(w), len(rix))).astype(np.float32)
    v = torch.tensor(vs, device="cuda", requires_grad=True)
    d = elastic_traces(v, solver, w, 40, 3, rix, 2)
    J = torch.sum(d * torch.tensor(R, device="cuda"))
    J.backward()
    g = v.grad.cpu().numpy()
    assert np.isfinite(g).all() and np.abs(g).max() > 0

    def J64(vs64):
        dd = o.elastic_forward(grid, *o.gardner_parameters(vs64), w, 40, 3, rix, 2,
                               precision="f64")
        return float(np.sum(dd * R))

    rng = np.random.default_rng(4)
    cells = [(int(rng.integers(1, 30)), int(rng.integers(14, 66))) for _ in range(16)]
    fd, an = [], []
    for iz, ix in cells:
        h = 1e-3 * float(vs[iz, ix])
        vp = vs.astype(np.float64).copy()
        vm = vp.copy()
        vp[iz, ix] += h
        vm[iz, ix] -= h
        fd.append((J64(vp) - J64(vm)) / (2 * h))
        an.append(float(g[iz, ix]))
    fd, an = np.array(fd), np.array(an)
    err = np.linalg.norm(an - fd) / np.linalg.norm(fd)
    print(f"elastic gradient vs central differences on 16 cells: rel-L2 {err:.2e}")
    for (iz, ix), a, f in zip(cells, an, fd):
        print(f"  cell ({iz},{ix}) adjoint {a:+.5e} finite-difference {f:+.5e}")
    assert err < 2e-2


def test_batch_of_shots_equals_single_shots():
    """Three shots with their own models, sources and wavelets advanced as one batch:
    traces and per-shot gradients bit-identical to running each shot alone."""
    from das_gb300.elastic import elastic_traces
    torch, solver, grid, w, rix = _setup()
    vs, vs_true = _model()
    models = [vs, vs_true, (vs * 1.05).astype(np.float32)]
    sources = [(20, 3), (40, 2), (61, 5)]
    waves = [w, (w * 0.5).astype(np.float32), np.roll(w, 7)]
    rng = np.random.default_rng(9)
    weights = [torch.tensor(rng.standard_normal((len(w), len(rix))).astype(np.float32),
                            device="cuda") for _ in range(3)]
    singles = []
    for m, (six, siz), wk, R in zip(models, sources, waves, weights):
        v = torch.tensor(m, device="cuda", requires_grad=True)
        d = elastic_traces(v, solver, wk, six, siz, rix, 2)
        (d * R).sum().backward()
        singles.append((d.detach().cpu().numpy(), v.grad.cpu().numpy()))
    vb = torch.tensor(np.stack(models), device="cuda", requires_grad=True)
    db = elastic_traces(vb, solver, np.stack(waves), [s[0] for s in sources],
                        [s[1] for s in sources], rix, 2)
    (db * torch.stack(weights)).sum().backward()
    for k in range(3):
        np.testing.assert_array_equal(db[k].detach().cpu().numpy(), singles[k][0])
        np.testing.assert_array_equal(vb.grad[k].cpu().numpy(), singles[k][1])


@pytest.mark.parametrize("nz,nx,free_surface", [(40, 80, True), (70, 300, False), (37, 261, True)])
def test_tiled_adjoint_equals_per_cell_adjoint(nz, nx, free_surface):
    """The TMA-tiled adjoint passes against the per-cell kernels on grids with several
    and ragged tiles, two shots: the same gradient to float32 rounding (the passes
    differ only in how the compiler contracts multiply-adds)."""
    import torch
    from das_gb300.elastic import ElasticSolver2D, elastic_traces
    from das_gb300.wave_solver import ricker_wavelet
    w, _ = ricker_wavelet(15.0, DT, 0.12)
    w = (w * 1e6).astype(np.float32)
    rng = np.random.default_rng(nx)
    z = np.arange(nz)[:, None] + 0.0 * np.arange(nx)[None, :]
    vs = (300.0 + 900.0 * z / (nz - 1)).astype(np.float32)
    models = np.stack([vs, (vs * 1.07).astype(np.float32)])
    rix = np.arange(2, nx - 2, 3)
    R = torch.tensor(rng.standard_normal((2, len(w), len(rix))).astype(np.float32), device="cuda")
    solver = ElasticSolver2D(nx, nz, DX, DX, DT, n_sponge=10, sponge_alpha=0.003,
                             free_surface_top=free_surface)
    grads = {}
    for form in ("cells", "tiled"):
        solver.set_adjoint(form)
        v = torch.tensor(models, device="cuda", requires_grad=True)
        d = elastic_traces(v, solver, np.stack([w, w]), [nx // 3, 2 * nx // 3], [3, 5], rix, 2)
        (d * R).sum().backward()
        grads[form] = v.grad.cpu().numpy().astype(np.float64)
    solver.close()
    a, b = grads["tiled"], grads["cells"]
    assert np.abs(b).max() > 0
    rel = np.linalg.norm(a - b) / np.linalg.norm(b)
    print(f"{nz} x {nx}: tiled vs per-cell adjoint rel L2 {rel:.2e}")
    assert rel < 1e-5


def test_tile_shapes_do_not_change_results():
    """Every supported step tile gives the same traces bit for bit (the step's float32
    operation order is fixed); every adjoint tile the same gradient to rounding."""
    from das_gb300.elastic import elastic_traces
    torch, solver, grid, w, rix = _setup()
    vs, _ = _model()
    R = torch.tensor(np.random.default_rng(4).standard_normal((len(w), len(rix))).astype(np.float32),
                     device="cuda")
    out = {}
    for step, adj in [((4, 2), (4, 1)), ((4, 4), (4, 2)), ((8, 2), (8, 1)), ((8, 1), (4, 2))]:
        solver.set_tiles(step, adj)
        v = torch.tensor(vs, device="cuda", requires_grad=True)
        d = elastic_traces(v, solver, w, 20, 3, rix, 2)
        (d * R).sum().backward()
        out[(step, adj)] = (d.detach().cpu().numpy(), v.grad.cpu().numpy().astype(np.float64))
    d0, g0 = out[((4, 2), (4, 1))]
    for k, (d, g) in out.items():
        np.testing.assert_array_equal(d, d0)
        assert np.linalg.norm(g - g0) <= 1e-6 * np.linalg.norm(g0), k
    with pytest.raises(Exception):
        solver.set_tiles((3, 3), (4, 2))


def test_programmatic_dependent_launch_does_not_change_results():
    """Step and tiled-adjoint kernels chained as programmatic dependents (default) and
    launched plainly: traces and gradients bit-identical, over several checkpoint
    segments (the copies between segments break the chain)."""
    from das_gb300.elastic import elastic_traces
    torch, solver, grid, w, rix = _setup()
    vs, _ = _model()
    R = torch.tensor(np.random.default_rng(5).standard_normal((len(w), len(rix))).astype(np.float32),
                     device="cuda")
    out = []
    for on in (True, False):
        solver.set_pdl(on)
        v = torch.tensor(np.stack([vs, vs * 1.03]).astype(np.float32), device="cuda",
                         requires_grad=True)
        d = elastic_traces(v, solver, np.stack([w, w]), [20, 50], [3, 4], rix, 2)
        (d * torch.stack([R, R])).sum().backward()
        out.append((d.detach().cpu().numpy(), v.grad.cpu().numpy()))
    solver.set_pdl(True)
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])


def test_shared_model_batch_equals_separate_copies():
    """Shots of one model: the batch stores the model once and every shot reads it
    (parameter stride 0); traces and per-shot gradients bit-identical to the batch with
    one copy per shot."""
    from das_gb300.elastic import elastic_traces
    torch, solver, grid, w, rix = _setup()
    vs, _ = _model()
    R = torch.tensor(np.random.default_rng(6).standard_normal((3, len(w), len(rix))).astype(
        np.float32), device="cuda")
    out = []
    for share in (True, False):
        solver.share_models = share
        v = torch.tensor(np.stack([vs, vs, vs]), device="cuda", requires_grad=True)
        d = elastic_traces(v, solver, np.stack([w, w * 0.5, w]), [15, 40, 60], [3, 3, 4], rix, 2)
        (d * R).sum().backward()
        out.append((d.detach().cpu().numpy(), v.grad.cpu().numpy()))
    solver.share_models = True
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
    assert not np.array_equal(out[0][1][0], out[0][1][1])  # per-shot gradients differ


def test_gradient_at_full_size_matches_finite_differences(capsys):
    """The elastic benchmark size: 1024 x 2048, dx 2 m, free surface, vs 300 -> 1200 m/s
    with a 20 m low-velocity zone dipping 70 degrees, vp = 1.73 vs, Gardner density,
    40-cell sponge, vertical-strain receivers on every interior column, 5 Hz Ricker at
    dt 0.2 ms -- cut to 600 steps (the wavelet taken from sample 700 on, so its main
    lobe, which peaks at sample 1000, falls inside the window).  dJ/dvs of
    J = sum(R * d) from the adjoint (checkpointed, through torch.autograd) against
    central differences on 16 random cells within reach of the source in 600 steps.
    The differences come from float32 GPU forward runs of the 32 perturbed models,
    advanced as one batch, with J summed in float64 on the host; the step (1 % of vs)
    sits far above float32 rounding of the traces and far below the model's scale."""
    import time
    import torch
    from das_gb300.elastic import ElasticSolver2D, elastic_traces
    from das_gb300.synthetic import elastic_fault_zone
    from das_gb300.wave_solver import ricker_wavelet
    t0 = time.perf_counter()
    nz, nx, d, dt, nt, first = 1024, 2048, 2.0, 2e-4, 600, 700
    vs = elastic_fault_zone(nz, nx, d)
    w_full, _ = ricker_wavelet(5.0, dt, 0.4)
    w = (w_full[first:first + nt] * 1e6).astype(np.float32)
    rix = np.arange(2, nx - 2)
    six, siz = nx // 2 - 300, 2
    solver = ElasticSolver2D(nx, nz, d, d, dt, n_sponge=40, sponge_alpha=0.0015)
    R = np.random.default_rng(21).standard_normal((nt, len(rix))).astype(np.float32)
    v = torch.tensor(vs, device="cuda", requires_grad=True)
    dd = elastic_traces(v, solver, w, six, siz, rix, 2)
    (dd * torch.tensor(R, device="cuda")).sum().backward()
    g = v.grad.cpu().numpy()
    assert np.isfinite(g).all() and np.abs(g).max() > 0
    rng = np.random.default_rng(5)
    cells = [(int(rng.integers(3, 16)), int(rng.integers(six - 16, six + 17))) for _ in range(16)]
    models = []
    hs = []
    for iz, ix in cells:
        h = 1e-2 * float(vs[iz, ix])
        hs.append(h)
        for sign in (1.0, -1.0):
            m = vs.copy()
            m[iz, ix] = np.float32(vs[iz, ix] + sign * h)
            models.append(m)
    fd = []
    with torch.no_grad():
        for b in range(0, len(models), 8):  # 4 cells (8 models) per batch
            part = models[b:b + 8]
            tr = elastic_traces(torch.tensor(np.stack(part), device="cuda"), solver, w,
                                [six] * len(part), [siz] * len(part), rix, 2).cpu().numpy()
            J = [float(np.sum(t.astype(np.float64) * R)) for t in tr]
            for k in range(0, len(part), 2):
                cell = (b + k) // 2
                # the perturbed values as float32 holds them
                step = float(models[b + k][cells[cell]]) - float(models[b + k + 1][cells[cell]])
                fd.append((J[k] - J[k + 1]) / step)
    fd = np.array(fd)
    an = np.array([float(g[c]) for c in cells])
    err = np.linalg.norm(an - fd) / np.linalg.norm(fd)
    solver.close()
    with capsys.disabled():
        print(f"\nelastic gradient 1024x2048 (600 steps) vs float32 central differences on 16 "
              f"cells: rel-L2 {err:.2e}; {time.perf_counter() - t0:.0f} s")
        for (iz, ix), a, f in zip(cells, an, fd):
            print(f"  cell ({iz},{ix}) adjoint {a:+.5e} finite-difference {f:+.5e}")
    assert err < 1e-2
