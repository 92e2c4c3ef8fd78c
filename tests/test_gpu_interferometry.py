"""Virtual-source gathers on the GPU against the reference's golden vectors.

Tolerances: the correlations are computed as direct sums (float32 samples, exact
products, double-float accumulation, one rounding to float32), while the reference
uses a float32 FFT; both are compared with the float64 correlation: ours must be
within 1e-7 relative L2 of it (float32 rounding is ~3e-8), and within 1e-6 of the
reference (its own FFT error is ~6e-8).  Where the reference's arithmetic is plain
float32 / float64 element work (np.gradient, branch averaging, interp1d) the GPU
result is bit-identical.  The frequency-domain derivative (a float32 FFT in the
reference, a float64 DFT here) agrees within 1e-5 relative L2.
"""
import numpy as np
import pytest

from oracle import interferometry_oracle as io

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def test_cross_correlation_golden(golden):
    from das_gb300.interferometry import compute_cross_correlation
    g = golden("interferometry")
    dt, lag = float(g["dt"]), float(g["max_lag"])
    for s in g["src"]:
        for k in range(3):
            c, lags = compute_cross_correlation(g[f"data{k}"], int(s), lag, dt, g["rec"])
            ex = io.correlation_exact(g[f"data{k}"], int(s), lag, dt, g["rec"])
            assert c.dtype == np.float32 and c.shape == g[f"ccf_s{s}_f{k}"].shape
            np.testing.assert_array_equal(lags, g["lags"])
            assert _rel(c, ex) < 1e-7
            assert _rel(c, g[f"ccf_s{s}_f{k}"]) < 1e-6
    c, lags = compute_cross_correlation(g["data2"][:300], 5, 0.5, dt)
    assert c.shape == g["ccf_all"].shape and _rel(c, g["ccf_all"]) < 1e-6
    np.testing.assert_array_equal(lags, g["lags_all"])
    # lag longer than half the FFT: the reference keeps wrapped rows; so does the GPU
    c, lags = compute_cross_correlation(g["data2"][:120], 7, 3.0, dt, g["rec"][:5])
    ex = io.correlation_exact(g["data2"][:120], 7, 3.0, dt, g["rec"][:5])
    assert c.shape == g["ccf_long"].shape == ex.shape
    assert _rel(c, ex) < 1e-7 and _rel(c, g["ccf_long"]) < 1e-5
    np.testing.assert_array_equal(lags, g["lags_long"])


def test_stack_over_windows_golden(golden):
    """All sources at once, three windows (one shorter), float32 stack then /= 3."""
    from das_gb300.interferometry import CrossCorrelationStack
    g = golden("interferometry")
    dt = float(g["dt"])
    st = CrossCorrelationStack(1500, g["data0"].shape[1], g["src"], g["rec"],
                               float(g["max_lag"]), dt)
    for k in range(3):
        st.add(g[f"data{k}"])
    res = st.result()
    for s in g["src"]:
        ex = [io.correlation_exact(g[f"data{k}"], int(s), float(g["max_lag"]), dt, g["rec"])
              for k in range(3)]
        # the float32 stack of the rounded exact correlations, to within float64 sum order
        np.testing.assert_array_max_ulp(res[int(s)][0],
                                        io.stack([e.astype(np.float32) for e in ex]), maxulp=2)
        assert _rel(res[int(s)][0], sum(ex) / 3.0) < 1e-7
        assert _rel(res[int(s)][0], g[f"stack_s{s}"]) < 1e-6
    st.close()


def test_stack_from_device_windows_equals_host_windows(golden):
    import torch
    from das_gb300.interferometry import CrossCorrelationStack
    g = golden("interferometry")
    dt = float(g["dt"])
    a = CrossCorrelationStack(1500, 96, g["src"], g["rec"], 2.0, dt)
    b = CrossCorrelationStack(1500, 96, g["src"], g["rec"], 2.0, dt)
    for k in range(2):
        a.add(g[f"data{k}"])
        b.add_device(torch.tensor(g[f"data{k}"], device="cuda"))
    ra, rb = a.result(), b.result()
    for s in ra:
        np.testing.assert_array_equal(ra[s][0], rb[s][0])


def test_derivatives_branches_resampling_golden(golden):
    from das_gb300.interferometry import (build_virtual_shot_gather, full_green_function,
                                          resample_gather_to_sim_dt, time_derivative_greens)
    g = golden("interferometry")
    dt = float(g["dt"])
    st = g[f"stack_s{int(g['src'][0])}"]
    np.testing.assert_array_equal(time_derivative_greens(st, dt), g["green_central"])
    np.testing.assert_array_equal(full_green_function(st, g["lags"]), g["green_full"])
    fr = time_derivative_greens(st, dt, scheme="frequency")
    assert _rel(fr, g["green_freq"]) < 1e-5
    coords = np.arange(96) * float(g["dx"])
    for b in ("causal", "anticausal", "symmetric"):
        for d in (True, False):
            vs = build_virtual_shot_gather(st, g["lags"], 0, int(g["src"][0]), coords, g["rec"], b,
                                           d)
            tag = f"{b}_{int(d)}"
            np.testing.assert_array_equal(vs.shot_gather, g[f"vs_{tag}_gather"])
            np.testing.assert_array_equal(vs.time_axis, g[f"vs_{tag}_time"])
            np.testing.assert_array_equal(vs.offsets, g[f"vs_{tag}_offsets"])
            assert vs.dt == float(g[f"vs_{tag}_dt"])
    for k in range(4):
        dts, nts = g[f"rs{k}_args"]
        out = resample_gather_to_sim_dt(g["vs_causal_1_gather"], dt, float(dts), int(nts))
        np.testing.assert_array_equal(out, g[f"rs{k}_out"])


def test_errors_are_raised_not_faulted():
    from das_gb300 import _lib
    from das_gb300.interferometry import (CrossCorrelationStack, compute_cross_correlation,
                                          time_derivative_greens)
    d = np.zeros((50, 8), np.float32)
    with pytest.raises(IndexError):
        compute_cross_correlation(d, 8, 0.1, 0.01)
    with pytest.raises(IndexError):
        compute_cross_correlation(d, 0, 0.1, 0.01, np.array([1, 9]))
    with pytest.raises(_lib.W2DError):
        time_derivative_greens(np.zeros((1, 3), np.float32), 0.01)
    st = CrossCorrelationStack(50, 8, [0], None, 0.1, 0.01)
    with pytest.raises(ValueError):
        st.add(np.zeros((51, 8), np.float32))
    with pytest.raises(_lib.W2DError):  # a much shorter window has other correlation rows
        st.add(np.zeros((4, 8), np.float32))
    st.close()
