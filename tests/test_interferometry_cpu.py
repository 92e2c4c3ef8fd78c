"""Virtual-source gather generation on the CPU side: the oracle against the
reference's golden vectors (bit for bit), and the library's host-side row mapping
of the cross-correlation against the reference's slice semantics."""
import ctypes

import numpy as np
import pytest

from oracle import interferometry_oracle as io


def test_oracle_cross_correlation_and_stack_bitwise(golden):
    g = golden("interferometry")
    dt, lag = float(g["dt"]), float(g["max_lag"])
    for s in g["src"]:
        per = []
        for k in range(3):
            c, lags = io.cross_correlation(g[f"data{k}"], int(s), lag, dt, g["rec"])
            np.testing.assert_array_equal(c, g[f"ccf_s{s}_f{k}"])
            per.append(c)
        np.testing.assert_array_equal(lags, g["lags"])
        np.testing.assert_array_equal(io.stack(per), g[f"stack_s{s}"])
    c, lags = io.cross_correlation(g["data2"][:300], 5, 0.5, dt)
    np.testing.assert_array_equal(c, g["ccf_all"])
    np.testing.assert_array_equal(lags, g["lags_all"])
    c, lags = io.cross_correlation(g["data2"][:120], 7, 3.0, dt, g["rec"][:5])
    np.testing.assert_array_equal(c, g["ccf_long"])  # rows wrap: lag longer than the window
    np.testing.assert_array_equal(lags, g["lags_long"])


def test_oracle_exact_correlation_is_the_reference_up_to_fft_rounding(golden):
    g = golden("interferometry")
    dt = float(g["dt"])
    s = int(g["src"][0])
    ex = io.correlation_exact(g["data0"], s, float(g["max_lag"]), dt, g["rec"])
    ref = g[f"ccf_s{s}_f0"]
    err = np.linalg.norm(ref - ex) / np.linalg.norm(ex)
    assert err < 1e-6  # the reference's float32 FFT rounding
    assert np.linalg.norm(ex.astype(np.float32) - ex) / np.linalg.norm(ex) < err


def test_oracle_derivatives_branches_resampling_bitwise(golden):
    g = golden("interferometry")
    dt = float(g["dt"])
    st = g[f"stack_s{int(g['src'][0])}"]
    np.testing.assert_array_equal(io.gradient_central(st, dt), g["green_central"])
    np.testing.assert_array_equal(io.gradient_central(st, dt), g["green_full"])
    np.testing.assert_array_equal(io.derivative_frequency(st, dt), g["green_freq"])
    for b in ("causal", "anticausal", "symmetric"):
        for d in (True, False):
            gat, t = io.branch(io.gradient_central(st, dt) if d else st, g["lags"], b)
            np.testing.assert_array_equal(gat, g[f"vs_{b}_{int(d)}_gather"])
            np.testing.assert_array_equal(t, g[f"vs_{b}_{int(d)}_time"])
    for k in range(4):
        dts, nts = g[f"rs{k}_args"]
        out = io.resample_linear(g["vs_causal_1_gather"], dt, float(dts), int(nts))
        np.testing.assert_array_equal(out, g[f"rs{k}_out"])


@pytest.mark.parametrize("nt", [1, 2, 3, 7, 64, 65, 120, 1111, 1500, 4097])
def test_library_row_mapping_matches_slice_semantics(nt):
    from das_gb300 import _lib
    lib = _lib.load()
    for n_lags in (0, 1, 5, nt // 3, nt - 1, nt, nt + 3, 2 * nt + 9):
        lag0, rows = ctypes.c_int(), ctypes.c_int()
        assert lib.w2d_xcorr_rows(nt, n_lags, ctypes.byref(lag0), ctypes.byref(rows)) == 0
        want, _ = io.lag_rows(nt, n_lags * 0.01, 0.01)
        assert rows.value == len(want)
        if len(want):
            assert lag0.value == want[0]
            np.testing.assert_array_equal(np.arange(rows.value) + lag0.value, want)
