"""The forward modelling entry point that allocates no device memory.

For callers that cannot allocate device memory, w2d_forward_noalloc runs the
fused forward modelling on the caller's device buffers with its scratch in a
fixed file-scope device array.  Its traces must equal those of the allocating
path (WaveSolver2D.forward_propagate_acoustic -> w2d_forward) within the trace
tolerance used throughout the tests, on two calls in a row (the second call
must not see the first call's leftovers in the shared scratch).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TRACE_TOL = 1e-5


def _bind():
    import das_gb300
    lib = das_gb300.lib()
    fn = lib.w2d_forward_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                   ctypes.c_float, ctypes.c_float, ctypes.c_double, ctypes.c_int, ctypes.c_float,
                   ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                   ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    return lib, fn


def _rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_no_alloc_forward_matches_allocating_path_twice():
    import torch
    from das_gb300.wave_solver import WaveSolver2D, ricker_wavelet
    lib, fn = _bind()
    nz, nx, dx, dt, n_sp, alpha = 120, 300, 8.0, 8e-4, 25, 0.0015
    rng = np.random.default_rng(11)
    solver = WaveSolver2D(nx, nz, dx, dx, dt, n_sponge=n_sp, sponge_alpha=alpha)
    for call, (six, siz, n_rec) in enumerate([(150, 2, 280), (37, 4, 97)]):
        vel = rng.uniform(1600, 3000, (nz, nx)).astype(np.float32)
        w, _ = ricker_wavelet(10.0 + call, dt, 0.24)
        rix = np.sort(rng.integers(0, nx, size=n_rec)).astype(np.int32)
        want, _ = solver.forward_propagate_acoustic(vel, w, six, siz, rix, 3)
        v_d = torch.tensor(vel, device="cuda")
        w_d = torch.tensor(w, device="cuda")
        out_d = torch.full((len(w), n_rec), float("nan"), device="cuda")
        torch.cuda.synchronize()
        rc = fn(v_d.data_ptr(), w_d.data_ptr(), len(w), nx, nz, dx, dx, dt, n_sp, alpha, 1, six,
                siz, rix.ctypes.data, n_rec, 3, out_d.data_ptr(), None)
        assert rc == 0, lib.w2d_last_error()
        got = out_d.cpu().numpy()
        assert np.isfinite(got).all()
        assert _rel_l2(got, want) <= TRACE_TOL, f"call {call}"
        np.testing.assert_array_equal(got, want)


def test_no_alloc_rejects_oversized_grids():
    import torch
    lib, fn = _bind()
    nz, nx = 2048, 1024  # 2048 x 1024 pitched cells exceed the fixed scratch
    v_d = torch.ones((nz, nx), device="cuda")
    w_d = torch.zeros(8, device="cuda")
    out_d = torch.zeros((8, 4), device="cuda")
    rix = np.arange(4, dtype=np.int32)
    rc = fn(v_d.data_ptr(), w_d.data_ptr(), 8, nx, nz, 5.0, 5.0, 1e-4, 10, 0.0015, 1, 10, 2,
            rix.ctypes.data, 4, 2, out_d.data_ptr(), None)
    assert rc == 1 and b"scratch" in lib.w2d_last_error()


def test_no_alloc_refuses_host_memory():
    """A DEVICE argument that is host memory is refused with W2D_EINVAL before any
    work is queued.  The host buffer is page-locked, which the device could read
    through its mapping, so nothing could fault even if the check let it through;
    a following call with device buffers still succeeds."""
    import torch
    from das_gb300.pinned import pinned_array
    lib, fn = _bind()
    nz, nx, nt = 40, 64, 16
    host_vel = pinned_array((nz, nx))
    host_vel[...] = 2000.0
    w_d = torch.zeros(nt, device="cuda")
    out_d = torch.zeros((nt, 4), device="cuda")
    v_d = torch.full((nz, nx), 2000.0, device="cuda")
    rix = np.arange(4, dtype=np.int32)
    torch.cuda.synchronize()
    rc = fn(host_vel.ctypes.data, w_d.data_ptr(), nt, nx, nz, 5.0, 5.0, 5e-4, 10, 0.0015, 1, 10,
            2, rix.ctypes.data, 4, 2, out_d.data_ptr(), None)
    assert rc == 1 and b"not device memory" in lib.w2d_last_error()
    rc = fn(v_d.data_ptr(), w_d.data_ptr(), nt, nx, nz, 5.0, 5.0, 5e-4, 10, 0.0015, 1, 10, 2,
            rix.ctypes.data, 4, 2, out_d.data_ptr(), None)
    assert rc == 0, lib.w2d_last_error()
