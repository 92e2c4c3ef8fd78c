"""Differentiable acoustic modelling: RTM as the adjoint, behind torch.autograd.

``AcousticModeling.apply(vel, solver, wavelet, source_ix, source_iz, receiver_ix,
receiver_iz)`` returns the receiver traces (nt, n_rec) that
``WaveSolver2D.forward_propagate_acoustic`` would record in ``vel`` (the same
fused forward kernel), as a CUDA tensor.  Its backward runs the hand-written
adjoint kernel (``acoustic_adjoint_kernel``) over the forward wavefield
recomputed segment by segment from checkpoints, and returns dL/dvel: for a
least-squares misfit this is the velocity gradient, i.e. the adjoint-state
migration image of the data residual.

PyTorch is used only for this wrapper (tensors, autograd); the arithmetic runs
in ``libwave2d_cuda.so`` on the tensors' device memory.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .geometry import normalize_index, normalize_indices
from .wave_solver import WaveSolver2D


class AcousticModeling(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vel: torch.Tensor, solver: WaveSolver2D, wavelet, source_ix: int,
                source_iz: int, receiver_ix, receiver_iz: int = 2) -> torch.Tensor:
        if not vel.is_cuda or vel.dtype != torch.float32:
            raise TypeError("vel must be a float32 CUDA tensor")
        if tuple(vel.shape) != (solver.nz, solver.nx):
            raise ValueError(f"vel shape {tuple(vel.shape)} != {(solver.nz, solver.nx)}")
        w = np.ascontiguousarray(wavelet, dtype=np.float32).reshape(-1)
        rix = normalize_indices(receiver_ix, solver.nx, "receiver_ix")
        six = normalize_index(source_ix, solver.nx, "source_ix")
        siz = normalize_index(source_iz, solver.nz, "source_iz")
        riz = normalize_index(receiver_iz, solver.nz, "receiver_iz")
        v = vel.detach().contiguous()
        traces = torch.empty((len(w), len(rix)), dtype=torch.float32, device=vel.device)
        torch.cuda.current_stream(vel.device).synchronize()
        eng = solver._eng()
        _lib.check(solver._lib.w2d_fwi_forward(eng, v.data_ptr(), w.ctypes.data, len(w), six, siz,
                                               rix.ctypes.data, len(rix), riz, traces.data_ptr()))
        ctx.solver = solver
        ctx.shape = tuple(vel.shape)
        ctx.device = vel.device
        return traces

    @staticmethod
    def backward(ctx, grad_traces: torch.Tensor):
        solver = ctx.solver
        g = grad_traces.detach().to(torch.float32).contiguous()
        grad = torch.empty(ctx.shape, dtype=torch.float32, device=ctx.device)
        torch.cuda.current_stream(ctx.device).synchronize()
        _lib.check(solver._lib.w2d_fwi_gradient(solver._eng(), g.data_ptr(), grad.data_ptr()))
        return grad, None, None, None, None, None, None


def model_traces(vel: torch.Tensor, solver: WaveSolver2D, wavelet, source_ix, source_iz,
                 receiver_ix, receiver_iz=2) -> torch.Tensor:
    """Differentiable forward modelling (see AcousticModeling)."""
    return AcousticModeling.apply(vel, solver, wavelet, source_ix, source_iz, receiver_ix,
                                  receiver_iz)


def misfit_and_gradient(solver: WaveSolver2D, vel, wavelet, source_ix, source_iz, receiver_ix,
                        receiver_iz, observed):
    """J = 0.5 * ||d(vel) - observed||^2 and dJ/dvel (numpy in, numpy out)."""
    v = torch.tensor(np.asarray(vel, dtype=np.float32), device="cuda", requires_grad=True)
    d_obs = torch.tensor(np.asarray(observed, dtype=np.float32), device="cuda")
    d = model_traces(v, solver, wavelet, source_ix, source_iz, receiver_ix, receiver_iz)
    J = 0.5 * torch.sum((d - d_obs) ** 2)
    J.backward()
    return float(J.item()), v.grad.detach().cpu().numpy()
