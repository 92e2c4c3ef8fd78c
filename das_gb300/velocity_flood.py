"""Velocity-flood models, the input type of ``TSWRTMEngine.migrate_shot``.

Same fields and construction as tsw_rtm/velocity_flood.py:15-94 (Li et al. 2020
lateral flooding): the sediment flood repeats the column at the sediment flood
line across the rock side, the rock flood repeats the column at the rock flood
line across the sediment side, then optional fractional perturbations.  Cheap
host-side input construction (numpy), kept here so the engine can be used
without the reference package.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class FloodModels:
    true_model: np.ndarray
    sediment_flood: np.ndarray
    rock_flood: np.ndarray
    flood_line_sed: int
    flood_line_rock: int


def generate_velocity_flood_models(base_model: np.ndarray, fault_x_idx: int,
                                   sediment_is_left: bool = True, flood_offset_cells: int = 15,
                                   perturb_sediment: float = 0.0,
                                   perturb_rock: float = 0.0) -> FloodModels:
    nz, nx = base_model.shape
    if sediment_is_left:
        line_sed = min(nx - 1, fault_x_idx - flood_offset_cells)
        line_rock = max(0, fault_x_idx + flood_offset_cells)
        sed_cols = np.where(np.arange(nx) < line_sed, np.arange(nx), line_sed)
        rock_cols = np.where(np.arange(nx) >= line_rock, np.arange(nx), line_rock)
    else:
        line_sed = max(0, fault_x_idx + flood_offset_cells)
        line_rock = min(nx - 1, fault_x_idx - flood_offset_cells)
        sed_cols = np.where(np.arange(nx) >= line_sed, np.arange(nx), line_sed)
        rock_cols = np.where(np.arange(nx) < line_rock, np.arange(nx), line_rock)
    # column gathers reproduce the reference's slice copies and per-column fill
    # loops; a negative flood line indexes from the end, as in the reference
    sed = np.array(base_model[:, _wrap(sed_cols, nx)], dtype=base_model.dtype)
    rock = np.array(base_model[:, _wrap(rock_cols, nx)], dtype=base_model.dtype)
    if perturb_sediment != 0.0:
        sed = sed * (1.0 + perturb_sediment)
    if perturb_rock != 0.0:
        rock = rock * (1.0 + perturb_rock)
    return FloodModels(true_model=base_model.copy(), sediment_flood=sed.astype(np.float32),
                       rock_flood=rock.astype(np.float32), flood_line_sed=line_sed,
                       flood_line_rock=line_rock)


def _wrap(cols: np.ndarray, nx: int) -> np.ndarray:
    return np.where(cols < 0, cols + nx, cols)


def generate_velocity_flood_models_on_device(base_model, fault_x_idx: int,
                                             sediment_is_left: bool = True,
                                             flood_offset_cells: int = 15,
                                             perturb_sediment: float = 0.0,
                                             perturb_rock: float = 0.0) -> FloodModels:
    """The flood models of a float32 CUDA tensor ``base_model`` (nz, nx), built on its
    device: the same values as ``generate_velocity_flood_models`` on the same float32
    base model.  The FloodModels fields are CUDA tensors (``true_model`` a copy of the
    base); a flood line outside the model raises IndexError as the reference does."""
    import ctypes
    import torch
    from . import _lib
    if not (isinstance(base_model, torch.Tensor) and base_model.is_cuda):
        raise TypeError("base_model must be a CUDA tensor")
    if base_model.dtype != torch.float32 or base_model.dim() != 2:
        raise TypeError("base_model must be a 2-D float32 tensor")
    base = base_model.detach().contiguous()
    nz, nx = base.shape
    sed = torch.empty_like(base)
    rock = torch.empty_like(base)
    lines = (ctypes.c_int * 2)()
    lib = _lib.load()
    with torch.cuda.device(base.device):
        stream = torch.cuda.current_stream(base.device).cuda_stream
        rc = lib.w2d_flood_models(base.data_ptr(), nz, nx, int(fault_x_idx),
                                  1 if sediment_is_left else 0, int(flood_offset_cells),
                                  float(perturb_sediment), float(perturb_rock), sed.data_ptr(),
                                  rock.data_ptr(), lines, ctypes.c_void_p(stream))
    if rc != 0:
        msg = lib.w2d_last_error()
        msg = msg.decode() if isinstance(msg, bytes) else str(msg)
        if "flood line" in msg:
            raise IndexError(msg)
        _lib.check(rc)
    return FloodModels(true_model=base.clone(), sediment_flood=sed, rock_flood=rock,
                       flood_line_sed=int(lines[0]), flood_line_rock=int(lines[1]))

