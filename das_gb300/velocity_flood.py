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
