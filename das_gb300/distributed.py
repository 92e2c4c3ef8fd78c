"""Multi-GPU migration: shots sharded over ranks, one reduction of the image.

The reference migrates shots serially and stacks them (rtm_engine.py:125-143).
Shots are independent, so with one process per GPU each rank migrates its own
shots (round-robin by shot index) with no collective on the data path; one
reduction of the (nz, nx) stacked image and illumination follows, then the
post-stack steps (mute, normalisation, Laplacian: rtm_engine.py:145-171).

Two reductions:
* ``"ordered"`` gathers every shot's image and illumination on rank 0 and stacks
  them in shot order, reproducing the serial stack bit for bit;
* ``"sum"`` sums each rank's partial stack with one all-reduce (less traffic;
  float32 addition order differs from the serial loop, so equal within
  rounding).

``torch.distributed`` (NCCL between GPUs, gloo on CPU) is used only for the
reduction; the migration itself is the per-shot engine.
"""
from __future__ import annotations

from typing import Callable, List, Optional, Sequence

import numpy as np


def shard(n_shots: int, rank: int, world: int) -> List[int]:
    """Shot indices owned by `rank` (round-robin)."""
    return list(range(rank, n_shots, world))


def migrate_multiple_shots_distributed(engine, flood_models, source_waveforms: Sequence,
                                       source_coords_ix: Sequence[int],
                                       source_coords_iz: Sequence[int],
                                       receiver_gathers: Sequence, receiver_ix, receiver_iz=2,
                                       snapshot_interval=2, mute_sponge=True, reduce="ordered",
                                       migrate_fn: Optional[Callable] = None,
                                       post_stack_fn: Optional[Callable] = None):
    """Distributed ``TSWRTMEngine.migrate_multiple_shots``; every rank returns the result.

    migrate_fn(k) -> (image, illumination) of shot k defaults to
    ``engine.migrate_shot`` with the shot's arguments; post_stack_fn(stacked,
    illum) defaults to the engine's post-stack.
    """
    import torch
    import torch.distributed as dist

    rank = dist.get_rank() if dist.is_initialized() else 0
    world = dist.get_world_size() if dist.is_initialized() else 1
    n = len(source_coords_ix)
    if migrate_fn is None:
        def migrate_fn(k):
            return engine.migrate_shot(flood_models, source_waveforms[k], source_coords_ix[k],
                                       source_coords_iz[k], receiver_gathers[k], receiver_ix,
                                       receiver_iz, snapshot_interval)
    if post_stack_fn is None:
        from .rtm_engine import post_stack

        def post_stack_fn(stacked, illum):
            return post_stack(engine.solver, stacked, illum, mute_sponge)

    mine = shard(n, rank, world)
    results = {k: migrate_fn(k) for k in mine}
    shape = tuple(np.shape(flood_models.sediment_flood))
    stacked = np.zeros(shape, np.float32)
    illum = np.zeros(shape, np.float32)
    if reduce == "ordered":
        gathered = [results]
        if world > 1:
            gathered = [None] * world
            dist.all_gather_object(gathered, {k: (np.asarray(a), np.asarray(b))
                                              for k, (a, b) in results.items()})
        allres = {}
        for part in gathered:
            allres.update(part)
        for k in range(n):  # the serial loop's addition order
            stacked += allres[k][0]
            illum += allres[k][1]
    elif reduce == "sum":
        for k in mine:
            stacked += results[k][0]
            illum += results[k][1]
        if world > 1:
            t = torch.from_numpy(np.stack([stacked, illum]))
            if dist.get_backend() == "nccl":
                t = t.cuda()
            dist.all_reduce(t, op=dist.ReduceOp.SUM)
            t = t.cpu().numpy()
            stacked, illum = t[0].copy(), t[1].copy()
    else:
        raise ValueError("reduce must be 'ordered' or 'sum'")
    return post_stack_fn(stacked, illum)
