"""Multi-GPU migration: shots sharded over ranks, one reduction of the image.

The reference migrates shots serially and stacks them (rtm_engine.py:125-143).
Shots are independent, so with one process per GPU each rank migrates its own
shots (round-robin by shot index) with no collective on the data path; one
reduction of the (nz, nx) stacked image and illumination follows, then the
post-stack steps (mute, normalisation, Laplacian: rtm_engine.py:145-171).

Two reductions:
* ``"ordered"`` sends every shot's image and illumination to rank 0 alone (point
  to point, as tensors, in shot order), which stacks them in the serial loop's
  order -- bit for bit the serial stack -- and broadcasts the one stacked pair to
  every rank;
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
        if world == 1:
            for k in range(n):  # the serial loop's addition order
                stacked += results[k][0]
                illum += results[k][1]
        else:
            stacked, illum = _ordered_stack(dist, rank, world, n, results, shape)
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


def _ordered_stack(dist, rank: int, world: int, n: int, results: dict, shape):
    """Stack every shot's (image, illumination) in shot order on rank 0, then broadcast.

    Shot k lives on rank k % world.  Each rank sends its shots to rank 0 in
    increasing k; rank 0 receives them in that order too, so it never holds more
    than one remote pair at a time, and adds them in the serial loop's order.  One
    broadcast of the stacked pair follows.  Traffic: every remote shot once to rank
    0, then one (2, nz, nx) tensor to each rank.
    """
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    stacked = np.zeros(shape, np.float32)
    illum = np.zeros(shape, np.float32)
    buf = torch.empty((2,) + tuple(shape), dtype=torch.float32, device=dev)
    for k in range(n):
        owner = k % world
        if rank == 0:
            if owner == 0:
                a, b = results[k]
            else:
                dist.recv(buf, src=owner)
                pair = buf.cpu().numpy()
                a, b = pair[0], pair[1]
            stacked += np.asarray(a, np.float32)
            illum += np.asarray(b, np.float32)
        elif owner == rank:
            a, b = results[k]
            buf.copy_(torch.from_numpy(np.stack([np.asarray(a, np.float32),
                                                 np.asarray(b, np.float32)])))
            dist.send(buf, dst=0)
    out = torch.from_numpy(np.stack([stacked, illum])).to(dev)
    dist.broadcast(out, src=0)
    out = out.cpu().numpy()
    return out[0].copy(), out[1].copy()
