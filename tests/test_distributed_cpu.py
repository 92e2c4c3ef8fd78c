"""Shot sharding over ranks with one image reduction, on CPU ranks (gloo, world size 2).

The migration of each shot is the CPU oracle here (no GPU in this test); the
host logic under test -- sharding, the ordered gather that reproduces the
serial stack bit for bit, the all-reduce sum, post-stack on every rank -- is the
same code the GPU ranks run.
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from oracle import oracle as o


def _problem():
    nz, nx = 40, 64
    grid = o.Grid(nx, nz, 10.0, 10.0, 1e-3, 10, 0.0015, True)
    rng = np.random.default_rng(3)
    vel = rng.uniform(1800, 2600, (nz, nx)).astype(np.float32)
    w, _ = o.ricker_wavelet(15.0, grid.dt, 0.08)
    rix = np.arange(nx)
    six = [5, 20, 33, 47, 60]
    gathers = [o.forward_propagate_acoustic(grid, vel * 1.03, w, s, 2, rix, 2)[0] for s in six]
    return grid, vel, w, rix, six, gathers


def _worker(rank, world, port, reduce, out_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from das_gb300.distributed import migrate_multiple_shots_distributed, shard
    from das_gb300.velocity_flood import FloodModels
    grid, vel, w, rix, six, gathers = _problem()
    fm = FloodModels(vel, vel, vel, 0, 0)
    done = []

    def mig(k):
        done.append(k)
        return o.migrate_shot(grid, vel, vel, w, six[k], 2, gathers[k], rix, 2, 2)

    res = migrate_multiple_shots_distributed(None, fm, [w] * 5, six, [2] * 5, gathers, rix,
                                             reduce=reduce, migrate_fn=mig,
                                             post_stack_fn=lambda st, il: o.post_stack(grid, st, il))
    assert done == shard(5, rank, world)
    np.savez(out_path + f".{rank}.npz", raw=res.raw_image, lap=res.laplacian_image,
             norm=res.normalized_image)
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


@pytest.mark.parametrize("reduce", ["ordered", "sum"])
def test_two_rank_sharded_migration(tmp_path, reduce):
    out = str(tmp_path / "res")
    mp.spawn(_worker, args=(2, _free_port(), reduce, out), nprocs=2, join=True)
    grid, vel, w, rix, six, gathers = _problem()
    ref = o.migrate_multiple_shots(grid, vel, vel, [w] * 5, six, [2] * 5, gathers, rix, 2, 2)
    for r in range(2):
        got = np.load(out + f".{r}.npz")
        if reduce == "ordered":
            np.testing.assert_array_equal(got["raw"], ref.raw_image)
            np.testing.assert_array_equal(got["norm"], ref.normalized_image)
        else:
            assert o.rel_l2(got["raw"], ref.raw_image) < 1e-6
            assert o.rel_l2(got["lap"], ref.laplacian_image) < 1e-6
