"""Runs on several GPUs: one process per GPU (torchrun), no collective inside a launch.

Geodesics are independent, so a round shards by contiguous pixel-index ranges (or whole
images of a multi-image batch) with no exchange while it integrates. The one exchange
is the gather of the round's results before the mesh picks the next round
(Mesh::EndCurrentLoop needs every value of the round, Main.cpp:405-410): every rank
then updates an identical copy of the mesh, so no rank waits on another except there.
"""
import os

import numpy as np

from . import abi


def dist_env():
    """(rank, world size, local rank) from the torchrun environment; (0, 1, 0) alone."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard_range(n, rank, world):
    """Contiguous [lo, hi) of n units for `rank`; sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def shard_images(n_images, rank, world):
    """The image indices of `rank` when a multi-image batch is split by whole images."""
    lo, hi = shard_range(n_images, rank, world)
    return list(range(lo, hi))


def max_over_ranks(x, dist=None, device="cpu"):
    """The largest of every rank's x (step times: the job is as slow as its slowest rank)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sharded_round(px, integrate, rank, world, dist=None):
    """One mesh round split over the ranks: this rank integrates its contiguous slice of
    `px` with `integrate(slice) -> results`, then the slices are gathered so that every
    rank holds all len(px) results in pixel order (the input of Mesh::GeodesicFinished)."""
    lo, hi = shard_range(len(px), rank, world)
    mine = np.ascontiguousarray(integrate(px[lo:hi]), dtype=abi.RESULT_DTYPE)
    if world == 1 or dist is None:
        return mine
    parts = [None] * world
    dist.all_gather_object(parts, (lo, mine.tobytes()))
    out = np.zeros(len(px), dtype=abi.RESULT_DTYPE)
    for plo, buf in parts:
        part = np.frombuffer(buf, dtype=abi.RESULT_DTYPE)
        out[plo:plo + len(part)] = part
    return out


def sharded_run(mesh_specs, desc, integrate, rank, world, dist=None, on_round=None, waves=False, lookahead=0):
    """One FOORT run (Main.cpp:313-419) sharded over `world` ranks. Every rank holds an
    identical copy of the meshes, so every rank computes the same pixel list for a round;
    each rank integrates its contiguous slice with integrate(slice) -> results, the slices
    are gathered (sharded_round), and every rank hands the whole round's results to its
    meshes (Mesh::GeodesicFinished, Main.cpp:399) before they end the round
    (Mesh::EndCurrentLoop, Main.cpp:410). The gather is the run's only exchange, once per
    round. waves: the meshes' level waves are sharded and gathered instead (one exchange
    per wave) and the rounds replayed from their results (foort_gb300.run_by_waves, with
    `lookahead` the most pixels one sharded launch may hold, over all ranks).
    Returns the number of rounds; on_round(px, res) sees each whole round."""
    from . import run_by_waves, run_rounds
    shard = lambda px: sharded_round(px, integrate, rank, world, dist)  # noqa: E731
    if waves:
        return run_by_waves(mesh_specs, desc, shard, on_round, lookahead=lookahead)[0]
    return run_rounds(mesh_specs, desc, shard, on_round)

