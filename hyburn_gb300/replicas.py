"""Sweep points sharded over processes, one GPU each.

Sweep points are independent (engine.rs:496-842 couples nodes, never points), so a sweep spreads
over ranks by giving each rank a contiguous block of points: every rank runs its own engine on its
block with no communication while stepping, and the results are gathered once at the end, in
rank order, into the layout one engine over all points would return. Noise shared by all points
is the same array on every rank; noise per point is split with the points. The batch-mean BOLD
monitor averages over all points before its nonlinear Balloon-Windkessel step (engine.rs:786-801),
so it cannot be assembled from shards: sharded runs use per-point BOLD (HB_SEM_BOLD_PER_POINT).
"""
from __future__ import annotations

from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _abi
from .config import Unsupported
from .engine import BatchSweepResult


def shard_bounds(n_points: int, rank: int, world: int) -> Tuple[int, int]:
    """[lo, hi) of the points of `rank`: contiguous blocks whose sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of world {world}")
    base, extra = divmod(n_points, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def shard_values(values: Sequence[float], rank: int, world: int) -> np.ndarray:
    lo, hi = shard_bounds(len(values), rank, world)
    return np.asarray(values, np.float32)[lo:hi]


def shard_noise(noise: Optional[np.ndarray], n_points: int, semantics: int, rank: int, world: int):
    """The noise rows of `rank`: the whole shared array, or its block of a per-point array
    [n_steps, n_points, row]."""
    if noise is None or not (semantics & _abi.HB_SEM_NOISE_PER_POINT):
        return noise
    lo, hi = shard_bounds(n_points, rank, world)
    a = np.asarray(noise, np.float32)
    return np.ascontiguousarray(a.reshape(a.shape[0], n_points, -1)[:, lo:hi])


def check_shardable(semantics: int, n_bold_monitors: int, world: int) -> None:
    if world > 1 and n_bold_monitors > 0 and not (semantics & _abi.HB_SEM_BOLD_PER_POINT):
        raise Unsupported("the batch-mean BOLD monitor needs all sweep points in one engine; "
                          "use HB_SEM_BOLD_PER_POINT when sharding points over ranks")


def merge_results(parts: List[BatchSweepResult], n_steps: int) -> BatchSweepResult:
    """Concatenate per-rank results (in rank order) into the result of one engine over all points."""
    n_sub = len(parts[0].tavg)
    tavg = [np.concatenate([np.asarray(p.tavg[i]).ravel() for p in parts]) for i in range(n_sub)]
    fin = [np.concatenate([np.asarray(p.final_states[i]).ravel() for p in parts]) for i in range(n_sub)]
    traj = None
    if parts[0].trajectories is not None:
        traj = []
        for i in range(n_sub):
            blocks = [np.asarray(p.trajectories[i]).reshape(n_steps, p.n_sweep, -1) for p in parts]
            traj.append(np.concatenate(blocks, axis=1).ravel())
    bold = None
    if parts[0].bold is not None:
        bold = [np.concatenate([np.asarray(p.bold[m]).ravel() for p in parts]) for m in range(len(parts[0].bold))]
    return BatchSweepResult(param_values=np.concatenate([np.asarray(p.param_values) for p in parts]),
                            tavg=tavg, final_states=fin, trajectories=traj, bold=bold,
                            elapsed_ms=max(p.elapsed_ms for p in parts), n_sweep=sum(p.n_sweep for p in parts))


def gather_result(local: BatchSweepResult, n_steps: int, group=None) -> BatchSweepResult:
    """All ranks' results merged on every rank (torch.distributed.all_gather_object)."""
    import torch.distributed as dist

    world = dist.get_world_size(group)
    parts: List[Optional[BatchSweepResult]] = [None] * world
    dist.all_gather_object(parts, local, group=group)
    return merge_results(parts, n_steps)


def max_over_ranks(x: float, group=None) -> float:
    """Maximum of a host value over all ranks (a timing taken on every rank)."""
    import torch
    import torch.distributed as dist

    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
