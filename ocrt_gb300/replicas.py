"""Multi-GPU use of the solve path: replicas only.

Pixels (and wavelengths of a pixel list) are independent problems with no
exchange step, so several GPUs simply split a pixel list: each rank solves a
contiguous shard on its own GPU and the per-pixel results are concatenated
in the original order.  The only collectives are on results and timings
(after the compute), never on the data path.  These helpers take any
`torch.distributed` process group (NCCL on GPUs, gloo on CPU).
"""
import numpy as np


def shard_bounds(n_items, rank, world):
    """[lo, hi) of rank's contiguous shard; shards differ in size by at most one."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad rank / world")
    base, extra = divmod(n_items, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def max_over_ranks(value, group=None):
    """Max of a scalar over the ranks (the timing rule of the bench)."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size(group) == 1:
        return float(value)
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def solve_sharded(solve, cases, opts, aerosols=None, group=None):
    """Solve this rank's shard with `solve(cases, opts, aerosols)` (a numpy
    structured array per pixel, e.g. ocrt_gb300.solve_batch) and return the
    whole list's results in order on every rank."""
    import torch.distributed as dist
    n = len(cases)
    if not dist.is_available() or not dist.is_initialized():
        return solve(cases, opts, aerosols)
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    lo, hi = shard_bounds(n, rank, world)
    per = lambda x: x[lo:hi] if isinstance(x, (list, tuple)) else x
    mine = solve(cases[lo:hi], per(opts), per(aerosols)) if hi > lo else None
    parts = [None] * world
    dist.all_gather_object(parts, mine, group=group)
    parts = [p for p in parts if p is not None]
    return np.concatenate(parts) if parts else None
