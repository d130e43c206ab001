"""Env-range sharding across ranks (one process per GPU).

Environments never interact: every constraint, contact and BVH node belongs to exactly
one env (the reference partitions all arrays by ``vertexToEnv`` / ``triToEnv``,
``FF_SRL/FF_SRL/modelDO.py:991-992``). A multi-GPU job therefore gives each rank a
contiguous range of the env list and steps it on its own GPU with no exchange in the
step. The only cross-rank operations are host-side: the slowest rank's time for a
throughput figure, and an optional gather of per-env results.
"""

from __future__ import annotations


def env_range(num_envs: int, rank: int, world: int) -> tuple[int, int]:
    """[lo, hi) of the envs that ``rank`` owns: contiguous, sizes differing by at most one,
    lower ranks taking the remainder."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of {world}")
    if num_envs < 0:
        raise ValueError("num_envs must be >= 0")
    base, extra = divmod(num_envs, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def shard(items, rank: int, world: int):
    """The slice of a per-env list that ``rank`` owns."""
    lo, hi = env_range(len(items), rank, world)
    return items[lo:hi]


def _dist():
    try:
        import torch.distributed as dist
        return dist if dist.is_available() and dist.is_initialized() else None
    except Exception:
        return None


def max_over_ranks(value: float, device=None) -> float:
    """The maximum of ``value`` over all ranks (the value itself without a process group).
    ``device`` is where the reduction tensor lives: a CUDA device under NCCL, CPU under gloo."""
    dist = _dist()
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device=None) -> float:
    dist = _dist()
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def gather_env_results(local, num_envs: int, device=None):
    """Concatenates each rank's per-env result rows ([hi - lo, ...] tensors, in rank
    order) into the [num_envs, ...] array on every rank. Host-side metric gather only;
    nothing in the step calls it."""
    import torch
    dist = _dist()
    if dist is None:
        return local
    world = dist.get_world_size()
    sizes = [env_range(num_envs, r, world) for r in range(world)]
    rows = max(hi - lo for lo, hi in sizes)
    pad = torch.zeros((rows,) + tuple(local.shape[1:]), dtype=local.dtype, device=device or local.device)
    pad[: local.shape[0]] = local
    parts = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad)
    return torch.cat([p[: hi - lo] for p, (lo, hi) in zip(parts, sizes)])
