"""Query sharding for N independent GPU replicas.

Signed-distance and candidate queries are independent per query point, so
N GPUs each hold a replica of the mesh and its BVH and take a contiguous
range of the queries; nothing is exchanged on the data path.  The only
collective is gathering the per-rank results at the end, which a caller does
only if it needs all outputs on one rank.
"""
from __future__ import annotations


def shard_bounds(m: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous [lo, hi) range of m queries owned by `rank` of `world`."""
    if world < 1 or not (0 <= rank < world) or m < 0:
        raise ValueError("invalid shard request")
    base, extra = divmod(m, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def gather_shards(local, m: int, rank: int, world: int, group=None):
    """All-gather variable-sized 1-D shards into the full length-m result
    (torch.distributed; works with gloo on CPU and nccl on GPU tensors)."""
    import torch
    import torch.distributed as dist

    sizes = [shard_bounds(m, r, world)[1] - shard_bounds(m, r, world)[0] for r in range(world)]
    width = max(sizes)
    pad = torch.zeros(width, dtype=local.dtype, device=local.device)
    pad[: local.numel()] = local
    parts = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad, group=group)
    return torch.cat([p[:s] for p, s in zip(parts, sizes)])
