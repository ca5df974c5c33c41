"""Orientation sharding and the cross-device reduction of search maps.

The whole-orientation search shards over orientation ranges with no exchange
until the end: each device folds its own range into its own four maps (MIP,
best global index, sum, sum of squares).  The one exchange step is the
reduction of those maps, restated from Leopard-EM's
``aggregate_distributed_results`` (backend/process_results.py:7-64): the
element-wise maximum of the MIPs with the index taken from the first device
that holds the maximum (``np.argmax`` returns the first occurrence, so ties go
to the lowest rank), and element-wise sums of the sums and squared sums.

The reference gathers every rank's maps to rank 0 with ``dist.gather``
(core_match_template_distributed.py:327-342) and reduces them there on the
host; ``gather_search_maps`` does the same over any ``torch.distributed``
backend (``gloo`` on CPU tensors, ``nccl`` on device tensors).
"""

from __future__ import annotations

import torch

MAP_KEYS = ("mip", "best_global_index", "correlation_sum", "correlation_squared_sum")


def orientation_shards(n_orientations: int, world_size: int, batch: int = 1) -> list[tuple[int, int]]:
    """Contiguous orientation ranges, one per rank, balanced to whole batches.

    Ranges are cut on multiples of ``batch`` where possible so that every rank
    but the last runs full orientation batches.
    """
    if n_orientations < 0 or world_size < 1 or batch < 1:
        raise ValueError("n_orientations >= 0, world_size >= 1 and batch >= 1 are required")
    n_batches = -(-n_orientations // batch)
    out = []
    for r in range(world_size):
        b0 = (n_batches * r) // world_size
        b1 = (n_batches * (r + 1)) // world_size
        out.append((min(n_orientations, b0 * batch), min(n_orientations, b1 * batch)))
    return out


def reduce_search_maps(shards: list[dict]) -> dict:
    """Reduce per-device maps in rank order (process_results.py:37-51).

    ``shards[r]`` holds the four maps of rank ``r`` (any device, same shapes).
    The MIP is the element-wise maximum; the best index comes from the lowest
    rank whose MIP equals it; sums and squared sums add up (in the sums' own
    dtype, FP64 here).
    """
    if not shards:
        raise ValueError("no shards to reduce")
    for s in shards:
        missing = [k for k in MAP_KEYS if k not in s]
        if missing:
            raise ValueError(f"shard is missing maps {missing}")
        if any(tuple(s[k].shape) != tuple(shards[0]["mip"].shape) for k in MAP_KEYS):
            raise ValueError("all maps of all shards must have the same shape")
    dev = shards[0]["mip"].device
    mip = shards[0]["mip"].to(dev).clone()
    best = shards[0]["best_global_index"].to(dev).clone()
    s1 = shards[0]["correlation_sum"].to(dev).clone()
    s2 = shards[0]["correlation_squared_sum"].to(dev).clone()
    for s in shards[1:]:
        m = s["mip"].to(dev)
        # strict '>' in rank order: the first rank that holds the maximum keeps it
        take = m > mip
        mip = torch.where(take, m, mip)
        best = torch.where(take, s["best_global_index"].to(dev, best.dtype), best)
        s1 = s1 + s["correlation_sum"].to(dev, s1.dtype)
        s2 = s2 + s["correlation_squared_sum"].to(dev, s2.dtype)
    return {"mip": mip, "best_global_index": best, "correlation_sum": s1, "correlation_squared_sum": s2}


def gather_search_maps(maps: dict, dst: int = 0, group=None) -> dict | None:
    """Gather every rank's maps to ``dst`` and reduce them there.

    Collective over ``group``: every rank must call it with maps of the same
    shapes and dtypes.  ``dst`` is a rank *within* ``group`` (for the default
    group, the global rank); the maps are reduced in group-rank order, so ties
    go to the lowest group rank.  Returns the reduced maps on ``dst`` and
    ``None`` on the other ranks.
    """
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized():
        raise RuntimeError("gather_search_maps needs an initialised torch.distributed process group")
    rank = dist.get_rank(group)
    world = dist.get_world_size(group)
    if not 0 <= dst < world:
        raise ValueError(f"dst={dst} is not a rank of the group (size {world})")
    # torch.distributed.gather takes the destination as a global rank
    dst_global = dist.get_global_rank(group, dst) if group is not None else dst
    gathered: dict[str, list[torch.Tensor] | None] = {}
    for k in MAP_KEYS:
        t = maps[k].contiguous()
        bufs = [torch.empty_like(t) for _ in range(world)] if rank == dst else None
        dist.gather(t, gather_list=bufs, dst=dst_global, group=group)
        gathered[k] = bufs
    if rank != dst:
        return None
    return reduce_search_maps([{k: gathered[k][r] for k in MAP_KEYS} for r in range(world)])
