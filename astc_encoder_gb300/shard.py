"""Splitting encode work across ranks (one process per GPU).

ASTC blocks are independent, so the path shards without any exchange step:
a rank takes whole textures, or a contiguous range of block rows of one
texture, encodes them alone and owns the disjoint output bytes.  Collectives
are used only around the work (a barrier and a max-reduce of the elapsed time
for timing, or a gather when one rank wants every result).
"""
from __future__ import annotations

from typing import Any


def shard_range(n: int, world: int, rank: int) -> tuple[int, int]:
    """Contiguous [begin, end) share of n items for `rank` (sizes differ by <= 1)."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("bad world/rank")
    base, extra = divmod(n, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def shard_textures(count: int, world: int, rank: int) -> list[int]:
    b, e = shard_range(count, world, rank)
    return list(range(b, e))


def block_row_slice(height: int, block_dim: int, world: int, rank: int) -> tuple[int, int, int, int]:
    """Block rows [r0, r1) of a texture for `rank`, and the texel rows (y0, h) they read.

    Shard boundaries are block-aligned, so no block straddles two ranks and the
    border rule (zero or clamp) only ever applies at the texture's own edge.
    """
    nby = (height + block_dim - 1) // block_dim
    r0, r1 = shard_range(nby, world, rank)
    y0 = r0 * block_dim
    h = max(0, min(height, r1 * block_dim) - y0)
    return r0, r1, y0, h


def encode_rows(encode, img, r0: int, r1: int, block_dim: int, **opts):
    """Encodes block rows [r0, r1) of `img` (H, W, 4) with `encode(img_part, **opts)`."""
    y0 = r0 * block_dim
    y1 = min(img.shape[0], r1 * block_dim)
    if y1 <= y0:
        return img[:0].reshape(0, 16)
    return encode(img[y0:y1], block_dim=block_dim, **opts)


def max_over_ranks(value: float, dist: Any = None) -> float:
    """Max of a float over all ranks (identity without an initialised group)."""
    if dist is None:
        import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64)
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
