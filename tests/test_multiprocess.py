"""The N > 1 path on CPU: two gloo ranks, no GPU.

Each rank encodes its share (whole textures, or block rows of one texture)
with the oracle standing in for its GPU, the shares are gathered, and the
union must equal a single-process encode byte for byte -- the sharding is
exact and leaves no gaps or overlaps.  The timing max-reduce is checked too.
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from astc_encoder_gb300 import shard


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _texture(h, w, seed):
    rng = np.random.default_rng(seed)
    img = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    img[h // 3:, : w // 2] = (5, 150, 250, 128)
    return img


def _worker(rank, world, port, out_dir):
    import torch
    import torch.distributed as dist
    from oracle import oracle
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        # (1) block rows of one 6x6 texture with clamp border, height not a multiple of 6
        img = _texture(125, 77, 1)
        r0, r1, _, _ = shard.block_row_slice(img.shape[0], 6, world, rank)
        part = shard.encode_rows(oracle.encode, img, r0, r1, 6, has_alpha=True, srgb=True, border=1)
        parts = [None] * world
        dist.all_gather_object(parts, (r0, r1, part))
        # (2) whole textures
        mine = {i: oracle.encode(_texture(40 + i, 30 + 2 * i, i), block_dim=4)
                for i in shard.shard_textures(7, world, rank)}
        all_tex = [None] * world
        dist.all_gather_object(all_tex, mine)
        # (3) timing reduce
        m = shard.max_over_ranks(float(rank + 1), dist)
        if rank == 0:
            np.save(os.path.join(out_dir, "rows.npy"), np.concatenate([p[2] for p in sorted(parts)]))
            merged = {}
            for d in all_tex:
                merged.update(d)
            np.save(os.path.join(out_dir, "tex.npy"), np.concatenate([merged[i] for i in range(7)]))
            np.save(os.path.join(out_dir, "max.npy"), np.array([m]))
    finally:
        dist.destroy_process_group()


def test_shard_range_covers_everything():
    for n in (0, 1, 5, 341, 342):
        for world in (1, 2, 3, 8):
            spans = [shard.shard_range(n, world, r) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            assert max(e - b for b, e in spans) - min(e - b for b, e in spans) <= 1


@pytest.mark.timeout(300)
def test_two_gloo_ranks_reassemble_exactly(tmp_path, oracle):
    port = _free_port()
    mp.spawn(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    img = _texture(125, 77, 1)
    want_rows = oracle.encode(img, block_dim=6, has_alpha=True, srgb=True, border=1)
    assert np.array_equal(np.load(tmp_path / "rows.npy"), want_rows)
    want_tex = np.concatenate([oracle.encode(_texture(40 + i, 30 + 2 * i, i), block_dim=4) for i in range(7)])
    assert np.array_equal(np.load(tmp_path / "tex.npy"), want_tex)
    assert np.load(tmp_path / "max.npy")[0] == 2.0
