"""Seeded synthetic textures generated on the GPU (torch), for the batched
workloads whose inputs are too large to generate quickly on the host.

``mixed_batch`` builds the 256-texture workload: width and height drawn
log-uniformly from [64, 4096], 30% kept non-power-of-two and the rest rounded
to a power of two; formats 60% 4x4 RGB / 25% 6x6 RGBA sRGB (edge clamp) /
15% 4x4 normal map; content generated like synth.rgb_noise /
synth.rgba_cutout / synth.normal_map (same recipes, torch random streams);
each texture with its full box-filtered mip chain from the library's mip
kernel (sRGB textures filtered in linear light).
"""
from __future__ import annotations

import math

import numpy as np

from . import synth


def _value_noise(torch, h, w, period, gen):
    dev = "cuda"
    gy = torch.arange(h, device=dev, dtype=torch.float64) / period
    gx = torch.arange(w, device=dev, dtype=torch.float64) / period
    iy, ix = gy.floor().long(), gx.floor().long()
    fy, fx = (gy - iy).float(), (gx - ix).float()
    lat = torch.rand((int(iy[-1]) + 2, int(ix[-1]) + 2), generator=gen, device=dev)
    rows = lat[:, ix] * (1 - fx)[None, :] + lat[:, ix + 1] * fx[None, :]
    return rows[iy] * (1 - fy)[:, None] + rows[iy + 1] * fy[:, None]


def _octaves(torch, h, w, gen, periods, amps):
    acc = torch.zeros((h, w), device="cuda")
    for p, a in zip(periods, amps):
        acc += a * _value_noise(torch, h, w, p, gen)
    return acc


def _rgb(torch, h, w, gen, rng):
    out = torch.empty((h, w, 4), dtype=torch.uint8, device="cuda")
    for c in range(3):
        v = _octaves(torch, h, w, gen, (256, 64, 16, 4), (0.5, 0.25, 0.15, 0.1))
        out[..., c] = (v * 255.0).round().clamp(0, 255).to(torch.uint8)
    lo, hi = math.log(max(2.0, min(h, w) / 64.0)), math.log(max(4.0, min(h, w) / 4.0))
    for _ in range(32):
        rh, rw = int(math.exp(rng.uniform(lo, hi))), int(math.exp(rng.uniform(lo, hi)))
        y0, x0 = int(rng.integers(0, max(1, h - rh + 1))), int(rng.integers(0, max(1, w - rw + 1)))
        col = torch.tensor(rng.integers(0, 256, 3).tolist(), dtype=torch.uint8, device="cuda")
        out[y0:y0 + rh, x0:x0 + rw, :3] = col
    out[..., 3] = 255
    return out


def rgb_noise(torch, h, w, gen, rng):
    return _rgb(torch, h, w, gen, rng)


def rgba_cutout(torch, h, w, gen, rng):
    out = _rgb(torch, h, w, gen, rng)
    mask = (_value_noise(torch, h, w, 32, gen) >= 0.4).float()[None, None]
    k = torch.ones((1, 1, 1, 4), device="cuda") / 4.0
    m = torch.nn.functional.pad(mask, (2, 1, 0, 0), mode="replicate")
    m = torch.nn.functional.conv2d(m, k)
    m = torch.nn.functional.pad(m, (0, 0, 2, 1), mode="replicate")
    m = torch.nn.functional.conv2d(m, k.transpose(2, 3))
    out[..., 3] = (m[0, 0] * 255.0).round().clamp(0, 255).to(torch.uint8)
    return out


def normal_map(torch, h, w, gen, rng):
    periods = (512, 256, 128, 64, 32, 16)
    amps = tuple(0.5 ** i for i in range(6))
    height = _octaves(torch, h, w, gen, periods, amps) * (8.0 * 16.0 / sum(amps))
    p = torch.nn.functional.pad(height[None, None], (1, 1, 1, 1), mode="replicate")[0, 0]
    gx = ((p[:-2, 2:] + 2 * p[1:-1, 2:] + p[2:, 2:]) - (p[:-2, :-2] + 2 * p[1:-1, :-2] + p[2:, :-2])) / 8.0
    gy = ((p[2:, :-2] + 2 * p[2:, 1:-1] + p[2:, 2:]) - (p[:-2, :-2] + 2 * p[:-2, 1:-1] + p[:-2, 2:])) / 8.0
    inv = 1.0 / torch.sqrt(gx * gx + gy * gy + 1.0)
    out = torch.empty((h, w, 4), dtype=torch.uint8, device="cuda")
    for c, comp in enumerate((-gx * inv, -gy * inv, inv)):
        out[..., c] = ((comp + 1.0) * 127.5).round().clamp(0, 255).to(torch.uint8)
    out[..., 3] = 255
    return out


FORMATS = [
    ("4x4_rgb", 0.60, dict(block_dim=4, has_alpha=False, is_normal=False, srgb=False, border=0), rgb_noise),
    ("6x6_rgba_srgb", 0.25, dict(block_dim=6, has_alpha=True, is_normal=False, srgb=True, border=1),
     rgba_cutout),
    ("4x4_normal", 0.15, dict(block_dim=4, has_alpha=False, is_normal=True, srgb=False, border=0), normal_map),
]


def _size(rng) -> int:
    v = math.exp(rng.uniform(math.log(64), math.log(4096)))
    if rng.random() < 0.30:
        return int(round(v))
    return 1 << int(round(math.log2(v)))


def mixed_batch(torch, native, count: int = 256, seed: int = synth.SEED_BASE + 3, scale: float = 1.0):
    """List of textures: dicts with 'format', 'opts', 'levels' [(w, h, tensor)]."""
    rng = np.random.default_rng(seed)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    probs = [f[1] for f in FORMATS]
    out = []
    for _ in range(count):
        k = int(rng.choice(len(FORMATS), p=probs))
        name, _, opts, fn = FORMATS[k]
        w = max(1, int(_size(rng) * scale))
        h = max(1, int(_size(rng) * scale))
        base = fn(torch, h, w, gen, rng).contiguous()
        nlev = native.mip_levels(w, h)
        chain = torch.empty(max(4, native.mip_chain_bytes(w, h, nlev)), dtype=torch.uint8, device="cuda")
        native.generate_mips(base.data_ptr(), w, h, nlev, chain.data_ptr(), srgb=opts["srgb"],
                             stream=torch.cuda.current_stream().cuda_stream or None)
        levels = [(w, h, base)]
        off = 0
        for lw, lh in native.mip_sizes(w, h, nlev)[1:]:
            n = lw * lh * 4
            levels.append((lw, lh, chain[off:off + n].view(lh, lw, 4)))
            off += n
        out.append({"format": name, "opts": dict(opts), "levels": levels, "chain": chain})
    torch.cuda.synchronize()
    return out
