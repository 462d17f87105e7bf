"""Seeded synthetic RGBA8 textures for the encoder's workloads.

The reference ships one sample image and no benchmark data, so every
measurement runs on deterministic synthetic textures with documented shapes
and value distributions:

* ``rgb_noise``   -- per channel, 4 octaves of bilinear value noise (periods
  256/64/16/4 px, amplitudes 0.5/0.25/0.15/0.1) scaled to [0, 255], overlaid
  with 32 hard-edged axis-aligned rectangles of uniform random colour,
  alpha = 255.  (512x512 for the 4x4 RGB workload.)
* ``rgba_cutout`` -- the same RGB; alpha = value noise of period 32 px
  thresholded at 0.4 into {0, 255}, with a 4-px linear ramp across each
  alpha edge (a 4-wide box filter of the mask).  (2048x2048 for the 6x6 RGBA
  sRGB workload.)
* ``normal_map``  -- FBM height field (6 octaves, periods 512 -> 16 px,
  amplitudes halving, normalised to [0, 1], height scale 8 in units of the
  finest period, i.e. up to 128 px of relief) -> Sobel gradient -> unit normal;
  X/Y/Z mapped to [0, 255], alpha = 255.  (4096x4096 for the 4x4 normal-map
  workload; the encoder forces B = A = 255.)

Each generator takes a seed; the default seed of workload k is 20261203 + k.
"""
from __future__ import annotations

import numpy as np

SEED_BASE = 20261203


def value_noise(h: int, w: int, period: float, rng: np.random.Generator) -> np.ndarray:
    """Bilinear value noise in [0, 1): a random lattice every `period` px."""
    gy = np.arange(h, dtype=np.float64) / period
    gx = np.arange(w, dtype=np.float64) / period
    iy = np.floor(gy).astype(np.int64)
    ix = np.floor(gx).astype(np.int64)
    fy = (gy - iy).astype(np.float32)
    fx = (gx - ix).astype(np.float32)
    lat = rng.random((int(iy[-1]) + 2, int(ix[-1]) + 2), dtype=np.float32)
    rows = lat[:, ix] * (1.0 - fx)[None, :] + lat[:, ix + 1] * fx[None, :]
    return rows[iy] * (1.0 - fy)[:, None] + rows[iy + 1] * fy[:, None]


def _octaves(h: int, w: int, rng: np.random.Generator, periods, amps) -> np.ndarray:
    acc = np.zeros((h, w), np.float32)
    for p, a in zip(periods, amps):
        acc += np.float32(a) * value_noise(h, w, p, rng)
    return acc


def _rgb_layer(h: int, w: int, rng: np.random.Generator, rects: int = 32) -> np.ndarray:
    rgb = np.empty((h, w, 3), np.uint8)
    for c in range(3):
        v = _octaves(h, w, rng, (256, 64, 16, 4), (0.5, 0.25, 0.15, 0.1))
        rgb[..., c] = np.clip(np.rint(v * 255.0), 0, 255).astype(np.uint8)
    lo, hi = np.log(max(2.0, min(h, w) / 64.0)), np.log(max(4.0, min(h, w) / 4.0))
    for _ in range(rects):
        rh = int(np.exp(rng.uniform(lo, hi)))
        rw = int(np.exp(rng.uniform(lo, hi)))
        y0 = int(rng.integers(0, max(1, h - rh + 1)))
        x0 = int(rng.integers(0, max(1, w - rw + 1)))
        rgb[y0:y0 + rh, x0:x0 + rw] = rng.integers(0, 256, 3, dtype=np.uint8)
    return rgb


def rgb_noise(h: int = 512, w: int = 512, seed: int = SEED_BASE + 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    out = np.empty((h, w, 4), np.uint8)
    out[..., :3] = _rgb_layer(h, w, rng)
    out[..., 3] = 255
    return out


def _box4(m: np.ndarray, axis: int) -> np.ndarray:
    """4-wide box filter with edge padding (a 4-px linear ramp across a step)."""
    pad = [(0, 0)] * m.ndim
    pad[axis] = (2, 1)
    p = np.pad(m, pad, mode="edge")
    c = np.cumsum(p, axis=axis, dtype=np.float32)
    c = np.concatenate([np.zeros_like(np.take(c, [0], axis=axis)), c], axis=axis)
    n = m.shape[axis]
    hi = np.take(c, np.arange(4, n + 4), axis=axis)
    lo = np.take(c, np.arange(0, n), axis=axis)
    return (hi - lo) / 4.0


def rgba_cutout(h: int = 2048, w: int = 2048, seed: int = SEED_BASE + 1) -> np.ndarray:
    rng = np.random.default_rng(seed)
    out = np.empty((h, w, 4), np.uint8)
    out[..., :3] = _rgb_layer(h, w, rng)
    mask = (value_noise(h, w, 32, rng) >= 0.4).astype(np.float32)
    ramp = _box4(_box4(mask, 0), 1)
    out[..., 3] = np.clip(np.rint(ramp * 255.0), 0, 255).astype(np.uint8)
    return out


def normal_map(h: int = 4096, w: int = 4096, seed: int = SEED_BASE + 2) -> np.ndarray:
    rng = np.random.default_rng(seed)
    periods = (512, 256, 128, 64, 32, 16)
    amps = tuple(0.5 ** i for i in range(6))
    height = _octaves(h, w, rng, periods, amps) * np.float32(8.0 * 16.0 / sum(amps))
    p = np.pad(height, 1, mode="edge")
    # Sobel (normalised by 8) -> slope in height units per pixel
    gx = ((p[:-2, 2:] + 2 * p[1:-1, 2:] + p[2:, 2:]) - (p[:-2, :-2] + 2 * p[1:-1, :-2] + p[2:, :-2])) / 8.0
    gy = ((p[2:, :-2] + 2 * p[2:, 1:-1] + p[2:, 2:]) - (p[:-2, :-2] + 2 * p[:-2, 1:-1] + p[:-2, 2:])) / 8.0
    nz = np.ones_like(gx)
    inv = 1.0 / np.sqrt(gx * gx + gy * gy + nz)
    out = np.empty((h, w, 4), np.uint8)
    for c, comp in enumerate((-gx * inv, -gy * inv, nz * inv)):
        out[..., c] = np.clip(np.rint((comp + 1.0) * 127.5), 0, 255).astype(np.uint8)
    out[..., 3] = 255
    return out


def ui_shapes(h: int = 512, w: int = 512, seed: int = SEED_BASE + 5) -> np.ndarray:
    """Flat-colour graphics (UI, sprites): a background and 400 hard-edged
    rectangles and discs of random colours and sizes 2..40 px, A = 255.
    Blocks where three colours meet are where three-partition blocks pay."""
    rng = np.random.default_rng(seed)
    out = np.empty((h, w, 4), np.uint8)
    out[..., :3] = rng.integers(0, 256, 3)
    out[..., 3] = 255
    yy, xx = np.mgrid[0:h, 0:w]
    for _ in range(400):
        c = rng.integers(0, 256, 3)
        y0, x0 = int(rng.integers(0, h)), int(rng.integers(0, w))
        sh, sw = (int(v) for v in rng.integers(2, 40, 2))
        if rng.random() < 0.5:
            out[y0:y0 + sh, x0:x0 + sw, :3] = c
        else:
            r = max(sh, sw) / 2
            out[(yy - y0) ** 2 + (xx - x0) ** 2 < r * r, :3] = c
    return out


WORKLOADS = {
    "4x4_rgb_512": dict(gen=rgb_noise, shape=(512, 512), block_dim=4, has_alpha=False,
                        is_normal=False, srgb=False, border=0),
    "6x6_rgba_srgb_2048": dict(gen=rgba_cutout, shape=(2048, 2048), block_dim=6, has_alpha=True,
                               is_normal=False, srgb=True, border=1),
    "4x4_normal_4096": dict(gen=normal_map, shape=(4096, 4096), block_dim=4, has_alpha=False,
                            is_normal=True, srgb=False, border=0),
}


def workload(name: str, scale: float = 1.0) -> tuple[np.ndarray, dict]:
    """Texture + encoder options of a named workload (scale < 1 shrinks it)."""
    spec = dict(WORKLOADS[name])
    h, w = spec.pop("shape")
    h, w = max(1, int(h * scale)), max(1, int(w * scale))
    gen = spec.pop("gen")
    return gen(h, w), spec
