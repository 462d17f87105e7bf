"""Batched (persistent, CUDA-graph) encode, the packed-half2 precision, and
GPU mip chains.

* A texture's blocks are identical whether it is encoded alone (plain kernel,
  astc_encode_gpu) or inside a batch of textures of other sizes and formats,
  for both precisions; FP32 is also identical to the oracle.
* HALF2 is held to its quality gate: PSNR at most 0.05 dB below
  the FP64 oracle's on the same texture (decoded with the spec decoder, in
  the space the encoder fits).
"""
import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HALF2_MAX_LOSS_DB = 0.05


def _texture(h, w, seed):
    rng = np.random.default_rng(seed)
    img = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    yy, xx = np.mgrid[0:h, 0:w]
    img[..., 0] = ((xx * 3 + yy) % 256).astype(np.uint8)
    img[(yy // 7 + xx // 5) % 4 == 0] = np.array([200, 30, 90, 255], np.uint8)
    img[..., 3] = np.where((xx // 13) % 2 == 0, 255, img[..., 3])
    return img


FORMATS = list(itertools.product([4, 6], [False, True], [False, True], [False, True]))


def _batch_case(torch, seed=0, sizes=None):
    rng = np.random.default_rng(seed)
    sizes = sizes or [(1, 1), (2, 3), (5, 7), (64, 64), (37, 129), (300, 17), (128, 256), (96, 96)]
    cases = []
    for i, (dim, alpha, normal, srgb) in enumerate(FORMATS):
        h, w = sizes[i % len(sizes)]
        img = _texture(h, w, seed * 100 + i)
        opts = dict(block_dim=dim, has_alpha=alpha, is_normal=normal, srgb=srgb,
                    border=int(rng.integers(0, 2)))
        nb = ((w + dim - 1) // dim) * ((h + dim - 1) // dim)
        dev = torch.from_numpy(img).cuda()
        out = torch.zeros((nb, 16), dtype=torch.uint8, device="cuda")
        cases.append((img, opts, dev, out))
    return cases


def _items(cases):
    return [dict(rgba8=d.data_ptr(), width=img.shape[1], height=img.shape[0], out=o.data_ptr(), **opts)
            for img, opts, d, o in cases]


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_equals_alone_all_formats(native, oracle, precision):
    import torch
    cases = _batch_case(torch, seed=precision)
    with native.Batch(64, 1 << 20) as b:
        b.encode(_items(cases), precision=precision)
        for img, opts, dev, out in cases:
            alone = native.encode(img, precision=precision, **opts)
            got = out.cpu().numpy()
            assert np.array_equal(got, alone), opts
            if precision == 0:
                assert np.array_equal(got, oracle.encode(img, **opts)), opts


@pytest.mark.parametrize("quality", [1, 3, 4])
def test_batch_quality_modes(native, oracle, quality):
    """astc_batch_encode_quality: every texture's blocks equal its
    astc_encode_gpu result with the same quality (and the oracle's)."""
    import torch
    cases = _batch_case(torch, seed=10 + quality)
    torch.cuda.synchronize()
    with native.Batch(64, 1 << 20) as b:
        b.encode(_items(cases), quality=quality)
        for img, opts, dev, out in cases:
            got = out.cpu().numpy()
            assert np.array_equal(got, native.encode(img, quality=quality, **opts)), opts
            assert np.array_equal(got, oracle.encode(img, quality=quality, **opts)), opts
        with pytest.raises(native.AstcError) as e:
            b.encode(_items(cases), precision=1, quality=quality)
        assert e.value.status == native.Status.UNSUPPORTED


def test_batch_graph_reuse_and_many_mips(native, oracle):
    import torch
    stream = torch.cuda.Stream()
    with native.Batch(256, 1 << 22) as b:
        for rnd in range(3):                 # same formats -> the cached graph is replayed
            rng = np.random.default_rng(rnd)
            base = _texture(200 + 17 * rnd, 333, rnd)
            levels = native.mip_levels(base.shape[1], base.shape[0])
            sizes = native.mip_sizes(base.shape[1], base.shape[0], levels)
            chain = [base] + [_texture(h, w, rnd * 31 + l) for l, (w, h) in enumerate(sizes[1:])]
            opts = dict(block_dim=int(rng.choice([4, 6])), has_alpha=True, srgb=bool(rnd % 2), border=1)
            devs, outs = [], []
            for img in chain:
                h, w = img.shape[:2]
                d = opts["block_dim"]
                devs.append(torch.from_numpy(img).cuda())
                outs.append(torch.zeros(((w + d - 1) // d) * ((h + d - 1) // d), 16, dtype=torch.uint8,
                                        device="cuda"))
            items = [dict(rgba8=dv.data_ptr(), width=img.shape[1], height=img.shape[0], out=o.data_ptr(),
                          **opts) for img, dv, o in zip(chain, devs, outs)]
            torch.cuda.synchronize()
            b.encode(items, stream=stream.cuda_stream)
            stream.synchronize()
            for img, o in zip(chain, outs):
                assert np.array_equal(o.cpu().numpy(), oracle.encode(img, **opts))


def test_batch_pageable_items(native, oracle):
    """Items in ordinary pageable host memory: encoded in place where the device
    reads the host's page tables (blocks equal to the oracle's), rejected
    elsewhere."""
    import torch
    rng = np.random.default_rng(12)
    imgs = [rng.integers(0, 256, (h, w, 4), dtype=np.uint8) for h, w in ((37, 61), (128, 96), (5, 300))]
    opts = dict(block_dim=6, has_alpha=True, srgb=True, border=1)
    outs = [np.zeros((((w + 5) // 6) * ((h + 5) // 6), 16), np.uint8) for h, w in (i.shape[:2] for i in imgs)]
    items = [dict(rgba8=im.ctypes.data, width=im.shape[1], height=im.shape[0], out=o.ctypes.data, **opts)
             for im, o in zip(imgs, outs)]
    stream = torch.cuda.Stream()
    with native.Batch(8, 4096) as b:
        if not native.device_caps()["pageable_in_place"]:
            with pytest.raises(native.AstcError):
                b.encode(items, stream=stream.cuda_stream)
            return
        for prec in (0, 1):
            b.encode(items, precision=prec, stream=stream.cuda_stream)
            stream.synchronize()
            for im, o in zip(imgs, outs):
                assert np.array_equal(o, native.encode(im, precision=prec, **opts)), prec
            if prec == 0:
                assert np.array_equal(outs[0], oracle.encode(imgs[0], **opts))


def test_batch_rejects_over_capacity(native):
    import torch
    dev = torch.zeros((8, 8, 4), dtype=torch.uint8, device="cuda")
    out = torch.zeros((4, 16), dtype=torch.uint8, device="cuda")
    item = dict(rgba8=dev.data_ptr(), width=8, height=8, out=out.data_ptr())
    with native.Batch(2, 8) as b:
        with pytest.raises(native.AstcError):
            b.encode([item] * 3)                                 # more than max_textures
        with pytest.raises(native.AstcError):
            b.encode([dict(item, width=64, height=64)])          # more than max_blocks
        with pytest.raises(native.AstcError):
            b.encode([dict(item, out=out.data_ptr() + 4)])       # misaligned output
        b.encode([item])                                         # still usable afterwards


def _psnr(native, blocks, img, opts):
    """Decoded PSNR in the fit space; normal maps on the rebuilt unit normals
    (z = sqrt(max(0, 1 - x^2 - y^2)), numpy float64)."""
    h, w = img.shape[:2]
    dec = native.decode(blocks, w, h, opts["block_dim"])
    if opts.get("is_normal"):
        mse = native.normal_sse_numpy(dec, img) / (h * w * 3)
        return 10 * np.log10(255.0 ** 2 / mse)
    ref = native.fitted_reference(img, opts.get("srgb", False), False)
    ch = 4 if opts.get("has_alpha") else 3
    mse = np.mean((dec[..., :ch].astype(np.float64) - ref[..., :ch].astype(np.float64)) ** 2)
    return 10 * np.log10(255.0 ** 2 / mse)


@pytest.mark.parametrize("name", ["4x4_rgb_512", "6x6_rgba_srgb_2048", "4x4_normal_4096"])
def test_half2_quality_gate(native, oracle, name):
    from astc_encoder_gb300 import synth
    img, spec = synth.workload(name, scale=0.5)
    h2 = native.encode(img, precision=1, **spec)
    f64 = oracle.encode(img, fp64=True, **spec)
    f32 = native.encode(img, **spec)
    loss = _psnr(native, f64, img, spec) - _psnr(native, h2, img, spec)
    assert loss <= HALF2_MAX_LOSS_DB, loss
    # the FP32 kernel is the FP32 oracle bit for bit (its gap to the FP64 twin
    # is reported by the bench, not gated: it can go either way)
    assert _psnr(native, f32, img, spec) == _psnr(native, oracle.encode(img, **spec), img, spec)
    # many blocks still agree with the FP32 path bit for bit: most for UNORM
    # input; for sRGB input HALF2 fits the texels rounded to linear bytes
    # (the values the decode is measured against), FP32 the unrounded ones
    same = np.all(h2 == f32, axis=1).mean()
    assert same > (0.3 if spec["srgb"] else 0.5), same


def test_half2_edge_cases(native, oracle):
    for val in (0, 255, 77):
        img = np.full((12, 12, 4), val, np.uint8)
        for dim, alpha in ((4, False), (6, True)):
            h2 = native.encode(img, block_dim=dim, has_alpha=alpha, precision=1)
            assert np.array_equal(h2, oracle.encode(img, block_dim=dim, has_alpha=alpha))
    img = _texture(33, 47, 5)
    for dim in (4, 6):
        for srgb in (False, True):
            h2 = native.encode(img, block_dim=dim, has_alpha=True, srgb=srgb, precision=1, border=1)
            assert h2.shape == oracle.encode(img, block_dim=dim, has_alpha=True).shape


def _np_mips(img, levels, srgb):
    lut = np.where(np.arange(256) / 255.0 <= 0.04045, np.arange(256) / 255.0 / 12.92,
                   ((np.arange(256) / 255.0 + 0.055) / 1.055) ** 2.4).astype(np.float32)
    q = np.arange(4096) / 4095.0
    enc = np.where(q <= 0.0031308, q * 12.92, 1.055 * q ** (1 / 2.4) - 0.055)
    to_srgb = np.clip(np.floor(enc * 255.0 + 0.5), 0, 255).astype(np.uint8)
    out, cur = [], img
    for _ in range(1, levels):
        h, w = cur.shape[:2]
        dh, dw = max(1, h // 2), max(1, w // 2)
        ys = np.minimum(np.arange(dh)[:, None] * 2 + np.array([0, 1]), h - 1)
        xs = np.minimum(np.arange(dw)[:, None] * 2 + np.array([0, 1]), w - 1)
        quad = cur[ys[:, None, :, None], xs[None, :, None, :]].astype(np.int64)   # dh, dw, 2, 2, 4
        nxt = ((quad.sum(axis=(2, 3)) + 2) >> 2).astype(np.uint8)
        if srgb:
            lin = lut[cur[ys[:, None, :, None], xs[None, :, None, :]][..., :3]].astype(np.float32)
            s = lin[:, :, 0, 0] + lin[:, :, 0, 1] + lin[:, :, 1, 0] + lin[:, :, 1, 1]
            qq = np.clip(np.rint(s * np.float32(0.25) * np.float32(4095.0)), 0, 4095).astype(np.int64)
            nxt[..., :3] = to_srgb[qq]
        out.append(nxt)
        cur = nxt
    return out


# sizes: one tile, ragged tiles, one texel wide or high, several 64x64 tiles
# per level and chains longer than the six levels one launch writes
@pytest.mark.parametrize("h,w", [(64, 64), (37, 100), (1, 9), (6, 1), (300, 517), (2, 4100), (4099, 3),
                                 (1030, 2048)])
@pytest.mark.parametrize("srgb", [False, True])
def test_mip_chain_matches_numpy(native, h, w, srgb):
    import torch
    img = _texture(h, w, h * w)
    levels = native.mip_levels(w, h)
    dev = torch.from_numpy(img).cuda()
    out = torch.zeros(max(4, native.mip_chain_bytes(w, h, levels)), dtype=torch.uint8, device="cuda")
    native.generate_mips(dev.data_ptr(), w, h, levels, out.data_ptr(), srgb=srgb)
    got = out.cpu().numpy()
    off = 0
    for lvl, want in enumerate(_np_mips(img, levels, srgb), start=1):
        n = want.size
        g = got[off:off + n].reshape(want.shape)
        if srgb:
            # float rounding in the linear mean may move a texel by one code
            assert np.abs(g.astype(int) - want.astype(int)).max() <= 1, lvl
            assert np.array_equal(g[..., 3], want[..., 3])
        else:
            assert np.array_equal(g, want), lvl
        off += n
    assert off == native.mip_chain_bytes(w, h, levels)
