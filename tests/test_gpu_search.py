"""CUDA quality modes (search, THOROUGH, PARTITIONS, THREE_PARTITIONS) and the
max-accumulation axis vs the FP32 oracle, through the C ABI.

Bar: every block bit-identical to the oracle's search / max-accumulation
encode (the kernels follow the oracle's FP32 model and its integer scoring
step by step), at small sizes over every option and at the workloads' full
sizes; and the size-independent property of the search: its decoded error is
never above the fixed mode's.
"""
import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _texture(h, w, seed):
    """Noise, flat patches, ramps, two-colour stripes and alpha cut-outs."""
    rng = np.random.default_rng(seed)
    img = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    yy, xx = np.mgrid[0:h, 0:w]
    ramp = ((xx * 5 + yy * 2) % 256).astype(np.uint8)
    img[(yy // 5 + xx // 7) % 3 == 0] = np.array([40, 90, 200, 255], np.uint8)
    img[..., 0] = np.where((yy // 6) % 3 == 1, ramp, img[..., 0])
    img[..., 1] = np.where((xx // 9) % 2 == 0, ramp, img[..., 1])
    stripes = (xx // 3) % 2 == 0
    img[((yy // 13) % 4 == 2) & stripes] = np.array([250, 250, 250, 255], np.uint8)
    img[((yy // 13) % 4 == 2) & ~stripes] = np.array([5, 10, 15, 255], np.uint8)
    img[..., 3] = np.where((yy // 11) % 2 == 0, 255, img[..., 3])
    return img


def _psnr(a, b):
    mse = np.mean((a.astype(np.float64) - b.astype(np.float64)) ** 2)
    return float("inf") if mse == 0 else 10 * np.log10(255.0 ** 2 / mse)


GRID = [g for g in itertools.product([4, 6], [False, True], [False, True], [False, True], [0, 1, 2], [0, 1, 2, 3, 4])
        if (g[4] or g[5]) and not (g[5] >= 2 and g[4] != 0)]


@pytest.mark.parametrize("dim,alpha,normal,srgb,axis,quality", GRID)
def test_option_grid_bit_exact(native, oracle, dim, alpha, normal, srgb, axis, quality):
    img = _texture(71, 53, seed=dim * 131 + alpha * 17 + normal * 7 + srgb * 3 + axis * 2 + quality)
    opts = dict(block_dim=dim, has_alpha=alpha, is_normal=normal, srgb=srgb, border=1)
    got = native.encode(img, axis=axis, quality=quality, **opts)
    want = oracle.encode(img, axis=axis, quality=quality, **opts)
    same = np.all(got == want, axis=1)
    assert np.array_equal(got, want), f"{(~same).sum()} of {len(same)} blocks differ"


@pytest.mark.parametrize("h,w", [(1, 1), (5, 7), (6, 6), (13, 7), (33, 65), (3, 200)])
@pytest.mark.parametrize("dim", [4, 6])
def test_ragged_sizes(native, oracle, h, w, dim):
    img = _texture(h, w, seed=h * 1000 + w)
    for border in (0, 1):
        for quality in (1, 2, 3, 4):
            for alpha in (False, True):
                opts = dict(block_dim=dim, has_alpha=alpha, border=border, quality=quality)
                assert np.array_equal(native.encode(img, **opts), oracle.encode(img, **opts))


@pytest.mark.parametrize("h,w", [(4, 20000), (20001, 6)])
def test_extreme_aspect_ratios(native, oracle, h, w):
    """One block row of 5000 blocks, and one block column of 3334-5001: the
    block index arithmetic at the widths and heights the grid spans."""
    img = _texture(h, w, seed=h + w)
    for dim in (4, 6):
        for quality in (1, 2, 3, 4):
            opts = dict(block_dim=dim, border=1, quality=quality)
            assert np.array_equal(native.encode(img, **opts), oracle.encode(img, **opts)), (dim, quality)


def test_constant_images(native, oracle):
    for val in (0, 1, 127, 255):
        img = np.full((24, 24, 4), val, np.uint8)
        for dim, alpha in ((4, False), (6, True)):
            for axis in (0, 1):
                opts = dict(block_dim=dim, has_alpha=alpha, axis=axis, quality=1)
                got = native.encode(img, **opts)
                assert np.array_equal(got, oracle.encode(img, **opts))
                # a constant block is exact in the fixed mode already: kept
                assert np.array_equal(got, native.encode(img, block_dim=dim, has_alpha=alpha))


@pytest.mark.parametrize("quality", [1, 2, 3, 4])
@pytest.mark.parametrize("name", ["4x4_rgb_512", "6x6_rgba_srgb_2048", "4x4_normal_4096"])
def test_workloads_full_size(native, oracle, name, quality):
    """Full-size workloads: bit-exact, decodes cleanly, never worse than FAST."""
    from astc_encoder_gb300 import synth
    img, spec = synth.workload(name)
    got = native.encode(img, quality=quality, **spec)
    want = oracle.encode(img, quality=quality, **spec)
    same = np.all(got == want, axis=1)
    assert np.array_equal(got, want), f"{(~same).sum()} of {len(same)} blocks differ"
    h, w = img.shape[:2]
    dim = spec["block_dim"]
    fast = native.encode(img, **spec)
    ref = native.fitted_reference(img, spec.get("srgb", False), spec.get("is_normal", False))
    d_search = native.decode(got, w, h, dim, srgb=spec.get("srgb", False))
    d_fast = native.decode(fast, w, h, dim, srgb=spec.get("srgb", False))
    _, errors = oracle.decode(got, w, h, dim)
    assert errors == 0
    ch = 4 if spec.get("has_alpha") else 3
    p_search = _psnr(d_search[..., :ch], ref[..., :ch])
    p_fast = _psnr(d_fast[..., :ch], ref[..., :ch])
    assert p_search >= p_fast, (p_search, p_fast)


@pytest.mark.parametrize("dim,srgb,normal", [(4, False, False), (6, False, False), (4, True, False),
                                             (6, True, False), (4, False, True)])
def test_three_partitions_flat_graphics(native, oracle, dim, srgb, normal):
    """Flat-colour graphics, where three-partition blocks win: bit-exact with
    the oracle, some blocks carry three partitions, and the decode beats
    PARTITIONS'."""
    from astc_encoder_gb300 import synth
    img = synth.ui_shapes(160, 144, seed=40 + dim + 2 * srgb + 4 * normal)
    opts = dict(block_dim=dim, srgb=srgb, is_normal=normal, border=1)
    got = native.encode(img, quality=4, **opts)
    want = oracle.encode(img, quality=4, **opts)
    same = np.all(got == want, axis=1)
    assert np.array_equal(got, want), f"{(~same).sum()} of {len(same)} blocks differ"
    three = ((got.view("<u4")[:, 0] >> 11) & 3) == 2
    assert three.any()
    two = native.encode(img, quality=3, **opts)
    ref = native.fitted_reference(img, srgb, normal)
    ch = 2 if normal else 3
    d3 = native.decode(got, 144, 160, dim, srgb=srgb)
    d2 = native.decode(two, 144, 160, dim, srgb=srgb)
    assert _psnr(d3[..., :ch], ref[..., :ch]) >= _psnr(d2[..., :ch], ref[..., :ch])


def test_device_pointer_path(native, oracle):
    import torch
    img = _texture(96, 80, seed=5)
    want = oracle.encode(img, block_dim=6, has_alpha=True, quality=1, axis=1)
    dev = torch.from_numpy(img).cuda()
    out = torch.empty((len(want), 16), dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()        # without a stream the library runs on its own stream
    native.encode_device(dev.data_ptr(), 80, 96, out.data_ptr(), block_dim=6, has_alpha=True,
                         quality=1, axis=1)
    assert np.array_equal(out.cpu().numpy(), want)


def test_launch_counter_and_fixed_mode_unchanged(native, oracle):
    img = _texture(40, 40, seed=3)
    before = native.kernel_launch_count()
    native.encode(img, quality=1)
    assert native.kernel_launch_count() == before + 1
    # the default options still run the fixed pipeline, bit-exact
    assert np.array_equal(native.encode(img), oracle.encode(img))
