"""The oracle's modes beyond the reference's fixed pipeline.

* axis = 1: max_accumulation_pixel_direction (ASTC_Encode.hlsl:170-227), the
  endpoint fit the reference defines but leaves commented out at line 515;
* quality = 1: the search the reference sketches as choose_best_quantmethod
  (524-526): the fixed-mode block plus every single-partition 4x4-grid mode;
* quality 2-4: the search from the better of both fits with dual-plane
  blocks, then two- and three-partition blocks.

The reference never runs either, so there is no reference output to pin them
to; these tests pin them to the ASTC rules instead: the endpoint range is the
one the decoder derives, every search block decodes (spec decoder) to exactly
the error the search scored it with, the search is never worse than the fixed
mode, and the max-accumulation fit reproduces a two-colour block exactly.
"""
import numpy as np
import pytest

from astc_encoder_gb300 import synth

QUANT_LEVELS = [2, 3, 4, 5, 6, 8, 10, 12, 16, 20, 24, 32, 40, 48, 64, 80, 96, 128, 160, 192, 256]


def _ise_bits(q, n):
    levels = QUANT_LEVELS[q]
    b = 0
    while levels % 2 == 0:
        levels //= 2
        b += 1
    if levels == 3:
        return ((8 + 5 * b) * n + 4) // 5
    if levels == 5:
        return ((7 + 3 * b) * n + 2) // 3
    return n * b


@pytest.mark.parametrize("nvals", [6, 8])
def test_endpoint_range_is_the_decoders(oracle, nvals):
    for wq in range(12):
        wbits = _ise_bits(wq, 16)
        avail = 128 - 17 - wbits
        fits = [q for q in range(4, 21) if _ise_bits(q, nvals) <= avail]
        want = max(fits) if (24 <= wbits <= 96 and fits) else -1
        assert oracle.endpoint_quant(wq, nvals) == want
    # QUANT_2 weights (16 bits) are below the 24-bit minimum; QUANT_32 leaves
    # 31 bits: QUANT_32 endpoints for RGB, QUANT_12 for RGBA
    assert oracle.endpoint_quant(0, nvals) == -1
    assert oracle.endpoint_quant(11, nvals) == (11 if nvals == 6 else 7)


def _fit_texels(oracle, px, srgb):
    tex = px.reshape(-1, 4).astype(np.float32)
    if srgb:
        tex[:, :3] = oracle.srgb_lut()[px.reshape(-1, 4)[:, :3]]
    return tex


def _decoded_error(oracle, blk, tex, dim, alpha, srgb):
    """Squared error of the spec decode against the texels rounded to bytes."""
    dec, _ = oracle.decode(blk.reshape(1, 16), dim, dim, dim, dim, srgb)
    dec = dec.reshape(-1, 4).astype(np.int64)
    target = np.rint(tex).astype(np.int64)
    ch = 4 if alpha else 3
    return int(((dec[:, :ch] - target[:, :ch]) ** 2).sum())


def _random_block(rng, dim, kind):
    px = rng.integers(0, 256, (dim, dim, 4)).astype(np.uint8)
    if kind == 1:                                   # flat colour, noisy alpha
        px[..., :3] = px[:1, :1, :3]
    elif kind == 2:                                 # gradient with a little noise
        ramp = np.linspace(0, 255, dim * dim * 4).reshape(dim, dim, 4)
        px = np.clip(ramp + rng.integers(-6, 7, ramp.shape), 0, 255).astype(np.uint8)
    elif kind == 3:                                 # two colours
        a, b = rng.integers(0, 256, 4), rng.integers(0, 256, 4)
        mask = rng.random((dim, dim)) < 0.5
        px[mask], px[~mask] = a, b
    return px


@pytest.mark.parametrize("dim", [4, 6])
@pytest.mark.parametrize("alpha", [False, True])
@pytest.mark.parametrize("srgb", [False, True])
@pytest.mark.parametrize("axis", [0, 1, 2])
def test_search_scores_match_the_spec_decode(oracle, dim, alpha, srgb, axis):
    rng = np.random.default_rng(1000 * dim + 100 * alpha + 10 * srgb + axis)
    chosen = set()
    for trial in range(60):
        px = _random_block(rng, dim, trial % 4)
        tex = _fit_texels(oracle, px, srgb)
        blk, wq, err, err_fixed = oracle.search_block(tex, dim, alpha, srgb, axis)
        assert err <= err_fixed
        assert _decoded_error(oracle, blk, tex, dim, alpha, srgb) == err
        chosen.add(wq)
    assert len(chosen) >= 3          # several ranges win on mixed content


@pytest.mark.parametrize("dim", [4, 6])
@pytest.mark.parametrize("alpha", [False, True])
def test_search_image_never_worse_and_decodes(oracle, dim, alpha):
    """Whole images: no error blocks, and per-block error never above the fixed mode."""
    rgba = synth.rgb_noise(96, 80, seed=5) if not alpha else synth.rgba_cutout(96, 80, seed=6)
    fixed = oracle.encode(rgba, block_dim=dim, has_alpha=alpha, border=1)
    best = oracle.encode(rgba, block_dim=dim, has_alpha=alpha, border=1, quality=1)
    assert (best != fixed).any(axis=1).mean() > 0.2
    h, w = rgba.shape[:2]
    ch = 4 if alpha else 3
    dfix, e1 = oracle.decode(fixed, w, h, dim)
    dbest, e2 = oracle.decode(best, w, h, dim)
    assert e1 == 0 and e2 == 0

    def block_sse(d):
        diff = (d[..., :ch].astype(np.int64) - rgba[..., :ch]) ** 2
        nby, nbx = -(-h // dim), -(-w // dim)
        pad = np.zeros((nby * dim, nbx * dim, ch), np.int64)
        pad[:h, :w] = diff
        return pad.reshape(nby, dim, nbx, dim, ch).sum(axis=(1, 3, 4)).ravel()

    # clamp border: edge blocks score replicated texels too, so compare the
    # interior blocks exactly and the image as a whole
    nby, nbx = -(-h // dim), -(-w // dim)
    interior = np.zeros((nby, nbx), bool)
    interior[: h // dim, : w // dim] = True
    sf, sb = block_sse(dfix), block_sse(dbest)
    assert (sb[interior.ravel()] <= sf[interior.ravel()]).all()
    assert sb.sum() < sf.sum()


@pytest.mark.parametrize("dim", [4, 6])
@pytest.mark.parametrize("alpha", [False, True])
def test_thorough_picks_the_better_fit(oracle, dim, alpha):
    """quality 2 searches from whichever fit has the smaller fixed-mode
    error: on every block its error is at most the min of the two
    single-fit fixed modes, and it equals a quality-1 encode with the axis
    that fit came from."""
    rng = np.random.default_rng(77 + dim + alpha)
    wins = {0: 0, 1: 0}
    for trial in range(80):
        px = _random_block(rng, dim, trial % 4)
        if trial % 5 == 1:                           # flat colour, alpha cut-out
            px[..., :3] = 120
            px[..., 3] = np.where(rng.random((dim, dim)) < 0.5, 0, 255)
        tex = _fit_texels(oracle, px, False)
        blk, wq, err, err_fixed = oracle.search_block(tex, dim, alpha, False, 2)
        runs = [oracle.search_block(tex, dim, alpha, False, a) for a in (0, 1)]
        assert err_fixed == min(runs[0][3], runs[1][3])
        pick = 1 if runs[1][3] < runs[0][3] else 0
        wins[pick] += 1
        assert err <= runs[pick][2]
        if wq < 200:                                 # a single-plane block: the picked fit's search
            assert np.array_equal(blk, runs[pick][0]) and err == runs[pick][2]
    assert wins[0] and wins[1]


def _four_colour_block(rng, dim):
    """Two regions of two colours each: one partition cannot hold the four
    colours, two can."""
    cols = rng.integers(0, 256, (4, 4)).astype(np.uint8)
    yy, xx = np.mgrid[0:dim, 0:dim]
    region = (xx + rng.integers(-1, 2)) >= dim // 2
    pick = rng.random((dim, dim)) < 0.5
    px = np.empty((dim, dim, 4), np.uint8)
    px[region & pick], px[region & ~pick] = cols[0], cols[1]
    px[~region & pick], px[~region & ~pick] = cols[2], cols[3]
    return px


@pytest.mark.parametrize("dim", [4, 6])
@pytest.mark.parametrize("alpha", [False, True])
@pytest.mark.parametrize("srgb", [False, True])
def test_two_partitions_score_match_the_spec_decode(oracle, dim, alpha, srgb):
    rng = np.random.default_rng(500 + 10 * dim + 2 * alpha + srgb)
    partitioned = 0
    for trial in range(60):
        px = _four_colour_block(rng, dim) if trial % 2 else _random_block(rng, dim, trial % 4)
        tex = _fit_texels(oracle, px, srgb)
        blk, wq, err, _ = oracle.search_block(tex, dim, alpha, srgb, 2, partitions=True)
        _, _, err_thorough, _ = oracle.search_block(tex, dim, alpha, srgb, 2)
        assert err <= err_thorough
        assert _decoded_error(oracle, blk, tex, dim, alpha, srgb) == err
        if 100 <= wq < 200:
            partitioned += 1
            word = int.from_bytes(blk[:4].tobytes(), "little")
            assert (word >> 11) & 3 == 1                       # two partitions
            assert (word >> 23) & 3 == 0 and (word >> 25) & 0xF == (12 if alpha else 8)
    assert partitioned >= 10


@pytest.mark.parametrize("dim", [4, 6])
@pytest.mark.parametrize("alpha", [False, True])
def test_two_partitions_image(oracle, dim, alpha):
    rgba = synth.rgb_noise(96, 80, seed=15) if not alpha else synth.rgba_cutout(96, 80, seed=16)
    thorough = oracle.encode(rgba, block_dim=dim, has_alpha=alpha, border=1, quality=2)
    best = oracle.encode(rgba, block_dim=dim, has_alpha=alpha, border=1, quality=3)
    h, w = rgba.shape[:2]
    ch = 4 if alpha else 3
    d2, e2 = oracle.decode(thorough, w, h, dim)
    d3, e3 = oracle.decode(best, w, h, dim)
    assert e2 == 0 and e3 == 0
    sse = lambda d: int(((d[..., :ch].astype(np.int64) - rgba[..., :ch]) ** 2).sum())  # noqa: E731
    assert sse(d3) < sse(d2)
    assert ((best.view("<u4")[:, 0] >> 11) & 3).astype(bool).mean() > 0.05


@pytest.mark.parametrize("dim", [4, 6])
def test_search_fp64_twin_runs(oracle, dim):
    rgba = synth.rgb_noise(40, 40, seed=9)
    a = oracle.encode(rgba, block_dim=dim, quality=1)
    b = oracle.encode(rgba, block_dim=dim, quality=1, fp64=True)
    assert (a == b).all(axis=1).mean() > 0.8


@pytest.mark.parametrize("alpha", [False, True])
def test_max_accumulation_two_colour_block(oracle, alpha):
    """Two colours: every deviation above the mean is the bright colour's, so
    the axis is (bright - mean) and the endpoints are the two colours."""
    dark = np.array([10, 20, 30, 40 if alpha else 255], np.uint8)
    bright = np.array([210, 120, 60, 250 if alpha else 255], np.uint8)
    px = np.empty((4, 4, 4), np.uint8)
    pattern = (np.arange(16) % 3 == 0).reshape(4, 4)
    px[pattern], px[~pattern] = bright, dark
    blocks = oracle.encode(px, block_dim=4, has_alpha=alpha, axis=1)
    ep = np.zeros(8, np.uint32)
    for c in range(4):
        ep[2 * c], ep[2 * c + 1] = dark[c], bright[c]
    qw = np.where(pattern.ravel(), 5 if alpha else 11, 0).astype(np.uint32)
    want = oracle.assemble_symbolic(ep, qw, alpha)
    assert np.array_equal(blocks[0], want)


def test_max_accumulation_constant_block_equals_pca(oracle):
    px = np.full((6, 6, 4), [90, 140, 200, 255], np.uint8)
    assert np.array_equal(oracle.encode(px, block_dim=6, axis=1), oracle.encode(px, block_dim=6))


@pytest.mark.parametrize("dim", [4, 6])
@pytest.mark.parametrize("alpha", [False, True])
@pytest.mark.parametrize("srgb", [False, True])
def test_dual_plane_blocks(oracle, dim, alpha, srgb):
    """THOROUGH's dual-plane blocks: D bit set, the plane selector names the
    channel split off, and they decode to exactly their scored error."""
    rng = np.random.default_rng(900 + 10 * dim + 2 * alpha + srgb)
    dual = 0
    for trial in range(60):
        px = _random_block(rng, dim, trial % 4)
        if trial % 3 == 0:                          # one channel independent of the others
            px[..., 1] = rng.integers(0, 256, (dim, dim))
        tex = _fit_texels(oracle, px, srgb)
        blk, wq, err, _ = oracle.search_block(tex, dim, alpha, srgb, 2)
        assert _decoded_error(oracle, blk, tex, dim, alpha, srgb) == err
        if 200 <= wq < 300:
            dual += 1
            pc, q = (wq - 200) // 16, (wq - 200) % 16
            word = int.from_bytes(blk.tobytes(), "little")
            assert (word >> 10) & 1 == 1 and (word >> 11) & 3 == 0
            wbits = oracle.ise_bits(q, 32)
            assert (word >> (128 - wbits - 2)) & 3 == pc
            assert pc < (4 if alpha else 3)
    assert dual >= 10


def test_dual_plane_normal_map_gain(oracle):
    """Normal maps carry two independent channels: dual-plane blocks win most
    blocks and lift PSNR well above the single-plane search."""
    from astc_encoder_gb300 import synth
    img, spec = synth.workload("4x4_normal_4096", scale=0.0625)
    h, w = img.shape[:2]
    one = oracle.encode(img, quality=1, **spec)
    two = oracle.encode(img, quality=2, **spec)
    assert ((two.view("<u4")[:, 0] >> 10) & 1).mean() > 0.5

    def sse(blocks):
        d, errors = oracle.decode(blocks, w, h, 4)
        assert errors == 0
        return int(((d[..., :2].astype(np.int64) - img[..., :2]) ** 2).sum())
    assert sse(two) * 2 < sse(one)


def _three_colour_block(rng, dim):
    """Three flat colours in three regions cut by two straight edges, with
    +-2 noise: two partitions cannot hold them, three can."""
    cols = rng.integers(0, 256, (3, 4)).astype(np.int64)
    cols[:, 3] = 255
    yy, xx = np.mgrid[0:dim, 0:dim]
    a = xx * int(rng.integers(1, 4)) + yy * int(rng.integers(-2, 3)) >= int(rng.integers(2, 2 * dim))
    b = yy * int(rng.integers(1, 4)) - xx >= int(rng.integers(0, dim))
    region = np.where(a, 0, np.where(b, 1, 2))
    px = cols[region] + rng.integers(-2, 3, (dim, dim, 4)) * np.array([1, 1, 1, 0])
    return np.clip(px, 0, 255).astype(np.uint8)


@pytest.mark.parametrize("dim", [4, 6])
@pytest.mark.parametrize("alpha", [False, True])
@pytest.mark.parametrize("srgb", [False, True])
def test_three_partitions_score_match_the_spec_decode(oracle, dim, alpha, srgb):
    """Quality 4's three-partition blocks (RGB only: three RGBA partitions
    would need 24 colour endpoint integers, above the format's 18): three
    partitions in the header, one shared CEM, exact scored error, never worse
    than quality 3."""
    rng = np.random.default_rng(700 + 10 * dim + 2 * alpha + srgb)
    three = 0
    for trial in range(60):
        px = _three_colour_block(rng, dim) if trial % 4 else _random_block(rng, dim, trial % 4)
        tex = _fit_texels(oracle, px, srgb)
        blk, wq, err, _ = oracle.search_block(tex, dim, alpha, srgb, 2, partitions=2)
        _, _, err_two, _ = oracle.search_block(tex, dim, alpha, srgb, 2, partitions=1)
        assert err <= err_two
        assert _decoded_error(oracle, blk, tex, dim, alpha, srgb) == err
        if 300 <= wq < 400:
            three += 1
            word = int.from_bytes(blk[:4].tobytes(), "little")
            assert (word >> 11) & 3 == 2                       # three partitions
            assert (word >> 23) & 3 == 0 and (word >> 25) & 0xF == 8
    if alpha:
        assert three == 0
    else:
        assert three >= 6, three


@pytest.mark.parametrize("dim", [4, 6])
def test_three_partitions_image(oracle, dim):
    """Flat-colour graphics: quality 4 decodes cleanly and beats quality 3;
    RGBA input keeps quality 3's blocks."""
    rgba = synth.ui_shapes(96, 96, seed=21)
    q3 = oracle.encode(rgba, block_dim=dim, quality=3)
    q4 = oracle.encode(rgba, block_dim=dim, quality=4)
    d3, e3 = oracle.decode(q3, 96, 96, dim)
    d4, e4 = oracle.decode(q4, 96, 96, dim)
    assert e3 == 0 and e4 == 0
    sse = lambda d: int(((d[..., :3].astype(np.int64) - rgba[..., :3]) ** 2).sum())  # noqa: E731
    assert sse(d4) < sse(d3)
    assert (((q4.view("<u4")[:, 0] >> 11) & 3) == 2).any()
    a3 = oracle.encode(rgba, block_dim=dim, has_alpha=True, quality=3)
    assert np.array_equal(oracle.encode(rgba, block_dim=dim, has_alpha=True, quality=4), a3)


@pytest.mark.parametrize("dim", [4, 6])
@pytest.mark.parametrize("alpha", [False, True])
def test_best_fit_fast_mode(oracle, dim, alpha):
    """axis 2 with the fixed mode: every block is the PCA block or the
    max-accumulation block, whichever decodes with the smaller squared error
    (the PCA on ties)."""
    rgba = synth.rgb_noise(96, 96, seed=31) if not alpha else synth.rgba_cutout(96, 96, seed=32)
    blocks = [oracle.encode(rgba, block_dim=dim, has_alpha=alpha, axis=a) for a in (0, 1, 2)]
    ch = 4 if alpha else 3
    nb = -(-96 // dim)

    def block_sse(blk):
        d, errors = oracle.decode(blk, 96, 96, dim)
        assert errors == 0
        diff = (d[..., :ch].astype(np.int64) - rgba[..., :ch]) ** 2
        pad = np.zeros((nb * dim, nb * dim, ch), np.int64)
        pad[:96, :96] = diff
        return pad.reshape(nb, dim, nb, dim, ch).sum(axis=(1, 3, 4)).ravel()

    e0, e1, e2 = (block_sse(b) for b in blocks)
    # zero border: blocks cut by the image edge score their padded texels, so
    # compare the blocks inside the image
    inside = np.zeros((nb, nb), bool)
    inside[: 96 // dim, : 96 // dim] = True
    inside = inside.ravel()
    pick1 = e1 < e0
    want = np.where(pick1[:, None], blocks[1], blocks[0])
    assert np.array_equal(blocks[2][inside], want[inside])
    assert np.array_equal(e2[inside], np.minimum(e0, e1)[inside])
    assert pick1[inside].any() and (~pick1[inside]).any()


def test_bad_axis_and_quality_rejected(oracle):
    with pytest.raises(ValueError):
        oracle.encode(np.zeros((4, 4, 4), np.uint8), axis=3)
    with pytest.raises(ValueError):
        oracle.encode(np.zeros((4, 4, 4), np.uint8), quality=5)


def test_thorough_recovers_alpha_cutouts(oracle):
    """Flat colour with an alpha cut-out: the reference's PCA start vector has
    no alpha component, so the power iteration exits at once and the block
    collapses to its mean; the max-accumulation fit keeps the cut-out."""
    px = np.zeros((8, 8, 4), np.uint8)
    px[..., :3] = (100, 150, 200)
    px[..., 3] = np.where((np.arange(8)[:, None] + np.arange(8)[None, :]) % 3 == 0, 0, 255)
    fast = oracle.encode(px, block_dim=4, has_alpha=True)
    best = oracle.encode(px, block_dim=4, has_alpha=True, quality=2)
    dfast, _ = oracle.decode(fast, 8, 8, 4)
    dbest, _ = oracle.decode(best, 8, 8, 4)
    for by in (0, 4):                                  # alpha flattened per block
        for bx in (0, 4):
            assert len(np.unique(dfast[by:by + 4, bx:bx + 4, 3])) == 1
    assert np.array_equal(dbest[..., 3], px[..., 3])   # alpha kept exactly
