"""The exact FP32 shortcuts the CUDA kernels use, checked with IEEE float32
arithmetic on the CPU (numpy rounds every float32 operation to nearest even,
like the __f*_rn intrinsics).

* the length tests `sqrt(d) < 1e-5` (ASTC_Encode.hlsl:100, 323) become
  `d < 0x2EDBE6FD`;
* round-half-even of x in [0, 2^22] is (x + 2^23) - 2^23, read as an integer;
* a UNORM8 byte placed in the mantissa of 2^23 and minus 2^23 is the byte.
"""
import numpy as np

T = np.frombuffer(np.uint32(0x2EDBE6FD).tobytes(), np.float32)[0]
C = np.float32(1e-5)


def _floats_around(center_bits, radius):
    bits = np.arange(center_bits - radius, center_bits + radius, dtype=np.int64)
    bits = bits[(bits >= 0) & (bits < 0x7F800000)]
    return bits.astype(np.uint32).view(np.float32)


def test_length_threshold_equivalence_near_boundary():
    x = _floats_around(0x2EDBE6FD, 1 << 20)
    assert np.array_equal(np.sqrt(x) < C, x < T)


def test_length_threshold_equivalence_sampled_everywhere():
    rng = np.random.default_rng(0)
    bits = rng.integers(0, 0x7F800000, 2_000_000, dtype=np.int64).astype(np.uint32)
    x = bits.view(np.float32)
    assert np.array_equal(np.sqrt(x) < C, x < T)
    specials = np.array([0.0, -0.0, np.inf, np.nan, T, np.nextafter(T, np.float32(0))], np.float32)
    assert np.array_equal(np.sqrt(specials) < C, specials < T)


def test_rint_by_magic_add():
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.uniform(0, 300, 1_000_000).astype(np.float32),
                        np.arange(0, 512, 0.5, dtype=np.float32),          # every tie
                        np.array([0.0, -0.0, 4194304.0], np.float32)])
    magic = np.float32(8388608.0)
    got = ((x + magic).view(np.uint32) - np.uint32(0x4B000000)).astype(np.int64)
    assert np.array_equal(got, np.rint(x).astype(np.int64))


def test_byte_to_float_by_mantissa():
    c = np.arange(256, dtype=np.uint32)
    f = (np.uint32(0x4B000000) | c).view(np.float32) - np.float32(8388608.0)
    assert np.array_equal(f, c.astype(np.float32))
