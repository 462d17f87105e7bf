"""The C ABI without a GPU: symbols, argument checks, .astc file I/O.

None of these calls reaches a CUDA kernel: the library rejects bad arguments
before it touches the device, and file I/O is host-only.
"""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "astc_gb300.h")


def _declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_\s\*]*?\b(astc_[a-z0-9_]+)\s*\(", src, re.M)
    return sorted(set(names))


def test_header_declares_the_boundary():
    names = _declared_functions()
    for n in ("astc_encode_gpu", "astc_opts_init", "astc_save_file", "astc_load_file",
              "astc_decode_gpu", "astc_last_error"):
        assert n in names


def test_library_exports_every_declared_symbol(native):
    lib = native.load_library()
    missing = [n for n in _declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_fp32_peak_probe_is_built_apart(native):
    """The benchmark's FP32 FMA probe is its own library, not part of the encoder's."""
    import ctypes
    from astc_encoder_gb300 import build
    peak = ctypes.CDLL(build.PEAK_LIB)
    assert hasattr(peak, "astc_fp32_fma_peak")
    assert not hasattr(native.load_library(), "astc_fp32_fma_peak")


def test_library_links_no_oracle(native):
    # the product library must not carry the oracle's code
    data = open(native.library_path(), "rb").read()
    assert b"oracle_encode" not in data


def test_opts_init_matches_reference_defaults(native):
    o = native.AstcOpts()
    native.load_library().astc_opts_init(ctypes.byref(o))
    # encode_option(): is4x4 = true, everything else false (astc_encode.h:21-27)
    assert (o.block_dim, o.has_alpha, o.is_normal, o.srgb) == (4, 0, 0, 0)
    assert (o.border, o.precision, o.memory) == (0, 0, 0)
    assert o.stream is None


def test_encoded_size(native):
    lib = native.load_library()
    assert lib.astc_encoded_size(512, 512, 4) == 262144
    assert lib.astc_encoded_size(2048, 2048, 6) == 16 * 342 * 342
    assert lib.astc_encoded_size(1, 1, 4) == 16
    assert lib.astc_encoded_size(0, 5, 4) == 0
    assert lib.astc_encoded_size(5, 5, 5) == 0


@pytest.mark.parametrize("field,value", [("block_dim", 5), ("border", 2), ("precision", 7),
                                         ("memory", 3), ("axis", 3), ("quality", -1),
                                         ("quality", 5)])
def test_bad_options_rejected(native, field, value):
    lib = native.load_library()
    o = native.make_opts()
    setattr(o, field, value)
    buf = np.zeros((4, 4, 4), np.uint8)
    out = np.zeros(16, np.uint8)
    st = lib.astc_encode_gpu(buf.ctypes.data, 4, 4, ctypes.byref(o), out.ctypes.data)
    assert st == native.Status.INVALID_ARG
    assert lib.astc_last_error()


@pytest.mark.parametrize("axis,quality", [(1, 0), (2, 0), (0, 1), (1, 1), (2, 1), (0, 2), (0, 3), (0, 4)])
def test_half2_rejects_search_and_axis(native, axis, quality):
    """The max-accumulation axis and the mode search are FP32 only."""
    lib = native.load_library()
    o = native.make_opts(precision=native.Precision.HALF2, axis=axis, quality=quality)
    buf = np.zeros((4, 4, 4), np.uint8)
    out = np.zeros(16, np.uint8)
    st = lib.astc_encode_gpu(buf.ctypes.data, 4, 4, ctypes.byref(o), out.ctypes.data)
    assert st == native.Status.UNSUPPORTED
    assert b"FP32" in lib.astc_last_error()


def test_opts_init_defaults(native):
    o = native.AstcOpts()
    o.axis, o.quality = 7, 7
    native.load_library().astc_opts_init(ctypes.byref(o))
    assert (o.block_dim, o.precision, o.axis, o.quality) == (4, 0, native.Axis.PCA, native.Quality.FAST)


def test_bad_sizes_and_pointers_rejected(native):
    lib = native.load_library()
    o = native.make_opts()
    buf = np.zeros((4, 4, 4), np.uint8)
    out = np.zeros(16, np.uint8)
    assert lib.astc_encode_gpu(buf.ctypes.data, 0, 4, ctypes.byref(o), out.ctypes.data) == 1
    assert lib.astc_encode_gpu(buf.ctypes.data, 4, -1, ctypes.byref(o), out.ctypes.data) == 1
    assert lib.astc_encode_gpu(None, 4, 4, ctypes.byref(o), out.ctypes.data) == 1
    assert lib.astc_encode_gpu(buf.ctypes.data, 4, 4, ctypes.byref(o), None) == 1
    assert lib.astc_encode_gpu(buf.ctypes.data, 4, 4, None, out.ctypes.data) == 1
    assert lib.astc_encode_gpu(buf.ctypes.data, 1 << 24, 4, ctypes.byref(o), out.ctypes.data) == 1
    assert lib.astc_encode_gpu_pitched(buf.ctypes.data, 4, 4, 15, ctypes.byref(o), out.ctypes.data) == 1
    with pytest.raises(native.AstcError):
        native.encode(np.zeros((0, 4, 4), np.uint8))
    with pytest.raises(native.AstcError):
        native.encode(np.zeros((4, 4, 3), np.uint8))


def test_status_strings(native):
    lib = native.load_library()
    for s in native.Status:
        assert lib.astc_status_string(int(s))
    assert lib.astc_status_string(999) == b"unknown status"


def test_save_file_layout(native, tmp_path):
    # astc_header (astc_save.h:5-14) + blocks, as save_astc writes it
    blocks = np.arange(16 * 342 * 342, dtype=np.uint32).astype(np.uint8).reshape(-1, 16)
    p = str(tmp_path / "x.astc")
    native.save_astc(p, 6, 6, 2048, 2048, blocks)
    raw = open(p, "rb").read()
    assert raw[:4] == bytes([0x13, 0xAB, 0xA1, 0x5C])
    assert raw[4:7] == bytes([6, 6, 1])
    assert raw[7:10] == (2048).to_bytes(3, "little")
    assert raw[10:13] == (2048).to_bytes(3, "little")
    assert raw[13:16] == bytes([1, 0, 0])
    assert raw[16:] == blocks.tobytes()
    got, bx, by, w, h = native.load_astc(p)
    assert (bx, by, w, h) == (6, 6, 2048, 2048)
    assert np.array_equal(got, blocks)


def test_save_file_errors(native, tmp_path):
    blocks = np.zeros((4, 16), np.uint8)
    with pytest.raises(native.AstcError) as e:
        native.save_astc(str(tmp_path / "no" / "such" / "dir.astc"), 4, 4, 8, 8, blocks)
    assert e.value.status == native.Status.IO
    with pytest.raises(native.AstcError) as e:
        native.save_astc(str(tmp_path / "bad.astc"), 4, 4, 8, 9, blocks)   # wrong size
    assert e.value.status == native.Status.INVALID_ARG


def test_load_file_errors(native, tmp_path):
    p = tmp_path / "bad.astc"
    p.write_bytes(b"\x00" * 10)
    with pytest.raises(native.AstcError) as e:
        native.load_astc(str(p))
    assert e.value.status == native.Status.FORMAT
    p.write_bytes(b"\x00" * 32)
    with pytest.raises(native.AstcError) as e:
        native.load_astc(str(p))
    assert e.value.status == native.Status.FORMAT
    good = bytes([0x13, 0xAB, 0xA1, 0x5C, 4, 4, 1, 8, 0, 0, 8, 0, 0, 1, 0, 0]) + b"\x00" * 40
    p.write_bytes(good)                                      # 4 blocks need 64 bytes
    with pytest.raises(native.AstcError) as e:
        native.load_astc(str(p))
    assert e.value.status == native.Status.FORMAT
    with pytest.raises(native.AstcError) as e:
        native.load_astc(str(tmp_path / "missing.astc"))
    assert e.value.status == native.Status.IO


def test_encode_option_mirror(native):
    o = native.EncodeOption()
    assert o.block_dim == 4
    assert native.EncodeOption(is6x6=True).block_dim == 6
    # the reference's -4x4 leaves is4x4 true; its -6x6 is a no-op there
    assert native.EncodeOption(is4x4=True, has_alpha=True).block_dim == 4
