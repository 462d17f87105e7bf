"""The command line tool's image readers against the reference's own loader.

The reference loads its input with stb_image.h (stbi_load(..., 4),
main.cpp:23-24).  Where ASTC_REFERENCE_DIR names the reference tree, the
Makefile under oracle/ builds a harness over that header (oracle/_ref/
stb_load) and these tests compare, file by file, its RGBA with the C++
reader of astc_cs_enc and the Python reader astc_encoder_gb300.image_io, on
files of every format the readers take and on a corpus of mutated files.

Byte-equal RGBA is required except where the readers knowingly differ:
* JPEG: stb_image uses an integer inverse DCT and upsamples chroma
  bilinearly; these readers use a floating-point inverse DCT and replicate
  chroma, so values differ by a few codes (at most 3 without subsampling,
  16 with it);
* BMP with bit fields and a 40-byte header: this version of stb_image reads
  the pixels 12 bytes past the file's data offset (it has already read the
  three masks when it skips to the offset); these readers start at the
  offset, and the test shows the 12-byte shift exactly;
* PSD in grey or with 16-bit channels, and a 32-bit BMP with an alpha
  mask in a 56-byte header: stb_image refuses or stops on an assertion;
  these readers read them;
* PSD colours whose removed white matte falls below 0: stb_image converts
  that negative float to a byte, which C leaves undefined (x86 builds wrap
  it); these readers give 0.  Every other colour of a partly transparent
  PSD pixel is the same.
Corrupt files: the two readers of this repository agree with each other on
every mutated file (the same image or both refuse); where stb_image reads a
file too, the images match (outside the cases above).  stb_image reads
truncated files as if zeros followed; these readers refuse them.
"""
import os
import subprocess

import numpy as np
import pytest

import test_cli as T
from conftest import REFERENCE, ROOT

pytestmark = pytest.mark.skipif(not REFERENCE or not os.path.isfile(os.path.join(REFERENCE, "stb_image.h")),
                                reason="reference tree not given (set ASTC_REFERENCE_DIR)")

STB = os.path.join(ROOT, "oracle", "_ref", "stb_load")


@pytest.fixture(scope="module")
def stb():
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "stb-ref", f"REFERENCE={REFERENCE}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return STB


def _stb_read(stb, path):
    out = path + ".raw"
    try:
        r = subprocess.run([stb, path, out], capture_output=True, text=True, errors="replace", timeout=20)
    except subprocess.TimeoutExpired:
        return None
    if r.returncode != 0:
        return None
    data = open(out, "rb").read()
    head, rest = data.split(b"\n", 1)
    w, h = map(int, head.split())
    return np.frombuffer(rest, np.uint8).reshape(h, w, 4)


def _ours(native, path, tmp_path):
    """(Python reader's image or None, CLI reader's image or None), top-down."""
    from astc_encoder_gb300 import image_io
    try:
        py = image_io.load_image(path)
    except Exception:               # noqa: BLE001 -- any refusal
        py = None
    out = str(tmp_path / "dump.pam")
    r = subprocess.run([T.CLI, path, "--dump-rgba", out], capture_output=True, text=True, errors="replace",
                       timeout=60)
    cli = image_io.load_image(out)[::-1] if r.returncode == 0 else None
    return py, cli


ARR = T._smooth(21, 27, 3, 5)
RGBA = np.dstack([ARR, np.full(ARR.shape[:2], 200, np.uint8)])

# name, writer, how the reference loader compares
CORPUS = [
    ("a.png", lambda p: T._png(p, RGBA, 6), "equal"),
    ("b.png", lambda p: T._png(p, ARR[..., 0], 3, palette=np.arange(768) % 256), "equal"),
    ("o.png", lambda p: T._png(p, (ARR[..., 0] // 64).astype(np.int64), 3, 2, palette=np.arange(12).reshape(4, 3) * 20,
                               trns=np.array([0, 128]), interlace=True), "equal"),
    ("q.png", lambda p: T._png(p, ARR.astype(np.int64) * 257, 2, 16, trns=b"\x00\x01\x00\x02\x00\x03",
                               interlace=True), "equal"),
    ("c.jpg", lambda p: T._jpeg(p, ARR, sampling=(2, 2), restart=2), ("jpeg", 16)),
    ("c1.jpg", lambda p: T._jpeg(p, ARR), ("jpeg", 3)),
    ("d.jpg", lambda p: T._jpeg(p, ARR[..., 0]), ("jpeg", 3)),
    ("j.jpg", lambda p: T._jpeg(p, ARR, sampling=(2, 1), restart=3, mode="progressive"), ("jpeg", 16)),
    ("m.gif", lambda p: T._gif(p, (ARR[..., 0] // 16).astype(np.int64), np.arange(48, dtype=np.uint8).reshape(16, 3) * 5,
                               transparent=3, interlace=True), "equal"),
    ("n.hdr", lambda p: T._hdr(p, np.dstack([ARR, np.full(ARR.shape[:2], 130, np.uint8)])), "equal"),
    ("t.tga", lambda p: T._tga_mapped(p, (ARR[..., 2] // 8).astype(np.int64), np.arange(96).reshape(32, 3), 24, 3, True),
     "equal"),
    ("g.tga", lambda p: T._tga(p, RGBA, rle=True), "equal"),
    ("h.tga", lambda p: T._tga(p, ARR[..., 0], rle=True), "equal"),
    ("v.tga", lambda p: T._tga16(p, ARR[..., 0].astype(np.int64) * 257), "equal"),
    ("u.pic", lambda p: T._pic(p, RGBA, [(2, 0xE0), (1, 0x10)]), "equal"),
    ("w.pic", lambda p: T._pic(p, RGBA, [(0, 0xF0)]), "equal"),
    ("r.bmp", lambda p: T._bmp_indexed(p, (ARR[..., 1] // 16).astype(np.int64), np.arange(48).reshape(16, 3) * 5, 4),
     "equal"),
    ("f.bmp", lambda p: T._bmp(p, ARR), "equal"),
    ("x.bmp", lambda p: T._bmp(p, RGBA, top_down=True), "equal"),
    ("z.bmp", lambda p: T._bmp(p, np.dstack([ARR, np.zeros(ARR.shape[:2], np.uint8)])), "equal"),
    ("y.bmp", lambda p: T._bmp16(p, ARR[..., 0].astype(np.int64) * 200), "equal"),
    ("s.bmp", lambda p: T._bmp16(p, ARR[..., 0].astype(np.int64) * 200, (0xF800, 0x07E0, 0x1F)), "bitfield_offset"),
    ("k.psd", lambda p: T._psd(p, RGBA.transpose(2, 0, 1).copy(), 3, 16, True, 1), "stb_refuses"),
    ("l.psd", lambda p: T._psd(p, RGBA[..., :2].transpose(2, 0, 1).copy(), 1, 8, False), "stb_refuses"),
    ("p.psd", lambda p: T._psd(p, RGBA.transpose(2, 0, 1).copy(), 3, 8, True), "psd_matte"),
]


@pytest.mark.parametrize("name,write,rule", CORPUS, ids=[c[0] for c in CORPUS])
def test_reads_what_the_reference_loader_reads(stb, native, tmp_path, name, write, rule):
    path = str(tmp_path / name)
    write(path)
    ref = _stb_read(stb, path)
    py, cli = _ours(native, path, tmp_path)
    assert py is not None and cli is not None
    assert np.array_equal(py, cli)
    if rule == "stb_refuses":
        assert ref is None
        return
    assert ref is not None
    if rule == "equal":
        assert np.array_equal(py, ref)
    elif rule == "bitfield_offset":
        # the reference loader's image is this reader's image of the same file
        # with the pixel data moved 12 bytes further
        data = bytearray(open(path, "rb").read())
        off = int.from_bytes(data[10:14], "little")
        shifted = str(tmp_path / ("shifted_" + name))
        data[10:14] = (off + 12).to_bytes(4, "little")
        with open(shifted, "wb") as fh:
            fh.write(bytes(data) + bytes(12))
        sp, _ = _ours(native, shifted, tmp_path)
        assert not np.array_equal(py, ref) and np.array_equal(sp, ref)
    elif rule == "psd_matte":
        # every value but those the reference leaves to undefined behaviour
        a = py[..., 3:4].astype(np.float32)
        stored = RGBA[..., :3].astype(np.float32)
        # c / f + 255 (1 - 1 / f) < 0  <=>  c < 255 - A
        undefined = (a > 0) & (a < 255) & (stored < np.float32(255) - a)
        assert np.array_equal(np.where(undefined, 0, py[..., :3]), np.where(undefined, 0, ref[..., :3]))
        assert np.array_equal(py[..., 3], ref[..., 3]) and (py[..., :3][undefined] == 0).all()
    else:
        d = np.abs(py.astype(int) - ref.astype(int))
        assert d.max() <= rule[1] and d.mean() < 2.0, (d.max(), d.mean())


def test_mutated_files(stb, native, tmp_path):
    seeds = []
    for name, write, rule in CORPUS:
        path = str(tmp_path / name)
        write(path)
        seeds.append((path, rule))
    rng = np.random.default_rng(11)
    compared = 0
    for j in range(300):
        src, rule = seeds[int(rng.integers(len(seeds)))]
        data = bytearray(open(src, "rb").read())
        kind = int(rng.integers(5))
        if kind == 0:
            for i in rng.integers(0, len(data), 1 + int(rng.integers(8))):
                data[i] = int(rng.integers(256))
        elif kind == 1:
            for i in rng.integers(0, min(len(data), 80), 1 + int(rng.integers(4))):
                data[i] = int(rng.integers(256))
        elif kind == 2:
            data = data[:int(rng.integers(1, len(data)))]
        elif kind == 3:
            i = int(rng.integers(0, len(data)))
            data[i:i] = rng.integers(0, 256, int(rng.integers(1, 60)), dtype=np.uint8).tobytes()
        else:
            i = int(rng.integers(0, len(data) - 4))
            data[i:i + 2] = bytes([0xFF, int(rng.integers(256))])
        path = str(tmp_path / ("m%d%s" % (j, os.path.splitext(src)[1])))
        with open(path, "wb") as fh:
            fh.write(bytes(data))
        py, cli = _ours(native, path, tmp_path)
        assert (py is None) == (cli is None), path
        if py is None:
            continue
        assert np.array_equal(py, cli), path
        if rule != "equal":
            continue
        ref = _stb_read(stb, path)
        if ref is not None:
            assert ref.shape == py.shape and np.array_equal(ref, py), path
            compared += 1
    assert compared > 50
