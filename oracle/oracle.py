"""ctypes binding of the CPU oracle (oracle/astc_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline / reference legs of ``bench.py``, always as the
reference the GPU results are compared with or as the timed CPU restatement --
never as the product path.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libastc_oracle.so")
_lock = threading.Lock()
_lib: ctypes.CDLL | None = None


class OracleOpts(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("block_dim", "has_alpha", "is_normal", "srgb", "border",
                                            "axis", "quality")]


class OracleTrace(ctypes.Structure):
    f, i, u = ctypes.c_float, ctypes.c_int, ctypes.c_uint32
    _fields_ = [("start_w", f), ("mean", f * 4), ("cov", f * 16), ("early_exit", i), ("min_len", f), ("axis", f * 4),
                ("tmin", f), ("tmax", f), ("e0_fit", f * 4), ("e1_fit", f * 4), ("s0", f), ("s1", f),
                ("swapped", i), ("e0", f * 4), ("e1", f * 4), ("wlen", f), ("wproj", f * 16),
                ("minw", f), ("maxw", f), ("inv", f), ("wR", f * 16), ("ep", u * 8), ("qw", u * 16),
                ("block", ctypes.c_uint8 * 16)]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++, OpenMP)."""
    src = os.path.join(HERE, "astc_oracle.cpp")
    hdr = os.path.join(HERE, "astc_oracle.h")
    stale = (not os.path.exists(LIB_PATH) or
             max(os.path.getmtime(src), os.path.getmtime(hdr)) > os.path.getmtime(LIB_PATH))
    if force or stale:
        res = subprocess.run(["make", "-B" if force else "-s", "-C", HERE], capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    return LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            vp, ip = ctypes.c_void_p, ctypes.c_int
            L.oracle_encode_fp32.argtypes = [vp, ip, ip, ctypes.POINTER(OracleOpts), vp, ip]
            L.oracle_encode_fp64.argtypes = [vp, ip, ip, ctypes.POINTER(OracleOpts), vp, ip]
            L.oracle_encode_block_fp32.argtypes = [vp, ip, ip, vp, vp, vp]
            L.oracle_assemble_symbolic.argtypes = [vp, vp, ip, vp]
            L.oracle_ise_encode.argtypes = [ip, ip, vp, vp]
            L.oracle_three_classes.argtypes = [ip, vp, vp, vp, ip]
            L.oracle_ise_decode.argtypes = [ip, ip, vp, ip, vp]
            L.oracle_ise_bits.argtypes = [ip, ip]
            for n in ("oracle_table_trits", "oracle_table_quints", "oracle_table_btq",
                      "oracle_table_scramble", "oracle_srgb_lut"):
                getattr(L, n).argtypes = [vp]
                getattr(L, n).restype = None
            L.oracle_decode.argtypes = [vp, ip, ip, ip, ip, ip, vp]
            L.oracle_decode_block.argtypes = [vp, ip, ip, ip, vp]
            L.oracle_unquant_weight.argtypes = [ip, ip]
            L.oracle_unquant_color.argtypes = [ip, ip]
            L.oracle_grid_taps.argtypes = [ip, vp, vp]
            L.oracle_grid_taps.restype = None
            L.oracle_flops_per_block.argtypes = [ip, ip, ip]
            L.oracle_flops_per_block.restype = ctypes.c_double
            L.oracle_endpoint_quant.argtypes = [ip, ip]
            L.oracle_search_block_fp32.argtypes = [vp, ip, ip, ip, ip, ip, vp, vp, vp, vp]
            L.oracle_find_seed.argtypes = [vp, ip, ip, vp, vp, ip]
            L.oracle_trace_block_fp32.argtypes = [vp, ip, ip, ctypes.c_float, ctypes.POINTER(OracleTrace)]
            _lib = L
    return _lib


def _opts(block_dim, has_alpha, is_normal, srgb, border, axis=0, quality=0) -> OracleOpts:
    return OracleOpts(int(block_dim), int(bool(has_alpha)), int(bool(is_normal)), int(bool(srgb)),
                      int(border), int(axis), int(quality))


def encode(rgba: np.ndarray, block_dim: int = 4, has_alpha: bool = False, is_normal: bool = False,
           srgb: bool = False, border: int = 0, threads: int = 0, fp64: bool = False,
           axis: int = 0, quality: int = 0) -> np.ndarray:
    """FP32 (or FP64 twin) oracle encode of a (H, W, 4) uint8 image -> (n, 16) uint8.

    axis 1 = max_accumulation_pixel_direction instead of the PCA, axis 2 = both,
    the fit whose fixed-mode block decodes better (the PCA on ties); quality 1 =
    search over the single-partition weight/endpoint ranges; 2 = the search
    from the better of both fits plus dual-plane blocks; 3 = 2 plus
    two-partition blocks; 4 = 3 plus three-partition blocks."""
    a = np.ascontiguousarray(rgba, dtype=np.uint8)
    h, w = a.shape[:2]
    nb = ((w + block_dim - 1) // block_dim) * ((h + block_dim - 1) // block_dim)
    out = np.empty((nb, 16), np.uint8)
    fn = lib().oracle_encode_fp64 if fp64 else lib().oracle_encode_fp32
    rc = fn(a.ctypes.data, w, h,
            ctypes.byref(_opts(block_dim, has_alpha, is_normal, srgb, border, axis, quality)),
            out.ctypes.data, threads)
    if rc != 0:
        raise ValueError(f"oracle encode rejected the arguments ({rc})")
    return out


def encode_block(texels: np.ndarray, block_dim: int, has_alpha: bool):
    t = np.ascontiguousarray(texels, dtype=np.float32).reshape(-1)
    ep = np.zeros(8, np.uint32)
    qw = np.zeros(16, np.uint32)
    out = np.zeros(16, np.uint8)
    rc = lib().oracle_encode_block_fp32(t.ctypes.data, block_dim, int(has_alpha), ep.ctypes.data,
                                        qw.ctypes.data, out.ctypes.data)
    assert rc == 0
    return ep, qw, out


def trace_block(texels: np.ndarray, block_dim: int, has_alpha: bool, start_w: float = 0.0) -> dict:
    """Intermediate values of the FP32 fixed-mode pipeline for one block
    (texels: N x 4 floats, 0..255): scalars as floats/ints, vectors as float32
    arrays; ep / qw the quantised endpoints and weights, block the assembled
    block.  start_w seeds the alpha of the power iteration's start vector
    (0 in the shader)."""
    t = np.ascontiguousarray(texels, dtype=np.float32).reshape(-1)
    tr = OracleTrace()
    rc = lib().oracle_trace_block_fp32(t.ctypes.data, block_dim, int(has_alpha), float(start_w),
                                       ctypes.byref(tr))
    if rc != 0:
        raise ValueError("bad trace arguments")
    out = {}
    for name, _ in OracleTrace._fields_:
        v = getattr(tr, name)
        out[name] = np.array(v[:], dtype=np.uint32 if name in ("ep", "qw") else np.uint8 if name == "block"
                 else np.float32) \
            if hasattr(v, "_length_") else v
    return out


def find_seed(texels: np.ndarray, block_dim: int, has_alpha: bool, target: np.ndarray, seeds) -> float | None:
    """The first start-vector alpha seed (of `seeds`) under which the FP32
    fixed-mode pipeline assembles exactly the block `target`, or None."""
    t = np.ascontiguousarray(texels, dtype=np.float32).reshape(-1)
    tg = np.ascontiguousarray(target, dtype=np.uint8).reshape(16)
    sd = np.ascontiguousarray(seeds, dtype=np.float32)
    i = lib().oracle_find_seed(t.ctypes.data, block_dim, int(has_alpha), tg.ctypes.data, sd.ctypes.data, len(sd))
    if i < -1:
        raise ValueError("bad seed-search arguments")
    return None if i < 0 else float(sd[i])


def assemble_symbolic(ep, qw, has_alpha: bool) -> np.ndarray:
    e = np.ascontiguousarray(ep, dtype=np.uint32)
    q = np.ascontiguousarray(qw, dtype=np.uint32)
    out = np.zeros(16, np.uint8)
    rc = lib().oracle_assemble_symbolic(e.ctypes.data, q.ctypes.data, int(has_alpha), out.ctypes.data)
    if rc != 0:
        raise ValueError("symbolic values out of range")
    return out


def ise_encode(quant: int, values) -> np.ndarray:
    v = np.ascontiguousarray(values, dtype=np.uint32)
    out = np.zeros(16, np.uint8)
    rc = lib().oracle_ise_encode(quant, len(v), v.ctypes.data, out.ctypes.data)
    if rc != 0:
        raise ValueError("bad ISE arguments")
    return out


def ise_decode(quant: int, count: int, data: np.ndarray, bit_offset: int = 0) -> np.ndarray:
    d = np.ascontiguousarray(data, dtype=np.uint8)
    out = np.zeros(max(count, 1), np.uint32)
    lib().oracle_ise_decode(quant, count, d.ctypes.data, bit_offset, out.ctypes.data)
    return out[:count]


def ise_bits(quant: int, count: int) -> int:
    return int(lib().oracle_ise_bits(quant, count))


def table(name: str, n: int, dtype=np.int32) -> np.ndarray:
    out = np.zeros(n, dtype)
    getattr(lib(), name)(out.ctypes.data)
    return out


def srgb_lut() -> np.ndarray:
    return table("oracle_srgb_lut", 256, np.float32)


def decode(blocks: np.ndarray, width: int, height: int, block_w: int, block_h: int | None = None,
           srgb: bool = False) -> tuple[np.ndarray, int]:
    block_h = block_h or block_w
    b = np.ascontiguousarray(blocks, dtype=np.uint8)
    out = np.zeros((height, width, 4), np.uint8)
    errors = lib().oracle_decode(b.ctypes.data, width, height, block_w, block_h, int(srgb),
                                 out.ctypes.data)
    if errors < 0:
        raise ValueError("bad decode arguments")
    return out, int(errors)


def decode_block(block: np.ndarray, block_w: int, block_h: int, srgb: bool = False):
    b = np.ascontiguousarray(block, dtype=np.uint8)
    out = np.zeros((block_h, block_w, 4), np.uint8)
    rc = lib().oracle_decode_block(b.ctypes.data, block_w, block_h, int(srgb), out.ctypes.data)
    return out, int(rc)


def unquant_weight(quant: int, v: int) -> int:
    return int(lib().oracle_unquant_weight(quant, v))


def unquant_color(quant: int, v: int) -> int:
    return int(lib().oracle_unquant_color(quant, v))


def grid_taps(g: int):
    idx = np.zeros(4, np.int32)
    wt = np.zeros(4, np.float32)
    lib().oracle_grid_taps(g, idx.ctypes.data, wt.ctypes.data)
    return idx, wt


def flops_per_block(block_dim: int, has_alpha: bool, is_normal: bool = False) -> float:
    return float(lib().oracle_flops_per_block(block_dim, int(has_alpha), int(is_normal)))


def endpoint_quant(wq: int, nvals: int) -> int:
    """Endpoint quant method the decoder derives for a 4x4 weight grid of
    quant method wq (single partition), or -1 for an illegal mode."""
    return int(lib().oracle_endpoint_quant(wq, nvals))


def three_classes(dim: int) -> list:
    """[(seed, m1, m2)] -- the oracle's three-partition pattern classes."""
    seeds = np.zeros(1024, np.int32)
    m1 = np.zeros(1024, np.uint64)
    m2 = np.zeros(1024, np.uint64)
    n = lib().oracle_three_classes(dim, seeds.ctypes.data, m1.ctypes.data, m2.ctypes.data, 1024)
    assert n > 0
    return [(int(seeds[i]), int(m1[i]), int(m2[i])) for i in range(n)]


def search_block(texels: np.ndarray, block_dim: int, has_alpha: bool, srgb: bool = False, axis: int = 0,
                 partitions: int = 0):
    """Search-mode FP32 encode of one block of fit-space texels (N x 4 floats);
    partitions: 0 = single partition only, 1 = also two-partition blocks, 2 =
    also three-partition blocks.

    Returns (block bytes, chosen weight quant method -- -1 for the fixed-mode
    block, 100 + wq for a two-partition block, 200 + 16 * pc + wq for a
    dual-plane block, 300 + 16 * rank + wq for a three-partition block --, the
    squared error of its decode against the texels rounded to bytes, the
    fixed-mode block's)."""
    t = np.ascontiguousarray(texels, dtype=np.float32).reshape(-1)
    out = np.zeros(16, np.uint8)
    wq = ctypes.c_int(0)
    err = ctypes.c_uint32(0)
    err_fixed = ctypes.c_uint32(0)
    rc = lib().oracle_search_block_fp32(t.ctypes.data, block_dim, int(has_alpha), int(srgb), int(axis),
                                        int(partitions), out.ctypes.data, ctypes.byref(wq), ctypes.byref(err),
                                        ctypes.byref(err_fixed))
    assert rc == 0
    return out, wq.value, err.value, err_fixed.value
