"""GB300-native ASTC LDR block encoder (sm_103a CUDA behind a C ABI).

Python mirror of the reference's host interface (niepp/astc_encoder):

* :class:`EncodeOption`   -- ``encode_option`` (astc_encode.h:14-28)
* :func:`encode_astc`     -- ``encode_astc`` + ``read_gpu``
                             (astc_encode.h:87-194, astc_save.h:34-50)
* :func:`save_astc`       -- ``save_astc`` (astc_save.h:52-76)

Everything here is a thin ``ctypes`` layer over ``libastc_gb300.so``
(``include/astc_gb300.h``); the encode runs in the library's CUDA kernels.
There is no CPU fallback: if the library is missing, every call raises.
"""
from __future__ import annotations

import ctypes
import dataclasses
import enum
import os
from typing import Any

import numpy as np

__all__ = [
    "AstcError", "Status", "Border", "Precision", "Memory", "Axis", "Quality", "EncodeOption", "AstcOpts",
    "library_path", "load_library", "encoded_size", "encode", "encode_astc", "encode_device",
    "save_astc", "load_astc", "decode", "decode_device", "sse", "psnr_from_sse",
    "kernel_launch_count", "shutdown",
]

_PKG = os.path.dirname(os.path.abspath(__file__))


class Status(enum.IntEnum):
    OK = 0
    INVALID_ARG = 1
    UNSUPPORTED = 2
    CUDA = 3
    OUT_OF_MEMORY = 4
    IO = 5
    TIMEOUT = 6
    BUSY = 7
    CANCELLED = 8
    FORMAT = 9


class Border(enum.IntEnum):
    ZERO = 0
    CLAMP = 1


class Precision(enum.IntEnum):
    FP32 = 0
    HALF2 = 1


class Memory(enum.IntEnum):
    HOST = 0
    DEVICE = 1


class Axis(enum.IntEnum):
    PCA = 0                 # principal_component_analysis (ASTC_Encode.hlsl:514)
    MAX_ACCUMULATION = 1    # max_accumulation_pixel_direction (170-227, unused there)
    BEST = 2                # both fits, the better fixed-mode block (PCA on ties)


class Quality(enum.IntEnum):
    FAST = 0                # the reference's fixed mode (518-522)
    SEARCH = 1              # every single-partition 4x4-grid mode, least decoded error
    THOROUGH = 2            # SEARCH from the better of the PCA and max-accumulation fits, plus dual-plane blocks
    PARTITIONS = 3          # THOROUGH plus two-partition blocks
    THREE_PARTITIONS = 4    # PARTITIONS plus three-partition blocks (RGB input)


class AstcError(RuntimeError):
    def __init__(self, status: int, message: str):
        self.status = Status(status) if status in Status._value2member_map_ else status
        super().__init__(f"{self.status!s}: {message}")


class AstcOpts(ctypes.Structure):
    """``astc_opts`` of include/astc_gb300.h."""
    _fields_ = [
        ("block_dim", ctypes.c_int),
        ("has_alpha", ctypes.c_int),
        ("is_normal", ctypes.c_int),
        ("srgb", ctypes.c_int),
        ("border", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("memory", ctypes.c_int),
        ("stream", ctypes.c_void_p),
        ("axis", ctypes.c_int),
        ("quality", ctypes.c_int),
    ]


@dataclasses.dataclass
class EncodeOption:
    """Mirror of the reference's ``encode_option`` (astc_encode.h:14-28).

    The reference derives the block size from ``is4x4`` only and never reads
    ``is6x6``, so its ``-6x6`` flag is a no-op; here ``is6x6`` selects 6x6
    (the README's intent).
    """
    is4x4: bool = True
    is6x6: bool = False
    is_normal_map: bool = False
    has_alpha: bool = False
    srgb: bool = False

    @property
    def block_dim(self) -> int:
        return 6 if (self.is6x6 or not self.is4x4) else 4


def library_path() -> str:
    return os.path.join(_PKG, "_lib", "libastc_gb300.so")


_LIB: ctypes.CDLL | None = None


def load_library() -> ctypes.CDLL:
    """Load libastc_gb300.so (built in-tree by astc_encoder_gb300.build)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not os.path.exists(path):
        raise AstcError(Status.UNSUPPORTED,
                        f"native library not built: {path} (run python -m astc_encoder_gb300.build)")
    lib = ctypes.CDLL(path)
    u8p, vp, sz = ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t
    lib.astc_opts_init.argtypes = [ctypes.POINTER(AstcOpts)]
    lib.astc_opts_init.restype = None
    lib.astc_encoded_size.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
    lib.astc_encoded_size.restype = sz
    lib.astc_encode_gpu.argtypes = [u8p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(AstcOpts), u8p]
    lib.astc_encode_gpu.restype = ctypes.c_int
    lib.astc_encode_gpu_pitched.argtypes = [u8p, ctypes.c_int, ctypes.c_int, sz,
                                            ctypes.POINTER(AstcOpts), u8p]
    lib.astc_encode_gpu_pitched.restype = ctypes.c_int
    lib.astc_save_file.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_int, u8p, sz]
    lib.astc_save_file.restype = ctypes.c_int
    ip = ctypes.POINTER(ctypes.c_int)
    lib.astc_load_file.argtypes = [ctypes.c_char_p, ip, ip, ip, ip, u8p, sz, ctypes.POINTER(sz)]
    lib.astc_load_file.restype = ctypes.c_int
    lib.astc_decode_gpu.argtypes = [u8p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_int, vp, u8p]
    lib.astc_decode_gpu.restype = ctypes.c_int
    lib.astc_sse_gpu.argtypes = [u8p, u8p, sz, ctypes.c_int, vp, ctypes.POINTER(ctypes.c_uint64)]
    lib.astc_sse_gpu.restype = ctypes.c_int
    lib.astc_normal_sse_gpu.argtypes = [u8p, u8p, sz, ctypes.c_int, vp, ctypes.POINTER(ctypes.c_double)]
    lib.astc_normal_sse_gpu.restype = ctypes.c_int
    lib.astc_last_error.argtypes = []
    lib.astc_last_error.restype = ctypes.c_char_p
    lib.astc_status_string.argtypes = [ctypes.c_int]
    lib.astc_status_string.restype = ctypes.c_char_p
    lib.astc_kernel_launch_count.argtypes = []
    lib.astc_kernel_launch_count.restype = ctypes.c_uint64
    lib.astc_shutdown.argtypes = []
    lib.astc_shutdown.restype = None
    lib.astc_autotune.argtypes = [ctypes.c_int] * 6 + [ctypes.POINTER(TuneResult)]
    lib.astc_autotune.restype = ctypes.c_int
    lib.astc_set_kernel_choice.argtypes = [ctypes.c_int] * 6
    lib.astc_set_kernel_choice.restype = ctypes.c_int
    lib.astc_get_kernel_choice.argtypes = [ctypes.c_int] * 4 + [ip, ip]
    lib.astc_get_kernel_choice.restype = ctypes.c_int
    lib.astc_get_kernel_choice_for_size.argtypes = [ctypes.c_int] * 6 + [ip, ip]
    lib.astc_get_kernel_choice_for_size.restype = ctypes.c_int
    lib.astc_batch_create.argtypes = [ctypes.c_int, ctypes.c_longlong, ctypes.POINTER(ctypes.c_void_p)]
    lib.astc_batch_create.restype = ctypes.c_int
    lib.astc_batch_encode.argtypes = [ctypes.c_void_p, ctypes.POINTER(BatchItem), ctypes.c_int,
                                      ctypes.c_int, ctypes.c_void_p]
    lib.astc_batch_encode.restype = ctypes.c_int
    lib.astc_batch_encode_quality.argtypes = [ctypes.c_void_p, ctypes.POINTER(BatchItem), ctypes.c_int,
                                              ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    lib.astc_batch_encode_quality.restype = ctypes.c_int
    lib.astc_batch_destroy.argtypes = [ctypes.c_void_p]
    lib.astc_batch_destroy.restype = ctypes.c_int
    lib.astc_mip_levels.argtypes = [ctypes.c_int, ctypes.c_int]
    lib.astc_mip_levels.restype = ctypes.c_int
    lib.astc_mip_chain_bytes.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
    lib.astc_mip_chain_bytes.restype = ctypes.c_size_t
    lib.astc_generate_mips.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.astc_generate_mips.restype = ctypes.c_int
    lib.astc_get_device_caps.argtypes = [ctypes.POINTER(DeviceCaps)]
    lib.astc_get_device_caps.restype = ctypes.c_int
    vpp = ctypes.POINTER(ctypes.c_void_p)
    lib.astc_server_create.argtypes = [ctypes.POINTER(ServerConfig), vpp]
    lib.astc_server_create.restype = ctypes.c_int
    lib.astc_server_submit.argtypes = [ctypes.c_void_p, ctypes.POINTER(Request),
                                       ctypes.POINTER(ctypes.c_uint64)]
    lib.astc_server_submit.restype = ctypes.c_int
    lib.astc_server_wait.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int,
                                     ctypes.POINTER(RequestStats)]
    lib.astc_server_wait.restype = ctypes.c_int
    lib.astc_server_cancel.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
    lib.astc_server_cancel.restype = ctypes.c_int
    dp = ctypes.POINTER(ctypes.c_double)
    lib.astc_server_replay.argtypes = [ctypes.c_void_p, ctypes.POINTER(Request), dp, ctypes.c_int, dp, dp]
    lib.astc_server_replay.restype = ctypes.c_int
    lib.astc_server_get_stats.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ServerStats)]
    lib.astc_server_get_stats.restype = ctypes.c_int
    lib.astc_server_destroy.argtypes = [ctypes.c_void_p]
    lib.astc_server_destroy.restype = ctypes.c_int
    _LIB = lib
    return lib


class DeviceCaps(ctypes.Structure):
    """``astc_device_caps`` of include/astc_gb300.h."""
    _fields_ = [(n, ctypes.c_int) for n in ("sm_count", "l2_bytes", "unified_addressing", "can_map_host_memory",
                                            "pageable_memory_access", "pageable_uses_host_page_tables",
                                            "zero_copy", "pageable_in_place")]


def device_caps() -> dict:
    c = DeviceCaps()
    _check(load_library().astc_get_device_caps(ctypes.byref(c)))
    return {n: getattr(c, n) for n, _ in DeviceCaps._fields_}


class ServerConfig(ctypes.Structure):
    """``astc_server_config`` of include/astc_gb300.h."""
    _fields_ = [("pool_bytes", ctypes.c_size_t), ("max_batch", ctypes.c_int), ("inflight", ctypes.c_int),
                ("precision", ctypes.c_int), ("mode", ctypes.c_int), ("quality", ctypes.c_int)]


class Request(ctypes.Structure):
    """``astc_request`` of include/astc_gb300.h (host buffers)."""
    _fields_ = [("rgba8", ctypes.c_void_p), ("row_pitch", ctypes.c_size_t), ("width", ctypes.c_int),
                ("height", ctypes.c_int), ("block_dim", ctypes.c_int), ("has_alpha", ctypes.c_int),
                ("is_normal", ctypes.c_int), ("srgb", ctypes.c_int), ("border", ctypes.c_int),
                ("out", ctypes.c_void_p)]


class RequestStats(ctypes.Structure):
    _fields_ = [("submit_us", ctypes.c_double), ("admit_us", ctypes.c_double), ("done_us", ctypes.c_double),
                ("status", ctypes.c_int)]


class ServerStats(ctypes.Structure):
    """``astc_server_stats`` of include/astc_gb300.h."""
    _fields_ = [("launches", ctypes.c_longlong), ("requests", ctypes.c_longlong),
                ("max_requests_per_launch", ctypes.c_int), ("device_busy_s", ctypes.c_double),
                ("device_overlap_s", ctypes.c_double), ("device_slot_s", ctypes.c_double),
                ("device_span_s", ctypes.c_double)]


SERVE_BATCHED, SERVE_PER_REQUEST = 0, 1


def make_request(rgba_ptr: int, width: int, height: int, out_ptr: int, block_dim: int = 4,
                 has_alpha: bool = False, is_normal: bool = False, srgb: bool = False,
                 border: int = Border.ZERO, row_pitch: int = 0) -> Request:
    return Request(rgba_ptr, row_pitch, width, height, block_dim, int(has_alpha), int(is_normal), int(srgb),
                   int(border), out_ptr)


class Server:
    """Continuous-batching request server (astc_server_*) over host buffers."""

    def __init__(self, pool_bytes: int = 2 << 30, max_batch: int = 256, inflight: int = 3,
                 precision: int = Precision.FP32, mode: int = SERVE_BATCHED, quality: int = Quality.FAST):
        self._lib = load_library()
        cfg = ServerConfig(pool_bytes, max_batch, inflight, int(precision), int(mode), int(quality))
        h = ctypes.c_void_p()
        _check(self._lib.astc_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h

    def submit(self, req: Request) -> int:
        t = ctypes.c_uint64()
        _check(self._lib.astc_server_submit(self._h, ctypes.byref(req), ctypes.byref(t)))
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1) -> RequestStats:
        st = RequestStats()
        _check(self._lib.astc_server_wait(self._h, ticket, timeout_ms, ctypes.byref(st)))
        return st

    def try_wait(self, ticket: int, timeout_ms: int) -> tuple[int, RequestStats]:
        st = RequestStats()
        rc = self._lib.astc_server_wait(self._h, ticket, timeout_ms, ctypes.byref(st))
        return rc, st

    def cancel(self, ticket: int) -> int:
        return int(self._lib.astc_server_cancel(self._h, ticket))

    def replay(self, requests: list[Request], arrival_us) -> tuple[np.ndarray, float]:
        n = len(requests)
        arr = (Request * max(1, n))(*requests)
        arrival = np.ascontiguousarray(arrival_us, dtype=np.float64)
        lat = np.zeros(n, np.float64)
        wall = ctypes.c_double()
        dp = ctypes.POINTER(ctypes.c_double)
        _check(self._lib.astc_server_replay(self._h, arr, arrival.ctypes.data_as(dp), n,
                                            lat.ctypes.data_as(dp), ctypes.byref(wall)))
        return lat, wall.value

    def stats(self, reset: bool = False) -> dict:
        """Device-side record of the launches retired since the last reset."""
        st = ServerStats()
        _check(self._lib.astc_server_get_stats(self._h, int(reset), ctypes.byref(st)))
        return {name: getattr(st, name) for name, _ in ServerStats._fields_}

    def close(self) -> None:
        if self._h:
            self._lib.astc_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


class BatchItem(ctypes.Structure):
    """``astc_batch_item`` of include/astc_gb300.h."""
    _fields_ = [("rgba8", ctypes.c_void_p), ("row_pitch", ctypes.c_size_t), ("width", ctypes.c_int),
                ("height", ctypes.c_int), ("block_dim", ctypes.c_int), ("has_alpha", ctypes.c_int),
                ("is_normal", ctypes.c_int), ("srgb", ctypes.c_int), ("border", ctypes.c_int),
                ("out", ctypes.c_void_p)]


class Batch:
    """Batched encoder handle (astc_batch_*): one graph launch for many textures.

    ``items`` are dicts or tuples (rgba8_ptr, width, height, out_ptr, options...)
    of device pointers; see :meth:`encode`."""

    def __init__(self, max_textures: int, max_blocks: int):
        self._lib = load_library()
        h = ctypes.c_void_p()
        _check(self._lib.astc_batch_create(max_textures, max_blocks, ctypes.byref(h)))
        self._h = h

    def encode(self, items: list[dict], precision: int = Precision.FP32, stream: int | None = None,
               quality: int = Quality.FAST) -> None:
        arr = (BatchItem * max(1, len(items)))()
        for i, it in enumerate(items):
            arr[i] = BatchItem(it["rgba8"], it.get("row_pitch", 0), it["width"], it["height"],
                               it.get("block_dim", 4), int(it.get("has_alpha", False)),
                               int(it.get("is_normal", False)), int(it.get("srgb", False)),
                               int(it.get("border", Border.ZERO)), it["out"])
        if quality == Quality.FAST:
            _check(self._lib.astc_batch_encode(self._h, arr, len(items), int(precision), stream or None))
        else:
            _check(self._lib.astc_batch_encode_quality(self._h, arr, len(items), int(precision), int(quality),
                                                       stream or None))

    def close(self) -> None:
        if self._h:
            self._lib.astc_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


def mip_levels(width: int, height: int) -> int:
    return int(load_library().astc_mip_levels(width, height))


def mip_chain_bytes(width: int, height: int, levels: int) -> int:
    return int(load_library().astc_mip_chain_bytes(width, height, levels))


def mip_sizes(width: int, height: int, levels: int) -> list[tuple[int, int]]:
    """Sizes of levels 0..levels-1 (level l+1 = max(1, w/2) x max(1, h/2))."""
    out = [(width, height)]
    for _ in range(1, levels):
        width, height = max(1, width // 2), max(1, height // 2)
        out.append((width, height))
    return out


def generate_mips(rgba_ptr: int, width: int, height: int, levels: int, out_ptr: int, srgb: bool = False,
                  stream: int | None = None) -> None:
    """Box-filtered levels 1..levels-1 of a device RGBA8 image into `out_ptr`."""
    _check(load_library().astc_generate_mips(rgba_ptr, width, height, levels, int(srgb), out_ptr,
                                             stream or None))


class TuneResult(ctypes.Structure):
    """``astc_tune_result`` of include/astc_gb300.h."""
    _fields_ = [("store", ctypes.c_int), ("threads", ctypes.c_int), ("best_us", ctypes.c_float),
                ("default_us", ctypes.c_float)]


def autotune(block_dim: int, has_alpha: bool = False, is_normal: bool = False, srgb: bool = False,
             width: int = 2048, height: int = 2048) -> TuneResult:
    """Time every kernel variant for a format and install the fastest."""
    r = TuneResult()
    _check(load_library().astc_autotune(block_dim, int(has_alpha), int(is_normal), int(srgb), width,
                                        height, ctypes.byref(r)))
    return r


def set_kernel_choice(block_dim: int, has_alpha: bool, is_normal: bool, srgb: bool, store: int,
                      threads: int) -> None:
    _check(load_library().astc_set_kernel_choice(block_dim, int(has_alpha), int(is_normal), int(srgb),
                                                 store, threads))


def get_kernel_choice(block_dim: int, has_alpha: bool, is_normal: bool, srgb: bool) -> tuple[int, int]:
    s, t = ctypes.c_int(), ctypes.c_int()
    _check(load_library().astc_get_kernel_choice(block_dim, int(has_alpha), int(is_normal), int(srgb),
                                                 ctypes.byref(s), ctypes.byref(t)))
    return s.value, t.value


def get_kernel_choice_for_size(block_dim: int, has_alpha: bool, is_normal: bool, srgb: bool, width: int,
                               height: int) -> tuple[int, int]:
    """(store, threads) astc_encode_gpu uses for a texture of this size."""
    s, t = ctypes.c_int(), ctypes.c_int()
    _check(load_library().astc_get_kernel_choice_for_size(block_dim, int(has_alpha), int(is_normal), int(srgb),
                                                          width, height, ctypes.byref(s), ctypes.byref(t)))
    return s.value, t.value


def _check(status: int) -> None:
    if status != 0:
        msg = load_library().astc_last_error().decode(errors="replace")
        raise AstcError(status, msg)


def make_opts(block_dim: int = 4, has_alpha: bool = False, is_normal: bool = False,
              srgb: bool = False, border: int = Border.ZERO, precision: int = Precision.FP32,
              memory: int = Memory.HOST, stream: int | None = None, axis: int = Axis.PCA,
              quality: int = Quality.FAST) -> AstcOpts:
    o = AstcOpts()
    load_library().astc_opts_init(ctypes.byref(o))
    o.block_dim = int(block_dim)
    o.has_alpha = int(bool(has_alpha))
    o.is_normal = int(bool(is_normal))
    o.srgb = int(bool(srgb))
    o.border = int(border)
    o.precision = int(precision)
    o.memory = int(memory)
    o.stream = stream or None
    o.axis = int(axis)
    o.quality = int(quality)
    return o


def encoded_size(width: int, height: int, block_dim: int) -> int:
    return 16 * ((width + block_dim - 1) // block_dim) * ((height + block_dim - 1) // block_dim)


def encode(rgba: np.ndarray, block_dim: int = 4, has_alpha: bool = False, is_normal: bool = False,
           srgb: bool = False, border: int = Border.ZERO, precision: int = Precision.FP32,
           out: np.ndarray | None = None, axis: int = Axis.PCA,
           quality: int = Quality.FAST) -> np.ndarray:
    """Encode a host (H, W, 4) uint8 image; returns (nblocks, 16) uint8 blocks."""
    a = np.asarray(rgba)
    if a.dtype != np.uint8 or a.ndim != 3 or a.shape[2] != 4:
        raise AstcError(Status.INVALID_ARG, "rgba must be a (H, W, 4) uint8 array")
    h, w = a.shape[:2]
    if h == 0 or w == 0:
        raise AstcError(Status.INVALID_ARG, "empty image")
    a = np.ascontiguousarray(a)
    n = encoded_size(w, h, block_dim)
    if out is None:
        out = np.empty((n // 16, 16), np.uint8)
    elif out.nbytes != n or not out.flags.c_contiguous or out.dtype != np.uint8:
        raise AstcError(Status.INVALID_ARG, "out has the wrong size or layout")
    o = make_opts(block_dim, has_alpha, is_normal, srgb, border, precision, Memory.HOST, None, axis, quality)
    _check(load_library().astc_encode_gpu(a.ctypes.data, w, h, ctypes.byref(o), out.ctypes.data))
    return out


def encode_astc(rgba: np.ndarray, option: EncodeOption | None = None, **kw: Any) -> np.ndarray:
    """The reference's encode_astc + read_gpu: image in, block bytes out."""
    option = option or EncodeOption()
    return encode(rgba, block_dim=option.block_dim, has_alpha=option.has_alpha,
                  is_normal=option.is_normal_map, srgb=option.srgb, **kw)


def encode_device(rgba_ptr: int, width: int, height: int, out_ptr: int, block_dim: int = 4,
                  has_alpha: bool = False, is_normal: bool = False, srgb: bool = False,
                  border: int = Border.ZERO, precision: int = Precision.FP32,
                  stream: int | None = None, row_pitch: int | None = None, axis: int = Axis.PCA,
                  quality: int = Quality.FAST) -> None:
    """Encode from device memory to device memory (pointers, e.g. tensor.data_ptr()).

    With ``stream`` (a cudaStream_t handle) the call is asynchronous on it.
    """
    o = make_opts(block_dim, has_alpha, is_normal, srgb, border, precision, Memory.DEVICE, stream, axis,
                  quality)
    pitch = row_pitch if row_pitch is not None else width * 4
    _check(load_library().astc_encode_gpu_pitched(rgba_ptr, width, height, pitch, ctypes.byref(o),
                                                  out_ptr))


def save_astc(path: str, xdim: int, ydim: int, xsize: int, ysize: int, blocks: np.ndarray) -> None:
    """The reference's save_astc(path, xdim, ydim, xsize, ysize, buf, size)."""
    b = np.ascontiguousarray(blocks, dtype=np.uint8)
    _check(load_library().astc_save_file(os.fsencode(path), xdim, ydim, xsize, ysize,
                                         b.ctypes.data, b.nbytes))


def load_astc(path: str) -> tuple[np.ndarray, int, int, int, int]:
    """Read a .astc file: (blocks (n,16), block_x, block_y, width, height)."""
    lib = load_library()
    bx, by, w, h = (ctypes.c_int() for _ in range(4))
    size = ctypes.c_size_t()
    _check(lib.astc_load_file(os.fsencode(path), ctypes.byref(bx), ctypes.byref(by), ctypes.byref(w),
                              ctypes.byref(h), None, 0, ctypes.byref(size)))
    out = np.empty((size.value // 16, 16), np.uint8)
    _check(lib.astc_load_file(os.fsencode(path), ctypes.byref(bx), ctypes.byref(by), ctypes.byref(w),
                              ctypes.byref(h), out.ctypes.data, out.nbytes, ctypes.byref(size)))
    return out, bx.value, by.value, w.value, h.value


def decode(blocks: np.ndarray, width: int, height: int, block_w: int, block_h: int | None = None,
           srgb: bool = False) -> np.ndarray:
    """Integer-only ASTC LDR decode on the GPU; returns (H, W, 4) uint8."""
    block_h = block_h or block_w
    b = np.ascontiguousarray(blocks, dtype=np.uint8)
    need = encoded_size_xy(width, height, block_w, block_h)
    if b.nbytes != need:
        raise AstcError(Status.INVALID_ARG, "blocks has the wrong size")
    out = np.empty((height, width, 4), np.uint8)
    _check(load_library().astc_decode_gpu(b.ctypes.data, width, height, block_w, block_h, int(srgb),
                                          Memory.HOST, None, out.ctypes.data))
    return out


def decode_device(blocks_ptr: int, width: int, height: int, block_w: int, block_h: int,
                  out_ptr: int, srgb: bool = False, stream: int | None = None) -> None:
    _check(load_library().astc_decode_gpu(blocks_ptr, width, height, block_w, block_h, int(srgb),
                                          Memory.DEVICE, stream or None, out_ptr))


def encoded_size_xy(width: int, height: int, bw: int, bh: int) -> int:
    return 16 * ((width + bw - 1) // bw) * ((height + bh - 1) // bh)


def sse(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Per-channel (R, G, B, A) sum of squared differences of two RGBA8 images, on the GPU."""
    x = np.ascontiguousarray(a, dtype=np.uint8)
    y = np.ascontiguousarray(b, dtype=np.uint8)
    if x.shape != y.shape or x.size % 4:
        raise AstcError(Status.INVALID_ARG, "images must have the same RGBA8 shape")
    res = (ctypes.c_uint64 * 4)()
    _check(load_library().astc_sse_gpu(x.ctypes.data, y.ctypes.data, x.size // 4, Memory.HOST, None,
                                       res))
    return np.array(list(res), dtype=np.uint64)


def normal_sse(a: np.ndarray, b: np.ndarray) -> float:
    """Squared error of two -norm layout RGBA8 normal maps on their rebuilt
    unit normals (z = sqrt(max(0, 1 - x^2 - y^2))), components scaled by 127.5;
    PSNR over 3 values per texel with peak 255.  On the GPU."""
    x = np.ascontiguousarray(a, dtype=np.uint8)
    y = np.ascontiguousarray(b, dtype=np.uint8)
    if x.shape != y.shape or x.size % 4:
        raise AstcError(Status.INVALID_ARG, "images must have the same RGBA8 shape")
    res = ctypes.c_double(0.0)
    _check(load_library().astc_normal_sse_gpu(x.ctypes.data, y.ctypes.data, x.size // 4, Memory.HOST, None,
                                              ctypes.byref(res)))
    return float(res.value)


def normal_sse_numpy(a: np.ndarray, b: np.ndarray) -> float:
    """The same measure as normal_sse in numpy (float64), for checking."""
    def rebuilt(img):
        xy = img[..., :2].astype(np.float64) * (2.0 / 255.0) - 1.0
        z = np.sqrt(np.maximum(0.0, 1.0 - xy[..., 0] ** 2 - xy[..., 1] ** 2))
        return np.concatenate([xy, z[..., None]], axis=-1)
    d = (rebuilt(np.asarray(a)) - rebuilt(np.asarray(b))) * 127.5
    return float(np.sum(d * d))


def srgb_texel_values() -> np.ndarray:
    """The texel value the encoder fits for each sRGB code (RGB channels):
    float(IEC 61966-2-1 sRGB -> linear, evaluated in double) * 255 in float."""
    x = np.arange(256, dtype=np.float64) / 255.0
    lin = np.where(x <= 0.04045, x / 12.92, ((x + 0.055) / 1.055) ** 2.4)
    return lin.astype(np.float32) * np.float32(255.0)


def fitted_reference(rgba: np.ndarray, srgb: bool, is_normal: bool = False) -> np.ndarray:
    """RGBA8 image in the space the encoder fits: sRGB codes linearised (and
    rounded back to bytes) when `srgb`, B = A = 255 for normal maps.  This is
    what a linear decode of the blocks approximates, so PSNR is taken here."""
    ref = np.array(rgba, dtype=np.uint8, copy=True)
    if srgb:
        lut = np.clip(np.rint(srgb_texel_values()), 0, 255).astype(np.uint8)
        ref[..., :3] = lut[ref[..., :3]]
    if is_normal:
        ref[..., 2:] = 255
    return ref


def psnr_from_sse(sse_value: float, count: int, peak: float = 255.0) -> float:
    if sse_value == 0:
        return float("inf")
    return float(10.0 * np.log10(peak * peak * count / float(sse_value)))


def kernel_launch_count() -> int:
    return int(load_library().astc_kernel_launch_count())


def shutdown() -> None:
    if _LIB is not None:
        _LIB.astc_shutdown()
