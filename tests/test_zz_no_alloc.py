"""astc_sse_gpu_noalloc: the SSE reduction for callers that may not allocate.

Hosts that own the whole device-memory budget (engines, streaming and serving
processes that admit work by memory) cannot let a library call cudaMalloc;
this entry point keeps its scratch in a fixed static device array instead.
The test calls it through the C ABI, twice in a row on different images (so
the second call must not see the first call's partial sums), and checks each
result against the existing entry point astc_sse_gpu with the exact equality
the other SSE test uses.  It is collected last on purpose and needs no state
from earlier tests, so it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lib(native):
    lib = native.load_library()
    fn = lib.astc_sse_gpu_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                   ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return lib, fn


def _existing(lib, a, b, texels, stream):
    out = (ctypes.c_uint64 * 4)()
    st = lib.astc_sse_gpu(a.data_ptr(), b.data_ptr(), texels, 1, stream, out)   # ASTC_MEMORY_DEVICE
    assert st == 0, lib.astc_last_error()
    return list(out)


def test_noalloc_matches_existing_entry_point(native):
    import torch
    lib, fn = _lib(native)
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(20261203)
    shapes = [(300, 200), (1024, 777)]            # two calls in a row, different sizes
    for h, w in shapes:
        a = torch.from_numpy(rng.integers(0, 256, (h, w, 4), dtype=np.uint8)).cuda()
        b = torch.from_numpy(rng.integers(0, 256, (h, w, 4), dtype=np.uint8)).cuda()
        out = torch.full((4,), -1, dtype=torch.int64, device="cuda")
        st = fn(a.data_ptr(), b.data_ptr(), h * w, stream, out.data_ptr())
        assert st == 0, lib.astc_last_error()
        torch.cuda.synchronize()
        got = [int(v) for v in out.cpu().tolist()]
        want = _existing(lib, a, b, h * w, stream)
        assert got == want
        ref = ((a.cpu().numpy().astype(np.int64) - b.cpu().numpy().astype(np.int64)) ** 2)
        assert got == ref.reshape(-1, 4).sum(0).tolist()


def test_noalloc_rejects_sizes_beyond_the_limit(native):
    import torch
    lib, fn = _lib(native)
    a = torch.zeros((16, 16, 4), dtype=torch.uint8, device="cuda")
    out = torch.zeros((4,), dtype=torch.int64, device="cuda")
    st = fn(a.data_ptr(), a.data_ptr(), (1 << 28) + 1, None, out.data_ptr())
    assert st == native.Status.INVALID_ARG
    assert b"static scratch limit" in lib.astc_last_error()
