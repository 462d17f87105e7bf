"""The continuous-batching server (astc_server_*).

The key property: a request's blocks are the same whether it is served alone
or in the middle of a stream of other requests of other sizes and formats
(exactly -- the tolerance is zero, since every path encodes each block with
the same arithmetic), in both serving modes and both precisions.
Failure handling is tested on the host: a request too large for the pool is
refused, a queued request can be cancelled, waits are bounded, and a server
shut down with work queued drains it.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FORMATS = [dict(block_dim=4), dict(block_dim=6, has_alpha=True, srgb=True, border=1),
           dict(block_dim=4, is_normal=True), dict(block_dim=4, has_alpha=True)]


def _img(h, w, seed):
    rng = np.random.default_rng(seed)
    img = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    img[h // 4:h // 2, w // 3:w // 2] = (10, 100, 200, 255)
    return img


class _Req:
    """Host buffers of one request (kept alive by the test)."""

    def __init__(self, native, h, w, seed, opts):
        self.img = _img(h, w, seed)
        self.opts = opts
        d = opts["block_dim"]
        self.out = np.zeros((((w + d - 1) // d) * ((h + d - 1) // d), 16), np.uint8)
        self.req = native.make_request(self.img.ctypes.data, w, h, self.out.ctypes.data, **opts)


def _mix(native, n, seed, max_side=300):
    rng = np.random.default_rng(seed)
    return [_Req(native, int(rng.integers(1, max_side)), int(rng.integers(1, max_side)), seed * 1000 + i,
                 FORMATS[i % len(FORMATS)]) for i in range(n)]


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("precision", [0, 1])
def test_alone_equals_in_the_mix(native, oracle, mode, precision):
    probe = _Req(native, 150, 221, 7, dict(block_dim=6, has_alpha=True, srgb=True, border=1))
    with native.Server(pool_bytes=64 << 20, max_batch=16, inflight=3, precision=precision, mode=mode) as srv:
        srv.wait(srv.submit(probe.req))
        alone = probe.out.copy()
        probe.out[:] = 0
        mix = _mix(native, 60, seed=mode * 2 + precision)
        tickets = [srv.submit(r.req) for r in mix[:30]]
        t_probe = srv.submit(probe.req)
        tickets += [srv.submit(r.req) for r in mix[30:]]
        srv.wait(t_probe)
        for t in tickets:
            srv.wait(t)
    assert np.array_equal(probe.out, alone)
    assert np.array_equal(alone, native.encode(probe.img, precision=precision, **probe.opts))
    for r in mix:
        assert np.array_equal(r.out, native.encode(r.img, precision=precision, **r.opts)), r.opts
    if precision == 0:
        assert np.array_equal(alone, oracle.encode(probe.img, **probe.opts))


def test_server_device_stats(native):
    """The device-side record: every retired launch and request counted,
    busy time within the span, overlap within busy, reset clears it."""
    with native.Server(pool_bytes=64 << 20, max_batch=8, inflight=3) as srv:
        mix = _mix(native, 40, seed=21, max_side=300)
        srv.stats(reset=True)
        tickets = [srv.submit(r.req) for r in mix]
        for t in tickets:
            srv.wait(t)
        st = srv.stats(reset=True)
        assert st["requests"] == len(mix)
        assert 1 <= st["launches"] <= len(mix)
        assert 1 <= st["max_requests_per_launch"] <= 8
        assert 0 < st["device_busy_s"] <= st["device_span_s"] + 1e-9
        assert 0 <= st["device_overlap_s"] <= st["device_busy_s"] + 1e-9
        assert st["device_slot_s"] >= st["device_busy_s"] - 1e-9
        assert srv.stats()["launches"] == 0
    with native.Server(pool_bytes=64 << 20, inflight=2, mode=1) as srv:
        mix = _mix(native, 12, seed=22, max_side=200)
        for t in [srv.submit(r.req) for r in mix]:
            srv.wait(t)
        st = srv.stats()
        assert st["launches"] == st["requests"] == 12 and st["max_requests_per_launch"] == 1


@pytest.mark.parametrize("mode", [0, 1])
def test_server_quality_mode(native, mode):
    """A THOROUGH server returns each request's astc_encode_gpu blocks with
    that quality, batched or per request; HALF2 with it is refused."""
    with native.Server(pool_bytes=32 << 20, max_batch=8, inflight=2, mode=mode, quality=2) as srv:
        mix = _mix(native, 16, seed=40 + mode, max_side=120)
        tickets = [srv.submit(r.req) for r in mix]
        for t in tickets:
            srv.wait(t)
    for r in mix:
        assert np.array_equal(r.out, native.encode(r.img, quality=2, **r.opts)), r.opts
    with pytest.raises(native.AstcError) as e:
        native.Server(pool_bytes=1 << 24, precision=1, quality=2)
    assert e.value.status == native.Status.UNSUPPORTED


def test_admission_by_memory_with_a_small_pool(native):
    # a 2 MiB pool holds only a few of these requests at a time; the rest wait
    mix = _mix(native, 40, seed=11, max_side=400)
    with native.Server(pool_bytes=2 << 20, max_batch=8, inflight=2) as srv:
        stats = [srv.wait(t) for t in [srv.submit(r.req) for r in mix]]
    for r in mix:
        assert np.array_equal(r.out, native.encode(r.img, **r.opts))
    assert all(s.status == 0 and s.submit_us <= s.admit_us <= s.done_us for s in stats)


def test_oversized_request_is_refused(native):
    big = _Req(native, 1024, 1024, 1, dict(block_dim=4))          # 4 MiB in + 1 MiB out
    with native.Server(pool_bytes=2 << 20, max_batch=4, inflight=1) as srv:
        with pytest.raises(native.AstcError) as e:
            srv.submit(big.req)
        assert e.value.status == native.Status.BUSY
        small = _Req(native, 64, 64, 2, dict(block_dim=4))
        srv.wait(srv.submit(small.req))                            # still serving
    assert np.array_equal(small.out, native.encode(small.img, block_dim=4))


def test_cancel_and_bounded_wait(native):
    mix = _mix(native, 30, seed=5, max_side=500)
    with native.Server(pool_bytes=1 << 20, max_batch=2, inflight=1) as srv:
        tickets = [srv.submit(r.req) for r in mix]
        # the last request is still queued behind 29 others in a 1 MiB pool
        rc = srv.cancel(tickets[-1])
        assert rc in (0, int(native.Status.BUSY))
        rc_wait, _ = srv.try_wait(tickets[0], 0)                   # bounded: returns at once
        assert rc_wait in (0, int(native.Status.TIMEOUT))
        for t in tickets[:-1]:
            if rc_wait == 0 and t == tickets[0]:
                continue
            srv.wait(t)
        last_rc, last_stats = srv.try_wait(tickets[-1], -1)
        assert last_rc == (int(native.Status.CANCELLED) if rc == 0 else 0)
    for r in mix[:-1]:
        assert np.array_equal(r.out, native.encode(r.img, **r.opts))


def test_replay_open_loop(native):
    mix = _mix(native, 64, seed=21)
    arrival = np.cumsum(np.random.default_rng(0).exponential(200.0, len(mix)))   # ~5000 req/s
    with native.Server(pool_bytes=32 << 20, max_batch=32, inflight=3) as srv:
        lat, wall = srv.replay([r.req for r in mix], arrival)
    assert np.all(lat > 0) and wall > 0
    for r in mix:
        assert np.array_equal(r.out, native.encode(r.img, **r.opts))


def test_shutdown_drains_queued_work(native):
    mix = _mix(native, 25, seed=31)
    srv = native.Server(pool_bytes=4 << 20, max_batch=4, inflight=2)
    for r in mix:
        srv.submit(r.req)
    srv.close()                                                    # waits for everything queued
    for r in mix:
        assert np.array_equal(r.out, native.encode(r.img, **r.opts))


def test_server_rejects_bad_config(native):
    lib = native.load_library()
    h = ctypes.c_void_p()
    for cfg in (native.ServerConfig(1 << 10, 4, 1, 0, 0), native.ServerConfig(1 << 24, 0, 1, 0, 0),
                native.ServerConfig(1 << 24, 4, 0, 0, 0), native.ServerConfig(1 << 24, 4, 1, 5, 0),
                native.ServerConfig(1 << 24, 4, 1, 0, 9)):
        assert lib.astc_server_create(ctypes.byref(cfg), ctypes.byref(h)) == native.Status.INVALID_ARG
