"""Benchmark of the GB300 ASTC encoder (one JSON line on rank 0).

Workload (default): the 6x6 LDR RGBA sRGB encode with edge clamp of a
2048x2048 RGBA8 texture (342x342 blocks) -- the configuration the headline
metric "encoded Mtexels/s" is quoted on.  One step encodes a batch of 16
distinct 2048x2048 textures (268 MB of input, larger than the 129 MB L2, so
no step reads its inputs from L2), each through the C ABI
(astc_encode_gpu_pitched, device memory), the launches spread round-robin
over --streams CUDA streams (default 2) forked from torch's current stream.

* value      -- Mtexels/s with inputs resident in HBM, timed with one CUDA
                event pair around each step on the timed stream (a dedicated
                non-default torch stream; the side streams join it before the
                closing event; max over ranks).  `one_stream` repeats the step
                with every launch on the timed stream, one after another.
* e2e        -- the same metric through the same entry point with pinned
                HOST buffers: each texture goes up through the library's upload
                ring (copy engine, 32 MiB slots overlapped with the encode) and
                the kernels write its blocks back in place over NVLink-C2C, all
                inside the timed region, one stream synchronize per step.
                `e2e_pageable` repeats it with ordinary pageable (numpy)
                buffers and synchronous calls, the reference's own usage.
* roofline   -- the dominant kernel's algorithmic bytes (4 B/texel read +
                16 B/block written) per launch over its mean launch time,
                against the measured HBM copy bandwidth; roofline_fp32 gives
                the same launch in algorithmic FP32 FLOPs (counted from the
                oracle) against an FP32 SGEMM peak measured in this run.
* cpu_baseline -- the FP32 oracle (a CPU restatement of the reference
                shader; the reference itself is D3D11-only) with OpenMP on all
                host cores, on a bounded sample of the same workload.
``--impl reference`` times that CPU restatement alone (the reference arm).
Under torchrun each rank encodes its own batch (weak scaling, no data-path
collective); a barrier and a max-reduce of the elapsed time bracket the run.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

TEXTURES_PER_STEP = 16
METRIC = "encoded Mtexels/s"


def _parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="6x6_rgba_srgb_2048")
    ap.add_argument("--streams", type=int, default=2,
                    help="CUDA streams the headline step's launches are spread over (1 = one after another)")
    ap.add_argument("--no-extra", action="store_true", help="skip the secondary workloads")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-batched", action="store_true", help="skip the mixed batched workload")
    ap.add_argument("--batched-count", type=int, default=256, help="textures in the mixed batch")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving sweep")
    ap.add_argument("--no-search", action="store_true",
                    help="skip the search-mode / max-accumulation throughput and PSNR leg")
    ap.add_argument("--serving-rates", default="100,1000,5000,10000,20000,30000,40000,50000,70000,100000",
                    help="offered request rates (req/s)")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "half2"],
                    help="precision of the main workload")
    ap.add_argument("--profile-batched", action="store_true",
                    help="small case for ncu: one FP32 and one HALF2 batched graph launch")
    ap.add_argument("--wave-sweep", action="store_true",
                    help="fixed-mode launch time against the number of full waves (6x6 RGBA sRGB); "
                         "prints one JSON line per texture size and exits")
    ap.add_argument("--profile-case", action="store_true",
                    help="small case for ncu: 2 textures per step, encode launches only")
    ap.add_argument("--profile-quality", default="fast",
                    choices=["fast", "best_fit", "search", "thorough", "partitions", "three_partitions"],
                    help="with --profile-case: the quality mode the launches use (FP32)")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# clocks during the timed region (NVML through ctypes; nvidia-smi fallback)
# ---------------------------------------------------------------------------
class ClockSampler:
    REASONS = {0x1: "gpu_idle", 0x2: "applications_clocks_setting", 0x4: "sw_power_cap",
               0x8: "hw_slowdown", 0x10: "sync_boost", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown",
               0x100: "display_clock_setting"}

    def __init__(self, index: int):
        self.index = index
        self.samples: list[tuple[int, int]] = []
        self.max_mhz = None
        self._stop = threading.Event()
        self._thr = None
        self._nvml = None
        self._handle = None
        try:
            nv = ctypes.CDLL("libnvidia-ml.so.1")
            if nv.nvmlInit_v2() == 0:
                h = ctypes.c_void_p()
                if nv.nvmlDeviceGetHandleByIndex_v2(index, ctypes.byref(h)) == 0:
                    self._nvml, self._handle = nv, h
                    m = ctypes.c_uint()
                    if nv.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(m)) == 0:   # NVML_CLOCK_SM
                        self.max_mhz = int(m.value)
        except OSError:
            pass

    def _sample(self):
        nv, h = self._nvml, self._handle
        c, r = ctypes.c_uint(), ctypes.c_ulonglong()
        ok = nv.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(c)) == 0
        ok &= nv.nvmlDeviceGetCurrentClocksEventReasons(h, ctypes.byref(r)) == 0
        if ok:
            self.samples.append((int(c.value), int(r.value)))

    def _run(self):
        while not self._stop.is_set():
            self._sample()
            time.sleep(0.002)

    def start(self):
        if self._nvml is not None:
            self._thr = threading.Thread(target=self._run, daemon=True)
            self._thr.start()

    def stop(self) -> dict:
        if self._thr is not None:
            self._stop.set()
            self._thr.join()
            self._sample()
        if not self.samples:
            return self._smi_once()
        mhz = sorted(s[0] for s in self.samples)
        bits = 0
        for _, r in self.samples:
            bits |= r
        reasons = [n for b, n in self.REASONS.items() if bits & b and n != "gpu_idle"]
        return {"sm_mhz": mhz[len(mhz) // 2], "sm_max_mhz": self.max_mhz, "reasons": reasons,
                "samples": len(self.samples), "source": "nvml"}

    def _smi_once(self) -> dict:
        try:
            q = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=clocks.sm,clocks.max.sm",
                                "--format=csv,noheader,nounits"], capture_output=True, text=True,
                               timeout=20).stdout.strip().split(",")
            return {"sm_mhz": int(q[0]), "sm_max_mhz": int(q[1]), "reasons": [], "samples": 1,
                    "source": "nvidia-smi (after the timed region)"}
        except Exception as exc:  # noqa: BLE001
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "error": str(exc)}


def _peaks() -> dict:
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        return {}


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def _texture_batch(torch, base: np.ndarray, count: int, salt: int):
    """`count` distinct device textures with the statistics of `base` (2-D shifts)."""
    dev = torch.from_numpy(base).cuda()
    h, w = base.shape[:2]
    out = []
    for i in range(count):
        dy = (i * 97 + salt * 389) % h
        dx = (i * 331 + salt * 151) % w
        out.append(torch.roll(dev, shifts=(dy, dx), dims=(0, 1)).contiguous())
    return out


def _fp32_peak_tflops(torch) -> float:
    """FP32 peak of this GPU, measured as an 8192^3 SGEMM with TF32 off."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    n = 8192
    a = torch.randn(n, n, device="cuda", dtype=torch.float32)
    b = torch.randn(n, n, device="cuda", dtype=torch.float32)
    for _ in range(2):
        torch.mm(a, b)
    best = float("inf")
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        torch.mm(a, b)
        e.record()
        torch.cuda.synchronize()
        best = min(best, s.elapsed_time(e) / 1e3)
    torch.backends.cuda.matmul.allow_tf32 = prev
    del a, b
    return 2.0 * n ** 3 / best / 1e12


def _fp32_fma_peak_tflops() -> float | None:
    """FP32 FMA throughput from the library's probe (8 independent FMA chains
    per thread on every SM; best of 5 launches), or None if it is missing."""
    from astc_encoder_gb300 import build
    if not os.path.exists(build.PEAK_LIB):
        return None
    lib = ctypes.CDLL(build.PEAK_LIB)
    lib.astc_fp32_fma_peak.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    out = ctypes.c_double(0.0)
    if lib.astc_fp32_fma_peak(5, ctypes.byref(out)) != 0:
        return None
    return out.value


def _cpu_baseline(img: np.ndarray, spec: dict, min_seconds: float = 2.0) -> dict:
    from oracle import oracle
    threads = os.cpu_count() or 1
    oracle.encode(img[:64, :64], **spec, threads=threads)            # build + warm
    reps, t0 = 0, time.perf_counter()
    while True:
        oracle.encode(img, **spec, threads=threads)
        reps += 1
        el = time.perf_counter() - t0
        if el >= min_seconds:
            break
    texels = img.shape[0] * img.shape[1] * reps
    return {"value": texels / el / 1e6, "unit": "Mtexels/s", "cores": threads, "kind": "port",
            "sample": f"{reps} full encodes of one {img.shape[1]}x{img.shape[0]} texture "
                      f"({el:.2f} s wall on {threads} threads)"}


def _config(workload: str, img: np.ndarray, spec: dict, precision: str, world: int) -> dict:
    """The workload description both arms print (identical dicts)."""
    h, w = img.shape[:2]
    d = spec["block_dim"]
    return {"workload": workload, "texture": f"{w}x{h}",
            "blocks_per_texture": ((w + d - 1) // d) * ((h + d - 1) // d),
            "textures_per_step": TEXTURES_PER_STEP, "block_dim": d, "has_alpha": bool(spec["has_alpha"]),
            "is_normal": bool(spec["is_normal"]), "srgb": bool(spec["srgb"]),
            "border": "clamp" if spec["border"] else "zero", "precision": precision,
            "l2": f"inputs {h * w * 4 * TEXTURES_PER_STEP / 2**20:.0f} MiB per step, distinct per texture "
                  "(> 129 MB L2); no flush needed",
            "parallelism": f"replicas{world}"}


def run_reference(args) -> None:
    world, rank, _ = _dist()
    if rank != 0:
        return
    from astc_encoder_gb300 import synth
    from oracle import oracle
    img, spec = synth.workload(args.workload)
    threads = os.cpu_count() or 1
    h, w = img.shape[:2]
    # the same step as the GPU arm: 16 distinct textures (2-D shifts of one)
    texs = [np.ascontiguousarray(np.roll(img, ((i * 97) % h, (i * 331) % w), axis=(0, 1)))
            for i in range(TEXTURES_PER_STEP)]
    oracle.encode(img[:64, :64], **spec, threads=threads)
    for _ in range(args.warmup):
        oracle.encode(texs[0], **spec, threads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for t in texs:
            oracle.encode(t, **spec, threads=threads)
    el = time.perf_counter() - t0
    texels = h * w * len(texs)
    value = texels * args.steps / el / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mtexels/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": el / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": _config(args.workload, img, spec, args.precision, world),
        "cpu_baseline": {"value": value, "unit": "Mtexels/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} timed steps of {len(texs)} textures; the reference "
                                   "shader is D3D11-only (unavailable on this box), so its FP32 "
                                   "CPU restatement (oracle/) runs with OpenMP"},
        "e2e": {"value": value, "unit": "Mtexels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


_SIDE_STREAMS: list = []


def _time_launches(torch, native, texs, outs, spec, steps, streams: int = 1):
    """Runs `steps` steps over the batch with a CUDA event pair around each step
    (on the launching stream); returns (mean ms per launch, step ms list, launches).

    With `streams` = 1 the launches of a step run back to back on the current
    stream, so step time / launches is the mean launch duration.  With more,
    launch i goes to stream i mod `streams`: the side streams wait for the
    current one at the start of the step and the current one waits for them
    at its end, so the event pair still brackets the whole step, and one
    texture's kernel fills the SM slots that the previous texture's last,
    partial wave leaves idle (the textures are independent); step time /
    launches is then the effective time per launch."""
    h, w = texs[0].shape[:2]
    stream = torch.cuda.current_stream()
    if stream.cuda_stream == 0:
        # a NULL stream means "synchronous on the library's own stream" in the C ABI
        raise RuntimeError("run the timed loop on a non-default stream")
    while len(_SIDE_STREAMS) < streams - 1:
        _SIDE_STREAMS.append(torch.cuda.Stream())
    side = _SIDE_STREAMS[:streams - 1]
    lib = native.load_library()
    opts = [native.make_opts(memory=native.Memory.DEVICE, stream=s.cuda_stream, **spec) for s in [stream] + side]
    ptrs = [(t.data_ptr(), o.data_ptr()) for t, o in zip(texs, outs)]
    enc = lib.astc_encode_gpu_pitched
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    l0 = native.kernel_launch_count()
    for s in range(steps):
        ev[s][0].record(stream)
        for ss in side:
            ss.wait_stream(stream)
        for i, (src, dst) in enumerate(ptrs):
            st = enc(src, w, h, w * 4, ctypes.byref(opts[i % len(opts)]), dst)
            if st != 0:
                raise native.AstcError(st, lib.astc_last_error().decode())
        for ss in side:
            stream.wait_stream(ss)
        ev[s][1].record(stream)
    torch.cuda.synchronize()
    launches = native.kernel_launch_count() - l0
    per_step = [a.elapsed_time(b) for a, b in ev]
    return sum(per_step) / max(1, launches), per_step, launches


def _bench_aux(torch, native, texs, outs, spec: dict, hbm_peak: float, passes: int = 5) -> dict:
    """The kernels around the encoder, on the headline's 16 textures and their
    blocks, device-resident: the integer LDR decoder (16 B/block in, 4 B/texel
    out), the no-alloc SSE reduction of source against decode (8 B/texel in)
    and the box-filtered mip chain (each level reads the level above and
    writes itself, 4 B/texel each way); algorithmic GB/s against the HBM copy
    bandwidth, timed with a CUDA event pair around `passes` passes over the
    16 textures (decoded images and sources above L2 size)."""
    h, w = texs[0].shape[:2]
    d = spec["block_dim"]
    n = len(texs)
    nb = ((w + d - 1) // d) * ((h + d - 1) // d)
    stream = torch.cuda.current_stream()
    lib = native.load_library()

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = native.kernel_launch_count()
        a.record(stream)
        for _ in range(passes):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1e3 / passes, (native.kernel_launch_count() - l0) // passes

    def entry(seconds, launches, nbytes, texels):
        gbs = nbytes / seconds / 1e9
        return {"GB_s": gbs, "frac_hbm": gbs / hbm_peak, "Mtexels_s": texels / seconds / 1e6,
                "us_per_texture": seconds * 1e6 / n, "launches_per_pass": int(launches),
                "alg_bytes_per_pass": int(nbytes)}

    dec = [torch.empty((h, w, 4), dtype=torch.uint8, device="cuda") for _ in texs]

    def decode_pass():
        for o, dd in zip(outs, dec):
            native.decode_device(o.data_ptr(), w, h, d, d, dd.data_ptr(), stream=stream.cuda_stream)

    t, l = timed(decode_pass)
    result = {"decode_ldr": entry(t, l, n * (nb * 16 + h * w * 4), n * h * w)}

    sse_fn = lib.astc_sse_gpu_noalloc
    sse_fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]
    sse_fn.restype = ctypes.c_int
    acc = torch.zeros(4, dtype=torch.int64, device="cuda")

    def sse_pass():
        for src, dd in zip(texs, dec):
            st = sse_fn(src.data_ptr(), dd.data_ptr(), h * w, stream.cuda_stream, acc.data_ptr())
            if st != 0:
                raise native.AstcError(st, lib.astc_last_error().decode())

    t, l = timed(sse_pass)
    result["sse_noalloc"] = entry(t, l, n * h * w * 8, n * h * w)
    del dec

    levels = native.mip_levels(w, h)
    sizes = native.mip_sizes(w, h, levels)
    chain = native.mip_chain_bytes(w, h, levels)
    mips = [torch.empty(chain, dtype=torch.uint8, device="cuda") for _ in texs]

    def mip_pass():
        for src, m in zip(texs, mips):
            native.generate_mips(src.data_ptr(), w, h, levels, m.data_ptr(), srgb=bool(spec["srgb"]),
                                 stream=stream.cuda_stream)

    t, l = timed(mip_pass)
    mip_bytes = sum(4 * (sizes[i - 1][0] * sizes[i - 1][1] + sizes[i][0] * sizes[i][1]) for i in range(1, levels))
    result["mip_chain" + ("_srgb" if spec["srgb"] else "")] = entry(t, l, n * mip_bytes, n * h * w)
    result["mip_chain" + ("_srgb" if spec["srgb"] else "")]["levels"] = levels
    del mips
    return result


def _wave_sweep(torch, native, synth, warmup: int, steps: int) -> None:
    """Mean launch time of the fixed-mode 6x6 RGBA sRGB kernel for textures of
    0.5 to 4 full waves (12 resident warps per SM: 152 x 384 blocks per wave)
    and the 2048x2048 texture (2.004 waves): separates the per-launch cost
    (ramp-up and drain) from the cost of a further full wave."""
    spec = dict(block_dim=6, has_alpha=True, is_normal=False, srgb=True, border=1)
    per_wave = torch.cuda.get_device_properties(0).multi_processor_count * 384
    src = synth.rgba_cutout(3648, 2304)
    for h, w in [(456, 2304), (912, 2304), (1368, 2304), (1824, 2304), (1830, 2304), (2048, 2048),
                 (2736, 2304), (3648, 2304)]:
        img = np.ascontiguousarray(src[:h, :w]) if (h, w) != (2048, 2048) else synth.rgba_cutout(2048, 2048)
        texs = _texture_batch(torch, img, TEXTURES_PER_STEP, salt=0)
        nb = ((w + 5) // 6) * ((h + 5) // 6)
        outs = [torch.empty((nb, 16), dtype=torch.uint8, device="cuda") for _ in texs]
        _time_launches(torch, native, texs, outs, spec, warmup)
        per, _, _ = _time_launches(torch, native, texs, outs, spec, steps)
        print(json.dumps({"wave_sweep": f"{w}x{h}", "blocks": nb, "waves": round(nb / per_wave, 3),
                          "mean_launch_us": round(per * 1e3, 2),
                          "Mtexels_s": round(w * h / (per * 1e3), 1)}), flush=True)
        del texs, outs


# DRAM bytes (read + write) of one launch of the production kernel, from the
# ncu capture summarised in profiles/ (the capture's command is given there):
# (workload, precision, texel store) -> bytes, capture
_NCU_TRAFFIC = {
    ("6x6_rgba_srgb_2048", 0, 2): (16_833_536, "astc_encode_blocks_fp32_6x6_rgba_srgb_2048.md: "
                                               "16.83 MB read, 0 B written (blocks still in L2)"),
}


# Warp instructions of one launch of the production kernel, from the same ncu
# capture: (workload, precision, texel store) -> instructions, capture
_NCU_INSTRUCTIONS = {
    ("6x6_rgba_srgb_2048", 0, 2): (11_141_869, "astc_encode_blocks_fp32_6x6_rgba_srgb_2048.md: "
                                               "11.14 M warp-instructions per launch"),
}


def _issue_roofline(workload: str, prec: int, tuned, mean_launch_s: float, sm_mhz, sms: int) -> dict | None:
    """Warp instructions issued per second against the SMs' issue ceiling (4
    schedulers per SM, one warp-instruction per cycle each, at the SM clock
    sampled during the timed region); None without a capture of this kernel."""
    key = (workload, prec, getattr(tuned, "store", None))
    if key not in _NCU_INSTRUCTIONS or not sm_mhz:
        return None
    n, src = _NCU_INSTRUCTIONS[key]
    achieved = n / mean_launch_s / 1e9
    peak = sms * 4 * float(sm_mhz) / 1e3
    return {"bound": "instruction_issue", "achieved": achieved, "peak": peak,
            "unit": "G warp-instructions/s", "frac": achieved / peak, "instructions_per_launch": n,
            "peak_source": f"{sms} SMs x 4 schedulers x {sm_mhz} MHz (median SM clock in the timed region)",
            "instructions_source": "profiles/" + src}


def _traffic(workload: str, prec: int, tuned) -> dict:
    key = (workload, prec, getattr(tuned, "store", None))
    if key not in _NCU_TRAFFIC:
        return {"traffic": None, "traffic_source": "no ncu capture of this kernel variant"}
    b, src = _NCU_TRAFFIC[key]
    return {"traffic": b, "traffic_unit": "bytes per launch", "traffic_source": "profiles/" + src}


def _psnr_blocks(native, blocks: np.ndarray, tex: np.ndarray, spec: dict) -> float:
    """Decoded PSNR (GPU decoder, GPU reduction) in the space the encoder fits:
    RGB(A) codes, sRGB linearised; normal maps on the rebuilt unit normals
    (z = sqrt(max(0, 1 - x^2 - y^2)) on both sides, 3 components)."""
    h, w = tex.shape[:2]
    d = native.decode(blocks, w, h, spec["block_dim"])
    if spec["is_normal"]:
        return native.psnr_from_sse(native.normal_sse(d, tex), h * w * 3)
    fitted = native.fitted_reference(tex, spec["srgb"], spec["is_normal"])
    ch = 4 if spec["has_alpha"] else 3
    s = native.sse(d, fitted)
    return native.psnr_from_sse(float(s[:ch].sum()), h * w * ch)


def _rmse(psnr_db: float, peak: float = 255.0) -> float:
    """RMSE (in 8-bit code units, the PSNR's peak of 255) of a PSNR."""
    return peak * 10.0 ** (-psnr_db / 20.0)


def _psnr_space(spec: dict) -> str:
    if spec["is_normal"]:
        return "rebuilt unit normals (x, y from R, G; z = sqrt(1 - x^2 - y^2)), 3 components x 127.5"
    return (("linearised sRGB x255 (what the encoder fits), " if spec["srgb"] else "") +
            f"{4 if spec['has_alpha'] else 3} channels")


def _bench_search(torch, native, headline: str, texs, outs, spec: dict) -> dict:
    """Throughput and decoded PSNR of the quality modes -- the search (every
    single-partition 4x4-grid mode, least decoded error), the max-accumulation
    axis, the better of both fits (ASTC_AXIS_BEST), THOROUGH (search from the better fit, plus dual-plane blocks),
    PARTITIONS (THOROUGH plus two-partition blocks) and THREE_PARTITIONS
    (PARTITIONS plus three-partition RGB blocks) -- against the fixed mode, on
    each workload and on flat-colour graphics (synth.ui_shapes, 4x4 RGB, where
    three partitions pay), device-resident inputs above L2 size as the
    headline."""
    from astc_encoder_gb300 import synth
    result = {}
    for name in (headline, "4x4_rgb_512", "4x4_normal_4096", "6x6_rgba_srgb_2048", "ui_shapes_4x4_1024"):
        if name in result:
            continue
        if name == headline:
            st, so, sspec = texs, outs, dict(spec)
        else:
            if name == "ui_shapes_4x4_1024":
                simg = synth.ui_shapes(1024, 1024)
                sspec = dict(block_dim=4, has_alpha=False, is_normal=False, srgb=False, border=0)
            else:
                simg, sspec = synth.workload(name)
            sh, sw = simg.shape[:2]
            sd = sspec["block_dim"]
            snb = ((sw + sd - 1) // sd) * ((sh + sd - 1) // sd)
            reps = max(1, (268 << 20) // (sh * sw * 4))
            st = _texture_batch(torch, simg, reps, salt=11)
            so = [torch.empty((snb, 16), dtype=torch.uint8, device="cuda") for _ in st]
        sh, sw = st[0].shape[:2]
        tex0 = st[0].cpu().numpy()
        entry = {"textures_per_step": len(st)}
        for label, kw in (("fast", {}), ("search", dict(quality=1)), ("max_accumulation", dict(axis=1)),
                          ("best_fit", dict(axis=2)),
                          ("thorough", dict(quality=2)), ("partitions", dict(quality=3)),
                          ("three_partitions", dict(quality=4))):
            run = dict(sspec, **kw)
            _time_launches(torch, native, st, so, run, 2)
            per, steps, _ = _time_launches(torch, native, st, so, run, 5)
            entry[label] = {"value": sh * sw * len(st) * 5 / (sum(steps) / 1e3) / 1e6, "unit": "Mtexels/s",
                            "mean_launch_us": per * 1e3,
                            "psnr_db": _psnr_blocks(native, so[0].cpu().numpy(), tex0, sspec)}
            entry[label]["rmse"] = _rmse(entry[label]["psnr_db"])
        entry["search_gain_db"] = entry["search"]["psnr_db"] - entry["fast"]["psnr_db"]
        entry["thorough_gain_db"] = entry["thorough"]["psnr_db"] - entry["fast"]["psnr_db"]
        entry["partitions_gain_db"] = entry["partitions"]["psnr_db"] - entry["fast"]["psnr_db"]
        entry["three_partitions_gain_db"] = entry["three_partitions"]["psnr_db"] - entry["fast"]["psnr_db"]
        result[name] = entry
        if name != headline:
            del st, so
    return result


def _bench_batched(torch, native, oracle, count: int, reps: int = 5) -> dict:
    """The mixed workload: `count` textures with full mip chains, mixed formats.

    plain   -- one astc_encode_gpu_pitched launch per texture level (FP32)
    batched -- one astc_batch_encode graph launch for everything (FP32, HALF2)
    Inputs resident in HBM; CUDA events on the work stream around each pass.
    """
    from astc_encoder_gb300 import synth_gpu
    stream = torch.cuda.current_stream()
    t0 = time.perf_counter()
    texs = synth_gpu.mixed_batch(torch, native, count)
    gen_s = time.perf_counter() - t0
    lib = native.load_library()
    jobs = []            # (w, h, in_tensor, out_tensor, opts)
    for t in texs:
        d = t["opts"]["block_dim"]
        for w, h, lvl in t["levels"]:
            nb = ((w + d - 1) // d) * ((h + d - 1) // d)
            jobs.append((w, h, lvl, torch.empty((nb, 16), dtype=torch.uint8, device="cuda"), t["opts"]))
    texels = sum(w * h for w, h, *_ in jobs)
    blocks = sum(o.shape[0] for *_, o, _ in jobs)
    # plain: one launch per level, options prebuilt
    plain_calls = []
    for w, h, lvl, out, opts in jobs:
        o = native.make_opts(memory=native.Memory.DEVICE, stream=stream.cuda_stream, **opts)
        plain_calls.append((lvl.data_ptr(), w, h, w * 4, o, out.data_ptr()))
    enc = lib.astc_encode_gpu_pitched

    def plain_pass():
        for src, w, h, pitch, o, dst in plain_calls:
            st = enc(src, w, h, pitch, ctypes.byref(o), dst)
            if st:
                raise native.AstcError(st, lib.astc_last_error().decode())

    items = (native.BatchItem * len(jobs))()
    for i, (w, h, lvl, out, opts) in enumerate(jobs):
        items[i] = native.BatchItem(lvl.data_ptr(), 0, w, h, opts["block_dim"], int(opts["has_alpha"]),
                                    int(opts["is_normal"]), int(opts["srgb"]), int(opts["border"]),
                                    out.data_ptr())
    batch = native.Batch(len(jobs), blocks)

    def batched_pass(prec):
        st = lib.astc_batch_encode(batch._h, items, len(jobs), prec, stream.cuda_stream)
        if st:
            raise native.AstcError(st, lib.astc_last_error().decode())

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        best, l0 = [], native.kernel_launch_count()
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            best.append(a.elapsed_time(b))
        return float(np.median(best)), (native.kernel_launch_count() - l0) // reps

    plain_ms, plain_launches = timed(plain_pass)
    fp32_ms, fp32_launches = timed(lambda: batched_pass(0))
    fp32_blocks = [o.cpu().numpy() for *_, o, _ in jobs]
    h2_ms, h2_launches = timed(lambda: batched_pass(1))
    # quality per texture (level 0): PSNR of FP32 / HALF2 against the FP64 oracle
    gaps, same, rmses = [], [], []
    k = 0
    for t in texs:
        w, h, lvl = t["levels"][0]
        opts = t["opts"]
        img = lvl.cpu().numpy()
        h2 = jobs[k][3].cpu().numpy()
        f32 = fp32_blocks[k]
        f64 = oracle.encode(img, fp64=True, **opts)

        def psnr(bl):
            return _psnr_blocks(native, bl, img, opts)
        p64, p32, p16 = psnr(f64), psnr(f32), psnr(h2)
        gaps.append((p64 - p32, p64 - p16))
        rmses.append((_rmse(p64), _rmse(p32), _rmse(p16)))
        same.append(float(np.all(h2 == f32, axis=1).mean()))
        k += len(t["levels"])
    batch.close()
    g32 = np.array([g[0] for g in gaps])
    g16 = np.array([g[1] for g in gaps])
    mtex = lambda ms: texels / (ms / 1e3) / 1e6  # noqa: E731
    return {
        "textures": count, "texture_levels": len(jobs), "texels": texels, "blocks": blocks,
        "formats": {f: sum(1 for t in texs if t["format"] == f) for f in ("4x4_rgb", "6x6_rgba_srgb", "4x4_normal")},
        "plain_fp32": {"ms": plain_ms, "Mtexels_s": mtex(plain_ms), "launches": plain_launches},
        "batched_fp32": {"ms": fp32_ms, "Mtexels_s": mtex(fp32_ms), "launches": fp32_launches,
                         "graph_launches": 1},
        "batched_half2": {"ms": h2_ms, "Mtexels_s": mtex(h2_ms), "launches": h2_launches, "graph_launches": 1},
        "speedup_batched_half2_vs_plain_fp32": plain_ms / h2_ms,
        "speedup_batched_fp32_vs_plain_fp32": plain_ms / fp32_ms,
        "speedup_half2_vs_fp32_batched": fp32_ms / h2_ms,
        "psnr_gap_to_fp64_db": {"fp32_mean": float(g32.mean()), "fp32_max": float(g32.max()),
                                "half2_mean": float(g16.mean()), "half2_max": float(g16.max()),
                                "half2_textures_within_0.05dB": int((g16 <= 0.05).sum())},
        "rmse_mean": {"fp64_oracle": float(np.mean([r[0] for r in rmses])),
                      "fp32": float(np.mean([r[1] for r in rmses])),
                      "half2": float(np.mean([r[2] for r in rmses])),
                      "half2_max_vs_fp64_pct": float(max(100.0 * (r[2] / r[0] - 1.0) for r in rmses)),
                      "unit": "8-bit codes, in each texture's PSNR space"},
        "half2_identical_blocks_vs_fp32_mean": float(np.mean(same)),
        "generation_s": gen_s,
    }


def _bench_serving(torch, native, rates, seconds: float = 2.0, max_requests: int = 2000,
                   host: str = "pinned") -> dict:
    """Open-loop serving: Poisson arrivals at each rate, single-texture requests.

    Request side lengths are log-uniform in [128, 2048] (square), formats mixed
    60% 4x4 RGB / 25% 6x6 RGBA sRGB / 15% 4x4 normal, content cropped from
    2048x2048 synthetic textures held in pinned host memory (`host` =
    "pageable": ordinary numpy buffers); 2 GiB device staging pool with
    admission by memory.  Batched = continuous batching through astc_batch;
    per-request = one plain launch per request.
    """
    from astc_encoder_gb300 import synth
    bases = {
        "4x4_rgb": (synth.rgb_noise(2048, 2048), dict(block_dim=4)),
        "6x6_rgba_srgb": (synth.rgba_cutout(2048, 2048), dict(block_dim=6, has_alpha=True, srgb=True, border=1)),
        "4x4_normal": (synth.normal_map(2048, 2048), dict(block_dim=4, is_normal=True)),
    }
    if host == "pinned":
        src_tex = {k: torch.from_numpy(v[0]).pin_memory() for k, v in bases.items()}
    else:
        src_tex = {k: torch.from_numpy(np.ascontiguousarray(v[0])) for k, v in bases.items()}
    names, probs = ["4x4_rgb", "6x6_rgba_srgb", "4x4_normal"], [0.60, 0.25, 0.15]
    rng = np.random.default_rng(synth.SEED_BASE + 4)
    n_max = max_requests
    kinds = rng.choice(3, size=n_max, p=probs)
    sides = np.exp(rng.uniform(np.log(128), np.log(2048), n_max)).astype(int)
    reqs_meta, out_bytes = [], 0
    for k, s in zip(kinds, sides):
        name = names[k]
        opts = bases[name][1]
        x0, y0 = int(rng.integers(0, 2048 - s + 1)), int(rng.integers(0, 2048 - s + 1))
        d = opts["block_dim"]
        nb = int(((int(s) + d - 1) // d) ** 2)
        reqs_meta.append((name, int(s), x0, y0, opts, out_bytes, nb))
        out_bytes += nb * 16
    # pageable: zero-filled, so every page is resident before the device writes
    # it (a service reuses its buffers; the device's first touch of a pageable
    # page faults it in through the host and is slow)
    out = torch.zeros(out_bytes, dtype=torch.uint8)
    if host == "pinned":
        out = out.pin_memory()
    requests = []
    for name, s, x0, y0, opts, off, nb in reqs_meta:
        base = src_tex[name]
        ptr = base.data_ptr() + (y0 * 2048 + x0) * 4
        requests.append(native.make_request(int(ptr), s, s, int(out.data_ptr() + off), row_pitch=2048 * 4, **opts))
    texels = np.array([m[1] * m[1] for m in reqs_meta], np.float64)
    result = {"pool_bytes": 2 << 30, "requests_max": n_max, "inflight_slots": 3, "max_batch": 256,
              "host_buffers": host, "rates": {}}
    for mode, label in ((native.SERVE_BATCHED, "batched"), (native.SERVE_PER_REQUEST, "per_request")):
        with native.Server(pool_bytes=2 << 30, max_batch=256, inflight=3, mode=mode) as srv:
            # warm-up: graphs and pools, single-request batches, and one pass over
            # every request's buffers (a device's first access to a pageable
            # page goes through the host and is slow)
            srv.replay(requests[:64], np.zeros(64))
            srv.replay(requests[:16], np.arange(16) * 2000.0)
            srv.replay(requests, np.zeros(len(requests)))
            for rate in rates:
                n = int(min(n_max, max(64, rate * seconds)))
                arrival = np.cumsum(np.random.default_rng(int(rate)).exponential(1e6 / rate, n))
                srv.stats(reset=True)
                lat, wall = srv.replay(requests[:n], arrival)
                dev = srv.stats(reset=True)
                busy = dev["device_busy_s"]
                result["rates"].setdefault(str(rate), {})[label] = {
                    "requests": n, "p50_ms": float(np.percentile(lat, 50)) / 1e3,
                    "p99_ms": float(np.percentile(lat, 99)) / 1e3, "mean_ms": float(lat.mean()) / 1e3,
                    "throughput_req_s": n / wall, "Mtexels_s": float(texels[:n].sum()) / wall / 1e6,
                    "offered_req_s": rate,
                    # device side (timing events on each slot's stream)
                    "launches": dev["launches"],
                    "requests_per_launch": dev["requests"] / max(1, dev["launches"]),
                    "gpu_busy_frac": busy / wall if wall > 0 else None,
                    "slots_in_flight_mean": dev["device_slot_s"] / busy if busy > 0 else 0.0,
                    "overlap_frac": dev["device_overlap_s"] / busy if busy > 0 else 0.0}
    # the knee: the lowest offered rate at which per-request launches fall
    # behind batching: p99 above twice the batched p99, or under 90% of the
    # batched throughput served
    knee = None
    for rate in rates:
        r = result["rates"].get(str(rate), {})
        if "batched" not in r or "per_request" not in r:
            continue
        b, p = r["batched"], r["per_request"]
        if p["p99_ms"] > 2 * b["p99_ms"] or p["throughput_req_s"] < 0.9 * b["throughput_req_s"]:
            knee = {"offered_req_s": rate, "p99_ms_batched": b["p99_ms"], "p99_ms_per_request": p["p99_ms"],
                    "served_req_s_batched": b["throughput_req_s"],
                    "served_req_s_per_request": p["throughput_req_s"]}
            break
    result["knee"] = knee
    return result


def run_ours(args) -> None:
    import torch
    world, rank, local = _dist()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import astc_encoder_gb300 as native
    from astc_encoder_gb300 import build, synth
    build.build()
    native.load_library()
    # every launch and event goes to one dedicated (non-default) stream
    work_stream = torch.cuda.Stream()
    torch.cuda.set_stream(work_stream)

    if args.profile_batched:
        # the mixed batch, one FP32 and one HALF2 graph launch; nothing else
        from astc_encoder_gb300 import synth_gpu
        texs_b = synth_gpu.mixed_batch(torch, native, args.batched_count)
        items, n_blocks = [], 0
        keep = []
        for t in texs_b:
            d = t["opts"]["block_dim"]
            for lw, lh, lvl in t["levels"]:
                nb = ((lw + d - 1) // d) * ((lh + d - 1) // d)
                o = torch.empty((nb, 16), dtype=torch.uint8, device="cuda")
                keep.append(o)
                items.append(dict(rgba8=lvl.data_ptr(), width=lw, height=lh, out=o.data_ptr(), **t["opts"]))
                n_blocks += nb
        with native.Batch(len(items), n_blocks) as b:
            for prec in (0, 1):
                b.encode(items, precision=prec, stream=work_stream.cuda_stream)
            torch.cuda.synchronize()
        print(json.dumps({"profile_batched": len(items), "blocks": n_blocks}), flush=True)
        return

    if args.wave_sweep:
        _wave_sweep(torch, native, synth, max(3, args.warmup), max(5, min(args.steps, 20)))
        return

    img, spec = synth.workload(args.workload)
    h, w = img.shape[:2]
    dim = spec["block_dim"]
    nblocks = ((w + dim - 1) // dim) * ((h + dim - 1) // dim)
    prec = 1 if args.precision == "half2" else 0
    # the autotuner picks the kernel variant (texel store, CTA size) for this
    # format; the profiling case keeps the built-in default (under a profiler
    # every launch is serialised and the autotuner's timings are meaningless)
    tuned = None if args.profile_case else native.autotune(dim, spec["has_alpha"], spec["is_normal"],
                                                           spec["srgb"], w, h)
    texs = _texture_batch(torch, img, 2 if args.profile_case else TEXTURES_PER_STEP, salt=rank)
    outs = [torch.empty((nblocks, 16), dtype=torch.uint8, device="cuda") for _ in texs]
    spec_run = dict(spec, precision=prec)

    if args.profile_case:
        # only the encode launches: warm-up, then the timed steps; no other kernels
        quality, axis = {"fast": (0, 0), "best_fit": (0, 2), "search": (1, 0), "thorough": (2, 0),
                         "partitions": (3, 0), "three_partitions": (4, 0)}[args.profile_quality]
        spec_prof = dict(spec_run, quality=quality, axis=axis) if (quality or axis) else spec_run
        _time_launches(torch, native, texs, outs, spec_prof, max(3, args.warmup))
        per, _, launches = _time_launches(torch, native, texs, outs, spec_prof, args.steps)
        store, threads = native.get_kernel_choice(dim, spec["has_alpha"], spec["is_normal"], spec["srgb"])
        print(json.dumps({"profile_case": args.workload, "quality": args.profile_quality,
                          "launches": launches, "mean_launch_us": per * 1e3,
                          "kernel_variant": {"store": store, "threads_per_cta": threads}}), flush=True)
        return

    # warm-up (untimed) + a short sustained burn so clocks settle
    nstreams = max(1, args.streams)
    _time_launches(torch, native, texs, outs, spec_run, max(3, args.warmup), nstreams)
    t_end = time.perf_counter() + 0.5
    while time.perf_counter() < t_end:
        _time_launches(torch, native, texs, outs, spec_run, 2, nstreams)

    clocks = ClockSampler(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t0 = time.perf_counter()
    per, per_step, launches = _time_launches(torch, native, texs, outs, spec_run, args.steps, nstreams)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    # the same step with every launch on one stream (each launch's partial
    # last wave then runs with the GPU otherwise idle)
    if nstreams > 1:
        per1, per_step1, _ = _time_launches(torch, native, texs, outs, spec_run, args.steps, 1)
    else:
        per1, per_step1 = per, per_step
    dev_s = sum(per_step) / 1e3
    if world > 1:
        t = torch.tensor([dev_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        dev_s = float(t.item())
    texels_step = h * w * len(texs)
    value = world * texels_step * args.steps / dev_s / 1e6

    # e2e through the same entry point with pinned host buffers
    host_in = [t.cpu().pin_memory() for t in texs]
    host_out = [torch.empty((nblocks, 16), dtype=torch.uint8).pin_memory() for _ in texs]
    lib = native.load_library()
    # pinned buffers + a stream: the kernels read the texels and write the
    # blocks through the host link, asynchronously; one synchronize per step
    # ends the step with every block in host memory
    opts = native.make_opts(memory=native.Memory.HOST, stream=work_stream.cuda_stream, **spec_run)

    def e2e_step():
        for hi, ho in zip(host_in, host_out):
            st = lib.astc_encode_gpu(hi.data_ptr(), w, h, ctypes.byref(opts), ho.data_ptr())
            if st != 0:
                raise native.AstcError(st, lib.astc_last_error().decode())
        work_stream.synchronize()

    for _ in range(max(3, args.warmup)):
        e2e_step()
    e2e_steps = max(5, args.steps // 2)
    if world > 1:
        torch.distributed.barrier()
    t1 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    e2e_s = time.perf_counter() - t1
    if world > 1:
        t = torch.tensor([e2e_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = world * texels_step * e2e_steps / e2e_s / 1e6

    # the same entry point with ordinary pageable buffers (numpy arrays) and
    # no stream -- the reference's own usage: a malloc'd image in, a malloc'd
    # block buffer out, each call returning with the blocks in place
    page_in = [np.ascontiguousarray(t.cpu().numpy()) for t in texs]
    page_out = [np.empty((nblocks, 16), np.uint8) for _ in texs]
    opts_page = native.make_opts(memory=native.Memory.HOST, **spec_run)

    def e2e_pageable_step():
        for pi, po in zip(page_in, page_out):
            st = lib.astc_encode_gpu(pi.ctypes.data, w, h, ctypes.byref(opts_page), po.ctypes.data)
            if st != 0:
                raise native.AstcError(st, lib.astc_last_error().decode())

    for _ in range(max(3, args.warmup)):
        e2e_pageable_step()
    t1 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_pageable_step()
    e2e_page_s = time.perf_counter() - t1
    if world > 1:
        t = torch.tensor([e2e_page_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_page_s = float(t.item())
    e2e_page_value = world * texels_step * e2e_steps / e2e_page_s / 1e6
    page_caps = native.device_caps()
    del page_in, page_out

    if rank != 0:
        if world > 1:
            torch.distributed.barrier()
            torch.distributed.destroy_process_group()
        return

    # roofline of the dominant kernel
    from oracle import oracle
    peaks = _peaks()
    mean_launch_s = per / 1e3
    alg_bytes = h * w * 4 + nblocks * 16
    hbm_peak = peaks.get("hbm_gbs")
    # without the measured figure: one earlier GB300 copy-bandwidth measurement
    hbm_source = "MEASURED_PEAKS.json hbm_gbs (measured)" if hbm_peak else "fallback 6,800 GB/s (no measured figure)"
    hbm_peak = hbm_peak or 6800.0
    achieved_gbs = alg_bytes / mean_launch_s / 1e9
    flops = oracle.flops_per_block(dim, spec["has_alpha"], spec["is_normal"]) * nblocks
    sgemm_peak = _fp32_peak_tflops(torch)
    fma_peak = _fp32_fma_peak_tflops()
    # the denominator is the larger of the two measurements
    fp32_peak = max(sgemm_peak, fma_peak or 0.0)
    achieved_tf = flops / mean_launch_s / 1e12
    kernel = (f"astc_encode_blocks_{'h2' if prec else 'fp32'}<{dim},{int(spec['has_alpha'])},"
              f"{int(spec['is_normal'])},{int(spec['srgb'])}>")

    # quality of this workload: CUDA vs FP32 oracle (identical blocks) and
    # PSNR of both against the FP64 twin's PSNR, decoded by the GPU decoder
    got = outs[0].cpu().numpy()
    tex0 = texs[0].cpu().numpy()
    ora = oracle.encode(tex0, **spec)
    f64 = oracle.encode(tex0, **spec, fp64=True)

    def psnr(blocks):
        return _psnr_blocks(native, blocks, tex0, spec)

    quality = {"identical_blocks_vs_fp32_oracle": float(np.all(got == ora, axis=1).mean()),
               "psnr_db": psnr(got), "psnr_fp32_oracle_db": psnr(ora), "psnr_fp64_oracle_db": psnr(f64),
               "psnr_space": _psnr_space(spec) + ", spec LDR decode on the GPU"}
    quality["psnr_gap_to_fp64_db"] = quality["psnr_fp64_oracle_db"] - quality["psnr_db"]
    quality["rmse"] = {"ours": _rmse(quality["psnr_db"]), "fp32_oracle": _rmse(quality["psnr_fp32_oracle_db"]),
                       "fp64_oracle": _rmse(quality["psnr_fp64_oracle_db"]), "unit": "8-bit codes"}

    # plain (one launch per texture) FP32 and HALF2 on the three workloads
    extra = {}
    if not args.no_extra:
        for name in ("4x4_rgb_512", "6x6_rgba_srgb_2048", "4x4_normal_4096"):
            ximg, xspec = synth.workload(name)
            xh, xw = ximg.shape[:2]
            xd = xspec["block_dim"]
            xnb = ((xw + xd - 1) // xd) * ((xh + xd - 1) // xd)
            reps = max(1, (268 << 20) // (xh * xw * 4))     # keep each step above L2 size
            xt = _texture_batch(torch, ximg, reps, salt=7)
            xo = [torch.empty((xnb, 16), dtype=torch.uint8, device="cuda") for _ in xt]
            # the autotuner picks the FP32 mapping for this size (the
            # cooperative one competes for textures under one wave)
            xt_tuned = native.autotune(xd, xspec["has_alpha"], xspec["is_normal"], xspec["srgb"], xw, xh)
            entry = {"textures_per_step": reps,
                     "fp32_kernel_variant": {"store": xt_tuned.store, "threads_per_cta": xt_tuned.threads}}
            for label, xp in (("fp32", 0), ("half2", 1)):
                run = dict(xspec, precision=xp)
                _time_launches(torch, native, xt, xo, run, 3)
                xper, xsteps, _ = _time_launches(torch, native, xt, xo, run, 10)
                entry[label] = {"value": xh * xw * reps * 10 / (sum(xsteps) / 1e3) / 1e6,
                                "unit": "Mtexels/s", "mean_launch_us": xper * 1e3}
                if nstreams > 1:
                    # the same launches spread over the headline's streams
                    _time_launches(torch, native, xt, xo, run, 3, nstreams)
                    _, xsteps, _ = _time_launches(torch, native, xt, xo, run, 10, nstreams)
                    entry[label][f"value_{nstreams}_streams"] = xh * xw * reps * 10 / (sum(xsteps) / 1e3) / 1e6
            entry["speedup_half2_vs_fp32"] = entry["half2"]["value"] / entry["fp32"]["value"]
            extra[name] = entry
            del xt, xo

    aux = _bench_aux(torch, native, texs, outs, spec, hbm_peak)
    search = None if args.no_search else _bench_search(torch, native, args.workload, texs, outs, spec)
    batched = None if args.no_batched else _bench_batched(torch, native, oracle, args.batched_count)
    serving = None if args.no_serving else _bench_serving(
        torch, native, [int(r) for r in args.serving_rates.split(",") if r])
    # the same requests in ordinary pageable buffers at three rates
    serving_pageable = None if args.no_serving else _bench_serving(
        torch, native, [20000, 50000, 100000], host="pageable")
    cpu = None if args.no_cpu else _cpu_baseline(img, spec)

    hbm = {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
           "frac": (achieved_gbs / hbm_peak) if hbm_peak else None, "peak_source": hbm_source,
           "alg_bytes_per_launch": alg_bytes}
    issue = _issue_roofline(args.workload, prec, tuned, mean_launch_s, clk.get("sm_mhz"),
                            torch.cuda.get_device_properties(local).multi_processor_count)
    line = {
        "metric": METRIC, "value": value, "unit": "Mtexels/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_s / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": _config(args.workload, img, spec, args.precision, world),
        "launch": (f"one astc_encode_gpu_pitched call per texture, round-robin over {nstreams} CUDA streams "
                   "forked from and joined to the timed stream each step" if nstreams > 1 else
                   "one astc_encode_gpu_pitched call per texture, one after another on the timed stream"),
        "one_stream": {"value": world * texels_step * args.steps / (sum(per_step1) / 1e3) / 1e6,
                       "unit": "Mtexels/s", "mean_launch_us": per1 * 1e3},
        "kernel_variant": {"store": {0: "registers", 1: "shared", 2: "registers_capped"}.get(tuned.store, tuned.store),
                           "threads_per_cta": tuned.threads, "autotune_best_us": tuned.best_us},
        "e2e": {"value": e2e_value, "unit": "Mtexels/s",
                "h2d_bytes_per_step": texels_step * 4, "d2h_bytes_per_step": nblocks * 16 * len(texs),
                "entry_point": "astc_encode_gpu (ASTC_MEMORY_HOST, pinned buffers: inputs through the upload ring, blocks written in place over NVLink-C2C; one stream sync per step)",
                "steps": e2e_steps},
        "e2e_pageable": {"value": e2e_page_value, "unit": "Mtexels/s",
                         "h2d_bytes_per_step": texels_step * 4, "d2h_bytes_per_step": nblocks * 16 * len(texs),
                         "entry_point": "astc_encode_gpu (ASTC_MEMORY_HOST, pageable numpy buffers, no stream: "
                                        "each call returns with its blocks in place)",
                         "pageable_in_place": bool(page_caps["pageable_in_place"]), "steps": e2e_steps},
        "gpu_launches": int(launches),
        # the binding bound: FP32/INT issue (the per-block algebra is not a
        # contraction, so no tensor-core roof applies); HBM is the secondary roof
        "roofline": {"bound": "fp32_issue", "kernel": kernel, "achieved": achieved_tf, "peak": fp32_peak,
                     "unit": "TFLOP/s", "frac": achieved_tf / fp32_peak, "flops_per_launch": flops,
                     "mean_launch_us": mean_launch_s * 1e6,
                     "launch_time": ("step time / launches over the timed region (launches on "
                                     f"{nstreams} streams overlap where one texture's last wave ends)"
                                     if nstreams > 1 else "step time / launches over the timed region"),
                     "peak_source": "max of an FP32 FMA microbenchmark (libastc_fp32_peak.so) and an "
                                    "8192^3 SGEMM (TF32 off), both measured in this run",
                     "peak_fma_microbenchmark": fma_peak, "peak_sgemm": sgemm_peak,
                     **_traffic(args.workload, prec, tuned),
                     "hbm": hbm, "issue": issue},
        "clocks": clk,
        "wall_s_timed_region": wall,
        "search_mode": search,
        "aux_kernels": aux,
        "serving": serving,
        "serving_pageable": serving_pageable,
        "batched_mixed": batched,
        "extra_workloads": extra,
        "quality": quality,
    }
    # compact summary of the targets last, where a tail of the line keeps them
    ns = {"fp32_4x4_rgb_512_Mtexels_s": extra.get("4x4_rgb_512", {}).get("fp32", {}).get("value"),
          "fp32_4x4_rgb_floor_Mtexels_s": 20000,
          "speedup_half2_vs_fp32_plain": {k: v["speedup_half2_vs_fp32"] for k, v in extra.items()},
          "identical_blocks_vs_fp32_oracle": quality["identical_blocks_vs_fp32_oracle"],
          "psnr_gap_to_fp64_db": quality["psnr_gap_to_fp64_db"],
          "roofline_frac_fp32": achieved_tf / fp32_peak,
          "roofline_frac_hbm": hbm["frac"],
          "roofline_frac_issue": issue["frac"] if issue else None}
    if batched:
        ns["speedup_half2_vs_fp32_batched"] = batched["speedup_half2_vs_fp32_batched"]
        ns["batched_half2_max_gap_to_fp64_db"] = batched["psnr_gap_to_fp64_db"]["half2_max"]
        ns["batched_half2_vs_plain_fp32"] = batched["speedup_batched_half2_vs_plain_fp32"]
    if serving and serving.get("knee"):
        ns["serving_knee"] = serving["knee"]
    line["targets"] = ns
    if cpu is not None:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


def main() -> None:
    args = _parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
