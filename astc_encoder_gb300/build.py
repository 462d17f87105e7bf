"""In-tree build of the native library (libastc_gb300.so) and the CLI.

Every CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``) in parallel, then linked into
``astc_encoder_gb300/_lib/libastc_gb300.so`` (static CUDA runtime) and the
drop-in command line tool ``astc_encoder_gb300/_lib/astc_cs_enc`` (plus the
benchmark's FP32 throughput probe ``libastc_fp32_peak.so``).  Objects go
to ``astc_encoder_gb300/_build/``.  Nothing is installed outside the tree.

Usage: ``python -m astc_encoder_gb300.build [--force] [--verbose]``
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libastc_gb300.so")
CLI = os.path.join(LIBDIR, "astc_cs_enc")
PEAK_LIB = os.path.join(LIBDIR, "libastc_fp32_peak.so")      # FP32 FMA throughput, for the benchmark
INCLUDE = os.path.join(os.path.dirname(PKG), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-Wall",
          "--expt-relaxed-constexpr", "-I", CSRC, "-I", INCLUDE]

# (source, extra flags).  The encoder is built with --fmad=false so the
# compiler contracts nothing: every fused multiply-add is written explicitly.
LIB_SOURCES = [
    ("astc_encode.cu", ["--fmad=false"]),
    ("astc_encode_h2.cu", ["--fmad=false"]),
    ("astc_encode_search.cu", ["--fmad=false"]),
    ("astc_encode_thorough.cu", ["--fmad=false"]),
    ("astc_encode_partitions.cu", ["--fmad=false"]),
    ("astc_encode_three.cu", ["--fmad=false"]),
    ("astc_encode_best.cu", ["--fmad=false"]),
    ("astc_encode_coop.cu", ["--fmad=false"]),
    ("astc_batch.cu", ["--fmad=false"]),
    ("astc_mips.cu", []),
    ("astc_server.cu", []),
    ("astc_decode.cu", []),
    ("astc_capi.cu", []),
    ("astc_noalloc.cu", []),
    ("astc_tune.cu", []),
]
CLI_SOURCES = [
    ("astc_cs_enc.cpp", []),
    # FP32 expressions of the image readers are evaluated as written (no
    # fused multiply-add), as the reference's loader is on its own build
    ("image_load.cpp", ["-Xcompiler", "-ffp-contract=off"]),
]
HEADERS = ["astc_internal.h", "astc_tables.h", "astc_ise.h", "astc_block_common.cuh", "astc_pipeline_fp32.cuh",
           "astc_pipeline_h2.cuh", "astc_pipeline_search.cuh", "astc_pipeline_dual.cuh", "astc_pipeline_partition.cuh", "astc_pipeline_partition3.cuh", "astc_search_kernel.cuh",
           "astc_partition_table.h", "astc_srgb_table.h", "astc_sse.cuh", "image_load.h"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found (set NVCC or put CUDA's bin/ on PATH)")


def _newest_dep_mtime() -> float:
    paths = [os.path.join(CSRC, h) for h in HEADERS]
    paths.append(os.path.join(INCLUDE, "astc_gb300.h"))
    paths.append(os.path.abspath(__file__))
    return max(os.path.getmtime(p) for p in paths if os.path.exists(p))


def _stale(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources) or _newest_dep_mtime() > t


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed ({res.returncode}): {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    if verbose and (res.stdout or res.stderr):
        print(res.stdout + res.stderr, flush=True)


def _compile(src: str, extra: list[str], force: bool, verbose: bool) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    if force or _stale(obj, [path]):
        cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", path, "-o", obj]
        _run(cmd, verbose)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (if stale) and link the library and the CLI; returns the .so path."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    jobs = [(s, f) for s, f in LIB_SOURCES] + [(s, f) for s, f in CLI_SOURCES
                                               if os.path.exists(os.path.join(CSRC, s))] + [("fp32_peak.cu", [])]
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        futs = {s: ex.submit(_compile, s, f, force, verbose) for s, f in jobs}
        objs = {s: fu.result() for s, fu in futs.items()}
    lib_objs = [objs[s] for s, _ in LIB_SOURCES]
    if force or _stale(LIB, lib_objs):
        _run([nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", LIB, *lib_objs], verbose)
    cli_objs = [objs[s] for s, _ in CLI_SOURCES if s in objs]
    if len(cli_objs) == len(CLI_SOURCES) and (force or _stale(CLI, cli_objs + [LIB])):
        _run([nvcc(), *ARCH, "-o", CLI, *cli_objs, "-L", LIBDIR, "-lastc_gb300",
              "-Xlinker", "-rpath,$ORIGIN"], verbose)
    peak_obj = objs["fp32_peak.cu"]
    if force or _stale(PEAK_LIB, [peak_obj]):
        _run([nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", PEAK_LIB, peak_obj], verbose)
    return LIB


def main(argv: list[str] | None = None) -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    a = ap.parse_args(argv)
    print(build(force=a.force, verbose=a.verbose))
    return 0


if __name__ == "__main__":
    sys.exit(main())
