"""bench.py's JSON contract, on the CPU: the reference arm (the FP32 oracle
with OpenMP, the stand-in for the D3D11-only reference shader) prints one line
with the contract's keys, and only rank 0 prints under a multi-rank launch."""
import json
import os
import subprocess
import sys

from conftest import ROOT

BENCH = os.path.join(ROOT, "bench.py")


def _run(args, env_extra=None):
    env = dict(os.environ)
    env.update(env_extra or {})
    return subprocess.run([sys.executable, BENCH, *args], capture_output=True, text=True, env=env,
                          timeout=600, cwd=ROOT)


def test_reference_arm_line():
    r = _run(["--impl", "reference", "--steps", "1", "--warmup", "0", "--workload", "4x4_rgb_512"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["higher_is_better"] is True and d["value"] > 0
    assert d["config"]["workload"] == "4x4_rgb_512"
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    # the GPU arm prints the same config dict (same function, same workload)
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_mod", BENCH)
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    from astc_encoder_gb300 import synth
    img, wspec = synth.workload("4x4_rgb_512")
    assert d["config"] == bench._config("4x4_rgb_512", img, wspec, "fp32", 1)
    assert d["config"]["textures_per_step"] == bench.TEXTURES_PER_STEP


def test_reference_arm_other_ranks_are_silent():
    r = _run(["--impl", "reference", "--steps", "1", "--warmup", "0", "--workload", "4x4_rgb_512"],
             {"WORLD_SIZE": "2", "RANK": "1", "LOCAL_RANK": "1"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert not [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]


def test_help_lists_the_contract_flags():
    r = _run(["--help"])
    assert r.returncode == 0
    for flag in ("--gpus", "--steps", "--warmup", "--impl", "--wave-sweep"):
        assert flag in r.stdout


def test_issue_roofline_arithmetic():
    """roofline_issue: instructions per launch from the committed capture over
    the launch time, against 4 warp-instructions per SM per cycle."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_mod", BENCH)
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)

    class Tuned:
        store = 2
    r = bench._issue_roofline("6x6_rgba_srgb_2048", 0, Tuned(), 20e-6, 2000, 150)
    assert abs(r["peak"] - 150 * 4 * 2.0) < 1e-9
    assert abs(r["achieved"] - r["instructions_per_launch"] / 20e-6 / 1e9) < 1e-6
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-12
    assert bench._issue_roofline("4x4_rgb_512", 0, Tuned(), 20e-6, 2000, 150) is None
    assert bench._issue_roofline("6x6_rgba_srgb_2048", 0, Tuned(), 20e-6, None, 150) is None
