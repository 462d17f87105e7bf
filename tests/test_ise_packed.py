"""The ISE encoders of the search-mode assemblers (csrc/astc_ise.h: the rolled
loop for any range, the compile-time form of each range), compiled for the
host, against the oracle's integer sequence encoder
(ASTC_IntegerSequenceEncoding.hlsl encode_trits / encode_quints / bise_*):
every range QUANT_2..QUANT_256; the rolled loop at every length 1..32, the
compile-time forms at the lengths the assemblers use (6, 8, 12, 16, 18
endpoint values; 16 and 32 weights); random and extreme values.  Bar: all 16
bytes identical (the oracle's sequence is zero past its length)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "astc_encoder_gb300", "csrc")
LEVELS = [2, 3, 4, 5, 6, 8, 10, 12, 16, 20, 24, 32, 40, 48, 64, 80, 96, 128, 160, 192, 256]


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path_factory.mktemp("ise") / "ise_packed_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I", CSRC,
                    os.path.join(HERE, "ise_packed_check.cpp"), "-o", exe], check=True)
    return exe


@pytest.mark.parametrize("form", [0, 1])
def test_encoders_match_oracle(harness, form):
    rng = np.random.default_rng(11 + form)
    cases = []
    for quant, levels in enumerate(LEVELS):
        for count in (range(1, 33) if form == 0 else (6, 8, 12, 16, 18, 32)):
            if oracle.ise_bits(quant, count) > 128:
                continue
            for kind in range(4):
                if kind == 0:
                    v = rng.integers(0, levels, count)
                elif kind == 1:
                    v = np.full(count, levels - 1)
                elif kind == 2:
                    v = np.zeros(count, np.int64)
                else:
                    v = rng.choice([0, levels - 1], count)
                cases.append((quant, count, [int(x) for x in v]))
    text = "".join(f"{form} {q} {c} {' '.join(map(str, v))}\n" for q, c, v in cases)
    got = subprocess.run([harness], input=text, capture_output=True, text=True, check=True).stdout.split()
    assert len(got) == len(cases)
    for (q, c, v), hexbytes in zip(cases, got):
        want = oracle.ise_encode(q, v)
        assert bytes.fromhex(hexbytes) == bytes(want), (q, c, v)
