"""Generates astc_srgb_table.h: the FP32 texel value the encoder fits for each
sRGB code, float(IEC 61966-2-1 sRGB -> linear in double) * 255 in float,
stored as IEEE-754 bit patterns so every translation unit gets the same
constants at compile time.  Run: python astc_encoder_gb300/csrc/gen_srgb_table.py
"""
import os
import struct


def f32(x: float) -> float:
    return struct.unpack("<f", struct.pack("<f", x))[0]


def value(code: int) -> float:
    x = code / 255.0
    lin = x / 12.92 if x <= 0.04045 else ((x + 0.055) / 1.055) ** 2.4
    return f32(f32(lin) * f32(255.0))


def main() -> None:
    bits = [struct.unpack("<I", struct.pack("<f", value(c)))[0] for c in range(256)]
    lines = ["// Generated by gen_srgb_table.py -- do not edit.",
             "// sRGB code -> float(srgb_to_linear(code / 255)) * 255 (IEEE-754 bits).",
             "#pragma once", "#include <stdint.h>", "", "namespace astc {",
             "constexpr uint32_t kSrgbX255Bits[256] = {"]
    for i in range(0, 256, 8):
        lines.append("    " + ", ".join(f"0x{b:08X}u" for b in bits[i:i + 8]) + ",")
    lines += ["};", "}  // namespace astc", ""]
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "astc_srgb_table.h")
    with open(out, "w") as fh:
        fh.write("\n".join(lines))


if __name__ == "__main__":
    main()
