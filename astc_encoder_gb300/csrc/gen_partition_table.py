"""Generates astc_partition_table.h: for every partition index (seed 0..1023)
of a two-partition ASTC block, the texels the specification's partition hash
puts in partition 1, as a bit mask over the block's texels in row-major order
(bit y * dim + x), for 4x4 blocks (16 bits; "small block" rule: fewer than 31
texels doubles the coordinates) and 6x6 blocks (36 bits).
Run: python astc_encoder_gb300/csrc/gen_partition_table.py
"""
import os

M32 = 0xFFFFFFFF


def _hash(p: int) -> int:
    p ^= p >> 15
    p = (p - (p << 17)) & M32
    p = (p + (p << 7)) & M32
    p = (p + (p << 4)) & M32
    p ^= p >> 5
    p = (p + (p << 16)) & M32
    p ^= p >> 7
    p ^= p >> 3
    p = (p ^ (p << 6)) & M32
    p ^= p >> 17
    return p


def select_partition(seed: int, x: int, y: int, z: int, count: int, small: bool) -> int:
    """The specification's partition assignment of texel (x, y, z)."""
    if small:
        x, y, z = x << 1, y << 1, z << 1
    seed += (count - 1) * 1024
    rnum = _hash(seed)
    s = [(rnum >> (4 * i)) & 0xF for i in range(8)]
    s += [(rnum >> 18) & 0xF, (rnum >> 22) & 0xF, (rnum >> 26) & 0xF, ((rnum >> 30) | (rnum << 2)) & 0xF]
    s = [v * v for v in s]
    if seed & 1:
        sh1, sh2 = (4 if seed & 2 else 5), (6 if count == 3 else 5)
    else:
        sh1, sh2 = (6 if count == 3 else 5), (4 if seed & 2 else 5)
    sh3 = sh1 if seed & 0x10 else sh2
    for i in range(8):
        s[i] >>= sh1 if i % 2 == 0 else sh2
    for i in range(8, 12):
        s[i] >>= sh3
    a = (s[0] * x + s[1] * y + s[10] * z + (rnum >> 14)) & 0x3F
    b = (s[2] * x + s[3] * y + s[11] * z + (rnum >> 10)) & 0x3F
    c = (s[4] * x + s[5] * y + s[8] * z + (rnum >> 6)) & 0x3F
    d = (s[6] * x + s[7] * y + s[9] * z + (rnum >> 2)) & 0x3F
    if count < 4:
        d = 0
    if count < 3:
        c = 0
    if a >= b and a >= c and a >= d:
        return 0
    if b >= c and b >= d:
        return 1
    if c >= d:
        return 2
    return 3


def masks(dim: int) -> list:
    small = dim * dim < 31
    out = []
    for seed in range(1024):
        m = 0
        for y in range(dim):
            for x in range(dim):
                if select_partition(seed, x, y, 0, 2, small) == 1:
                    m |= 1 << (y * dim + x)
        out.append(m)
    return out


def classes(dim: int) -> list:
    """(seed, mask) of the smallest partition index of every class {pattern,
    complement} that splits the block, in index order.  Scanning these in
    order with a strict 'fewer mismatches' test picks the same index as
    scanning all 1024 (a pattern and its complement score alike, duplicates
    score alike, and ties go to the smallest index)."""
    full = (1 << (dim * dim)) - 1
    seen = set()
    out = []
    for seed, m in enumerate(masks(dim)):
        if m in (0, full):
            continue
        key = min(m, full ^ m)
        if key in seen:
            continue
        seen.add(key)
        out.append((seed, m))
    return out


def main() -> None:
    m4, m6 = masks(4), masks(6)
    c4, c6 = classes(4), classes(6)
    lines = ["// Generated by gen_partition_table.py -- do not edit.",
             "// Two-partition ASTC blocks: for each partition index 0..1023, the texels",
             "// (bit y * dim + x) that the specification's partition hash puts in partition 1.",
             "#pragma once", "#include <stdint.h>", "", "namespace astc {",
             "constexpr uint16_t kPartition2Mask4x4[1024] = {"]
    for i in range(0, 1024, 12):
        lines.append("    " + ", ".join(f"0x{v:04X}" for v in m4[i:i + 12]) + ",")
    lines.append("};")
    lines.append("constexpr uint64_t kPartition2Mask6x6[1024] = {")
    for i in range(0, 1024, 6):
        lines.append("    " + ", ".join(f"0x{v:09X}ull" for v in m6[i:i + 6]) + ",")
    lines.append("};")
    lines.append("// The smallest partition index of each {pattern, complement} class that")
    lines.append("// splits the block, in index order: (index << 16) | mask for 4x4, (index << 54) | mask")
    lines.append("// for 6x6.")
    lines.append(f"constexpr int kPartition2Classes4x4Count = {len(c4)};")
    lines.append(f"constexpr uint32_t kPartition2Classes4x4[{len(c4)}] = {{")
    for i in range(0, len(c4), 8):
        lines.append("    " + ", ".join(f"0x{(sd << 16) | m:08X}u" for sd, m in c4[i:i + 8]) + ",")
    lines.append("};")
    lines.append(f"constexpr int kPartition2Classes6x6Count = {len(c6)};")
    lines.append(f"constexpr uint64_t kPartition2Classes6x6[{len(c6)}] = {{")
    for i in range(0, len(c6), 4):
        lines.append("    " + ", ".join(f"0x{(sd << 54) | m:016X}ull" for sd, m in c6[i:i + 4]) + ",")
    lines += ["};", "}  // namespace astc", ""]
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "astc_partition_table.h")
    with open(out, "w") as fh:
        fh.write("\n".join(lines))


if __name__ == "__main__":
    main()
