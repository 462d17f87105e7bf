"""Generates astc_partition_table.h: for every partition index (seed 0..1023)
of a two-partition ASTC block, the texels the specification's partition hash
puts in partition 1, as a bit mask over the block's texels in row-major order
(bit y * dim + x), for 4x4 blocks (16 bits; "small block" rule: fewer than 31
texels doubles the coordinates) and 6x6 blocks (36 bits); the two-partition
pattern classes; and the three-partition pattern classes.
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


def classes3(dim: int) -> list:
    """(seed, m1, m2) of the smallest partition index of every distinct way a
    three-partition block splits its texels into three non-empty sets (two
    indices that split alike up to the partitions' order are one class), in
    index order; m1 / m2 = the texels in partitions 1 / 2 of that index."""
    small = dim * dim < 31
    seen = set()
    out = []
    for seed in range(1024):
        part = [select_partition(seed, i % dim, i // dim, 0, 3, small) for i in range(dim * dim)]
        if len(set(part)) < 3:
            continue
        order = []
        for v in part:
            if v not in order:
                order.append(v)
        canon = tuple(order.index(v) for v in part)          # relabelled in order of first texel
        if canon in seen:
            continue
        seen.add(canon)
        m1 = sum(1 << i for i, v in enumerate(part) if v == 1)
        m2 = sum(1 << i for i, v in enumerate(part) if v == 2)
        out.append((seed, m1, m2))
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
    t4, t6 = classes3(4), classes3(6)
    lines.append("};")
    lines.append("// Three-partition pattern classes: the smallest partition index of each")
    lines.append("// distinct split of the block into three non-empty sets, in index order.")
    lines.append("// 4x4: m1 | (m2 << 16) | (index << 32); 6x6: A = m1 | (index << 54), B = m2")
    lines.append("// (m1 / m2: the texels in partitions 1 / 2).")
    lines.append(f"constexpr int kPartition3Classes4x4Count = {len(t4)};")
    lines.append(f"constexpr uint64_t kPartition3Classes4x4[{len(t4)}] = {{")
    for i in range(0, len(t4), 4):
        lines.append("    " + ", ".join(f"0x{m1 | (m2 << 16) | (sd << 32):012X}ull" for sd, m1, m2 in t4[i:i + 4]) + ",")
    lines.append("};")
    lines.append(f"constexpr int kPartition3Classes6x6Count = {len(t6)};")
    lines.append(f"constexpr uint64_t kPartition3Classes6x6A[{len(t6)}] = {{")
    for i in range(0, len(t6), 4):
        lines.append("    " + ", ".join(f"0x{m1 | (sd << 54):016X}ull" for sd, m1, m2 in t6[i:i + 4]) + ",")
    lines.append("};")
    lines.append(f"constexpr uint64_t kPartition3Classes6x6B[{len(t6)}] = {{")
    for i in range(0, len(t6), 4):
        lines.append("    " + ", ".join(f"0x{m2:09X}ull" for sd, m1, m2 in t6[i:i + 4]) + ",")
    lines += ["};", "}  // namespace astc", ""]
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "astc_partition_table.h")
    with open(out, "w") as fh:
        fh.write("\n".join(lines))


if __name__ == "__main__":
    main()
