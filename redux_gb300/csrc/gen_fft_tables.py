"""Writes fft_tables.h: cos/sin(2 pi k/R) for the butterfly radices (build-time generator)."""
import math
import os

RADICES = (3, 5, 7, 9, 11, 13, 16)


def main():
    lines = ["// Constant tables for the odd-radix and radix-16 butterflies of rdxg_fft.cuh.",
             "// cos(2 pi k / R) and sin(2 pi k / R), k < R, rounded from double precision.",
             "// Generated by gen_fft_tables.py.", "#pragma once", ""]
    for R in RADICES:
        for nm, fn in (("Cos", math.cos), ("Sin", math.sin)):
            vals = ", ".join(repr(fn(2 * math.pi * k / R)) for k in range(R))
            lines.append(f"__device__ constexpr double k{nm}{R}d[{R}] = {{{vals}}};")
            valsf = ", ".join(repr(fn(2 * math.pi * k / R)) + "f" for k in range(R))
            lines.append(f"__device__ constexpr float k{nm}{R}f[{R}] = {{{valsf}}};")
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "fft_tables.h")
    with open(out, "w") as f:
        f.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
