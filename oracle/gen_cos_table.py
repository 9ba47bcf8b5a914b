"""Generate oracle/cos_table.h: the cosine values the DV25 IDCTs use.

TEST INFRASTRUCTURE (oracle). The reference DV transforms call libm ``cos`` on
arguments ``((2x+1) as f64 * u as f64 * PI) / 16.0`` and ``... / 8.0``
(crates/codecs/dv/src/decoder.rs:520-602). Every such argument equals
``fl(k * PI) / 16`` for an integer k in 0..127 (``fl(k*PI)/8 == fl(2k*PI)/16``
because doubling is exact). This script evaluates each cosine to 60 digits with
mpmath, rounds it to the nearest binary64, checks that the host libm
(``math.cos``, glibc here) returns the same double, and writes the values as
hex-float literals. Run from the repository root:

    python oracle/gen_cos_table.py
"""

import math
import os
import sys

import mpmath

mpmath.mp.dps = 60


def correctly_rounded_cos(k: int) -> float:
    arg = float(k) * math.pi / 16.0  # binary64 evaluation, left to right, no FMA
    exact = mpmath.cos(mpmath.mpf(arg))
    return float(exact)  # mpmath rounds to nearest binary64


def main() -> int:
    values = [correctly_rounded_cos(k) for k in range(128)]
    mismatches = [k for k in range(128) if math.cos(float(k) * math.pi / 16.0) != values[k]]
    if mismatches:
        print("host libm cos differs from the correctly rounded value at k =", mismatches)
        return 1
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "cos_table.h")
    with open(out, "w") as f:
        f.write("/* Generated by oracle/gen_cos_table.py -- do not edit.\n")
        f.write(" * ORC_COS16[k] = cos(fl(k*PI)/16) correctly rounded; equal to glibc cos on the\n")
        f.write(" * generating host for every k. TEST INFRASTRUCTURE (oracle). */\n")
        f.write("static const double ORC_COS16[128] = {\n")
        for k, v in enumerate(values):
            f.write(f"    {v.hex()}, /* k={k} */\n")
        f.write("};\n")
    print("wrote", out)
    return 0


if __name__ == "__main__":
    sys.exit(main())
