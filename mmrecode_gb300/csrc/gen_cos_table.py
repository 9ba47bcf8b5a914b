"""Writes cos_table.inc: the cosine constants of the DV25 transforms.

The DV IDCTs (crates/codecs/dv/src/decoder.rs:520-602) use
cos(((2x+1) * u * PI) / 16) and cos(((2y+1) * v * PI) / 8), evaluated in
binary64 then passed to libm. Each argument is fl(k*PI)/16 for an integer
k < 128 (the /8 form is k' = 2k). The table holds the correctly rounded
cosine of each argument (mpmath, 60 digits); on glibc hosts these equal what
libm returns, which this script checks before writing. Device code reads the
table instead of calling a device cos, so results do not depend on any
device math library. Run from the repository root:

    python mmrecode_gb300/csrc/gen_cos_table.py
"""

import math
import os
import sys

import mpmath


def main() -> int:
    mpmath.mp.dps = 60
    vals = []
    for k in range(128):
        arg = float(k) * math.pi / 16.0
        vals.append(float(mpmath.cos(mpmath.mpf(arg))))
    bad = [k for k, v in enumerate(vals) if math.cos(float(k) * math.pi / 16.0) != v]
    if bad:
        print("libm disagrees with the correctly rounded cosine at k =", bad)
        return 1
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "cos_table.inc")
    with open(path, "w") as f:
        f.write("// Generated by gen_cos_table.py: cos(fl(k*PI)/16), k = 0..127, correctly rounded.\n")
        for k, v in enumerate(vals):
            f.write(f"{v.hex()},\n")
    print("wrote", path)
    return 0


if __name__ == "__main__":
    sys.exit(main())
