"""Writes trig_table.inc: cos, sin and cos - 1 of a_j = j / 128 for
j = 0 .. TRIG_N - 1, each correctly rounded to double (mpmath at 80 digits),
as C hex-float literals.  The table feeds the table-based sin / cos / atan2
of common.cuh.

    python stochasticsampling_gb300/csrc/gen_trig_table.py
"""
import os
import struct

import mpmath

TRIG_N = 808          # a_j up to 807 / 128 = 6.305 > 2 pi + 2^-8
LIMIT = 6.3           # angles below this take the table; round(128 * 6.3) = 806


def rounded(x):
    """x (an mpf at high precision) correctly rounded to a double, as a C hex literal."""
    with mpmath.workprec(53):
        d = float(mpmath.mpf(x))
    return d.hex()


def main(path=None):
    mpmath.mp.dps = 80
    rows, cm1 = [], []
    for j in range(TRIG_N):
        a = mpmath.mpf(j) / 128
        rows.append(f"{{{rounded(mpmath.cos(a))}, {rounded(mpmath.sin(a))}}}")
        cm1.append(rounded(-2 * mpmath.sin(a / 2) ** 2))
    key = struct.unpack("<q", struct.pack("<d", LIMIT))[0]
    out = ["// generated by gen_trig_table.py: (cos, sin) and cos - 1 of j / 128, correctly rounded",
           f"constexpr int kTrigN = {TRIG_N};",
           f"constexpr long long kTrigMaxKey = 0x{key:016X}ll;  // bits of {LIMIT}",
           "static __device__ double2 kTrig[kTrigN] = {"]
    out += [f"    {r}," for r in rows]
    out += ["};", "static __device__ double kTrigCm1[kTrigN] = {"]
    out += [f"    {c}," for c in cm1]
    out += ["};", ""]
    path = path or os.path.join(os.path.dirname(os.path.abspath(__file__)), "trig_table.inc")
    with open(path, "w") as f:
        f.write("\n".join(out))


if __name__ == "__main__":
    main()
