"""Writes trig_table.inc: cos, sin and cos - 1 of a_j = j / 128 for
j = 0 .. TRIG_N - 1, each correctly rounded to double (mpmath at 80 digits),
as C hex-float literals.  The table feeds the table-based sin / cos / atan2
of common.cuh.

Also writes trig_table_f.inc: cos and sin of a_j = j / 512 for
j = 0 .. TRIGF_N - 1 as float pairs (hi, lo): hi the value correctly rounded
to float, lo the remainder value - hi correctly rounded to float.  That table
feeds the two-float sin / cos / atan2 of f32x2.cuh.

    python stochasticsampling_gb300/csrc/gen_trig_table.py
"""
import os
import struct

import mpmath

TRIG_N = 808          # a_j up to 807 / 128 = 6.305 > 2 pi + 2^-8
LIMIT = 6.3           # angles below this take the table; round(128 * 6.3) = 806
TRIGF_N = 3228        # a_j up to 3227 / 512 = 6.303 > 6.3 + 2^-10; round(512 * 6.3) = 3226


def rounded(x):
    """x (an mpf at high precision) correctly rounded to a double, as a C hex literal."""
    with mpmath.workprec(53):
        d = float(mpmath.mpf(x))
    return d.hex()


def rounded_f(x):
    """x (an mpf at high precision) correctly rounded to a float, as a C hex literal."""
    with mpmath.workprec(24):
        f = float(+mpmath.mpf(x))
    return f, f.hex() + "f"


def split_f(x):
    """(hi, lo) float literals: hi = x rounded to float, lo = x - hi rounded to float."""
    h, hs = rounded_f(x)
    _, ls = rounded_f(x - mpmath.mpf(h))
    return hs, ls


def main_f(path=None):
    mpmath.mp.dps = 80
    rows = []
    for j in range(TRIGF_N):
        a = mpmath.mpf(j) / 512
        ch, cl = split_f(mpmath.cos(a))
        sh, sl = split_f(mpmath.sin(a))
        rows.append(f"{{{ch}, {cl}, {sh}, {sl}}}")
    key = struct.unpack("<q", struct.pack("<d", LIMIT))[0]
    out = ["// generated by gen_trig_table.py: (cos hi, cos lo, sin hi, sin lo) of j / 512 as float pairs",
           f"constexpr int kTrigFN = {TRIGF_N};",
           f"constexpr long long kTrigFMaxKey = 0x{key:016X}ll;  // bits of {LIMIT}",
           "SS_TRIGF_ATTR float4 kTrigF[kTrigFN] = {"]
    out += [f"    {r}," for r in rows]
    out += ["};", ""]
    path = path or os.path.join(os.path.dirname(os.path.abspath(__file__)), "trig_table_f.inc")
    with open(path, "w") as f:
        f.write("\n".join(out))


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
    main_f()
