#!/usr/bin/env python3
"""Write acos_table.cuh: the constants of the correctly rounded arc cosine in acos.cuh.

Rows 0..127 hold the Taylor coefficients of asin,
    asin(t) = sum_k C_k t^(2k+1),  C_k = (2k)! / (4^k (k!)^2 (2k+1))   (exact rationals),
row 128 holds pi/2 and row 129 holds pi. Every row is an unsigned 256-bit fixed-point number with
253 fractional bits (little-endian 64-bit limbs), rounded to nearest from the exact value; pi comes
from mpmath at 600 bits. A computation with fewer limbs uses the top limbs of each row.

  python gen_acos_table.py [output]
"""
import os
import sys
from fractions import Fraction
from math import factorial

TERMS = 128
LIMBS = 4
FRAC = 64 * LIMBS - 3


def to_fraction(x):
    man, exp = x.man_exp
    return Fraction(man) * (Fraction(2) ** exp)


def fixed(v):
    """Round v (a Fraction) to the nearest multiple of 2^-FRAC; return the limbs, little-endian."""
    n = int((v * (1 << FRAC) + Fraction(1, 2)) // 1)
    assert 0 <= n < 1 << (64 * LIMBS)
    return [(n >> (64 * i)) & ((1 << 64) - 1) for i in range(LIMBS)]


def main():
    import mpmath
    mpmath.mp.prec = 600
    here = os.path.dirname(os.path.abspath(__file__))
    out = sys.argv[1] if len(sys.argv) > 1 else os.path.join(here, "acos_table.cuh")
    rows = [Fraction(factorial(2 * k), 4 ** k * factorial(k) ** 2 * (2 * k + 1)) for k in range(TERMS)]
    pi = to_fraction(mpmath.mpf(mpmath.pi))
    rows += [pi / 2, pi]
    lines = ["// Generated by gen_acos_table.py -- do not edit.",
             "// Rows 0..%d: Taylor coefficients of asin; row %d: pi/2; row %d: pi." % (TERMS - 1, TERMS, TERMS + 1),
             "// 256-bit fixed point, %d fractional bits, rounded to nearest, little-endian 64-bit limbs." % FRAC,
             "#pragma once", "",
             "#define SID_ACOS_TABLE_TERMS %d" % TERMS,
             "#define SID_ACOS_TABLE_ROWS %d" % len(rows),
             "#define SID_ACOS_TABLE_INIT { \\"]
    for v in rows:
        lines.append("    {%s}, \\" % ", ".join("0x%016xull" % l for l in fixed(v)))
    lines += ["}", ""]
    with open(out, "w") as f:
        f.write("\n".join(lines))
    print(out)


if __name__ == "__main__":
    main()
