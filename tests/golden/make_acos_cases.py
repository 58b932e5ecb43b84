#!/usr/bin/env python3
"""Write tests/golden/acos_cases.txt: arguments of the directed arc cosine with the exact downward and
upward roundings, computed with mpmath at 300 bits (the reference rounds acos with MPFR at the number
type's precision, ivarp/src/interval_acos.cpp:29-34).

Lines: "<d|f> <argument bits> <rounded-down bits> <rounded-up bits>" (hex; 'f' rows hold float results
for float arguments, the argument written as a double). The set: edge cases, seeded uniform arguments,
arguments next to +-1 and +-1/2, tiny and subnormal ones, float arguments, and the structured arguments
x = 1 - c^2 2^-k whose arc cosines lie unusually close to a double.

  python make_acos_cases.py
"""
import math
import os
import struct

import mpmath
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "acos_cases.txt")


def expected(x, digits):
    with mpmath.workprec(300):
        v = mpmath.acos(mpmath.mpf(x))
        if v == 0:
            return 0.0, 0.0
        if digits == 53:
            d = float(v)
            if mpmath.mpf(d) > v:
                d = math.nextafter(d, -math.inf)
            assert mpmath.mpf(d) < v
            return d, math.nextafter(d, math.inf)
        f = np.float32(float(v))
        if mpmath.mpf(float(f)) > v:
            f = np.nextafter(f, np.float32(-np.inf))
        assert mpmath.mpf(float(f)) < v
        return float(f), float(np.nextafter(f, np.float32(np.inf)))


def double_args():
    rng = np.random.default_rng(0xAC05)
    xs = [0.0, -0.0, 0.5, -0.5, 1.0, -1.0, 5e-324, -5e-324, 2.0 ** -1022, 2.0 ** -74, 2.0 ** -75, 0.25, -0.25,
          0.75, -0.75, 1.0 - 2.0 ** -53, -1.0 + 2.0 ** -53, 0.5 + 2.0 ** -53, 0.5 - 2.0 ** -54, -0.5 - 2.0 ** -53,
          1.0 / 3.0]
    xs += list(rng.uniform(-1.0, 1.0, 600))
    for sign in (1.0, -1.0):
        xs += [sign * (1.0 - k * 2.0 ** -53) for k in range(1, 20)]
        xs += [sign * (1.0 - 2.0 ** -e) for e in range(1, 54)]
        xs += list(sign * (1.0 - np.exp2(-rng.uniform(1.0, 53.0, 100))))
        xs += list(sign * np.exp2(-rng.uniform(1.0, 1074.0, 40)))
        xs += list(sign * (0.5 + rng.integers(-2000, 2000, 40) * 2.0 ** -53))
    structured = sorted({1.0 - c * c * 2.0 ** -k for c in range(1, 200) for k in range(1, 54)
                         if c * c * 2.0 ** -k < 0.5 and (c * c * 2.0 ** -k / 2.0 ** -53).is_integer()})
    xs += structured[::8] + [1.0 - 9 * 2.0 ** -49]
    return [float(x) for x in xs]


def float_args():
    rng = np.random.default_rng(0xAC06)
    xs = list(rng.uniform(-1.0, 1.0, 300).astype(np.float32))
    xs += [np.float32(1.0) - np.float32(k) * np.float32(2.0 ** -24) for k in range(1, 20)]
    xs += [-(np.float32(1.0) - np.float32(k) * np.float32(2.0 ** -24)) for k in range(1, 20)]
    xs += [np.float32(0.5), np.float32(-0.5), np.float32(0.0), np.float32(2.0 ** -149)]
    return [float(x) for x in xs]


def main():
    lines = []
    for x in double_args():
        lo, hi = expected(x, 53)
        lines.append("d %s %s %s" % (struct.pack(">d", x).hex(), struct.pack(">d", lo).hex(),
                                     struct.pack(">d", hi).hex()))
    for x in float_args():
        lo, hi = expected(x, 24)
        lines.append("f %s %s %s" % (struct.pack(">d", x).hex(), struct.pack(">f", lo).hex(),
                                     struct.pack(">f", hi).hex()))
    with open(OUT, "w") as f:
        f.write("\n".join(lines) + "\n")
    print(OUT, len(lines))


if __name__ == "__main__":
    main()
