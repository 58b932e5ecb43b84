"""Expected results of the known-answer systems (tests/golden/kat), restated from the reference's tests.

expected_critical: ivarp/test/expected_criticals.cpp:31-96. expected_critical2:
ivarp/test/expected_criticals2.cpp:33-226. The critical boxes are computed here exactly (all values are
dyadic rationals representable in float and double, so plain Python floats are exact).
"""
import numpy as np

EC_COUNTS = dict(cuboids=(8 + 8 * 4) + (16 + 16 * 4) + (32 + 32 * 4) + 32 * 4,
                 leaves=8 * 4 + 16 * 4 + 2 * 32 * 4, criticals=128)

EC2_COUNTS = {
    0: dict(cuboids=1172 + 1152, leaves=2 * 1024, criticals=1024),
    1: dict(cuboids=4 + 16 + 8 * 16 + 64 * 16 + 4 * 16 + 4 * 4 * 16 + 256 * 8 + 256 * 64 + 256 * 8 + 256 * 64,
            leaves=1024 + 2 * 16384, criticals=16384),
    2: dict(cuboids=4 + 16 + 8 * 16 + 64 * 16 + 4 * 16 + 4 * 4 * 16 + 256 * 8 + 256 * 64 + 4 * 256 + 4 * 4 * 256
            + 8 * 4096 + 64 * 4096 + 8 * 4096 + 64 * 4096,
            leaves=1024 + 16384 + 262144 * 2, criticals=262144),
}


def expected_critical_boxes():
    """Critical boxes of expected_critical (32 x-ranges of width 1/16, 4 y-pieces each), sorted."""
    out = []
    for i in range(32):
        xlo, xhi = i / 16.0, (i + 1) / 16.0
        ymax = min(xhi, 3 - xlo)
        for j in range(4):
            miny = (ymax / 4) * j
            maxy = (ymax / 4) * (j + 1)
            lo = xlo
            if miny > 0 and lo < miny:
                lo = miny
            out.append([[lo, xhi], [miny, maxy]])
    return np.array(out, dtype=np.float64)


def splitter(lo, hi, n):
    w = (hi - lo) / n
    return [(lo + i * w if i < n else hi, lo + (i + 1) * w if i + 1 < n else hi) for i in range(n)]


def expected_critical2_gen2_boxes():
    """Criticals of expected_critical2 with 2 generations: the grid 64 x 64 x 8 x 8 of [0,1]^4, lexicographic."""
    w = splitter(0.0, 1.0, 64)
    y = splitter(0.0, 1.0, 8)
    out = np.empty((64, 64, 8, 8, 4, 2), dtype=np.float64)
    out[:, :, :, :, 0, :] = np.array(w)[:, None, None, None, :]
    out[:, :, :, :, 1, :] = np.array(w)[None, :, None, None, :]
    out[:, :, :, :, 2, :] = np.array(y)[None, None, :, None, :]
    out[:, :, :, :, 3, :] = np.array(y)[None, None, None, :, :]
    return out.reshape(-1, 4, 2)


def sort_boxes(b):
    """Lexicographic order of boxes by (lo, hi) of each variable in turn."""
    flat = b.reshape(len(b), -1)
    return b[np.lexsort(flat.T[::-1])]
